"""Python mirror of the reference's Core/ interface over the C ABI.

Names follow the reference (Core/material.h, Core/sphere.h, Core/Scene.h,
Core/camera.h, Core/CUDAOutputBuffer.h, Core/Renderer.h) so a user of
Renderer::Init / Draw / Cleanup finds the same calls.  Device memory for the
output and accumulation buffers is held in torch tensors (plumbing only); all
compute runs in libvenusaur_gb300.so.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import CAMERA_DTYPE, NODE_DTYPE, SPHERE_DTYPE, RenderOpts, RenderStats, SceneInfo, Tuning, check, lib, ptr

TUNING_FIELDS = ("traverse_variant", "refill_min", "traverse_block", "traverse_blocks_per_sm", "shade_block",
                 "shade_blocks_per_sm", "in_place_factor")


def _torch():
    import torch  # noqa: PLC0415  (imported lazily: only device buffers need it)
    return torch


_cuda_available = None


def _stream_handle(stream=None):
    """cudaStream_t of `stream` (default: torch's current stream).  Without a
    CUDA device this is NULL and the library itself reports the missing
    device (VENU_ERR_NO_DEVICE)."""
    global _cuda_available
    if stream is not None:
        return C.c_void_p(stream.cuda_stream)
    torch = _torch()
    if _cuda_available is None:
        _cuda_available = torch.cuda.is_available()
    if not _cuda_available:
        return None
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


# ---------------------------------------------------------------------------
# Material / Sphere (Core/material.h:6-33, Core/sphere.h:5-36)
# ---------------------------------------------------------------------------
class Material:
    Lambertian = 0
    Metal = 1
    Dielectric = 2

    def __init__(self, type: int, albedo=(0.0, 0.0, 0.0), fuzz: float = 0.0, ir: float = 0.0):
        self.m_type = int(type)
        self.m_albedo = tuple(float(np.float32(a)) for a in albedo)
        self.m_fuzz = float(np.float32(fuzz))
        self.m_ir = float(np.float32(ir))

    def GetType(self) -> int:
        return self.m_type

    def GetAlbedo(self):
        return self.m_albedo

    def GetFuzz(self) -> float:
        return self.m_fuzz

    def GetIR(self) -> float:
        return self.m_ir


class Sphere:
    def __init__(self, center, radius: float, material: Material):
        self.m_center = tuple(float(np.float32(c)) for c in center)
        self.m_radius = float(np.float32(radius))
        self.m_material = material

    def GetCenter(self):
        return self.m_center

    def GetRadius(self) -> float:
        return self.m_radius

    def GetMaterial(self) -> Material:
        return self.m_material

    def SetMaterial(self, material: Material) -> None:
        self.m_material = material

    def GetAABB(self):
        """Core/sphere.h:17-28, using |radius| (the reference computes it and
        then ignores it)."""
        r = abs(self.m_radius)
        c = self.m_center
        return (c[0] - r, c[1] - r, c[2] - r, c[0] + r, c[1] + r, c[2] + r)


def spheres_to_array(spheres) -> np.ndarray:
    a = np.zeros(len(spheres), SPHERE_DTYPE)
    for i, s in enumerate(spheres):
        m = s.GetMaterial()
        a[i]["center"] = s.GetCenter()
        a[i]["radius"] = s.GetRadius()
        a[i]["albedo"] = m.GetAlbedo()
        a[i]["fuzz"] = m.GetFuzz()
        a[i]["ir"] = m.GetIR()
        a[i]["material"] = m.GetType()
    return a


def array_to_spheres(a: np.ndarray):
    out = []
    for r in a:
        m = Material(int(r["material"]), tuple(r["albedo"]), float(r["fuzz"]), float(r["ir"]))
        out.append(Sphere(tuple(r["center"]), float(r["radius"]), m))
    return out


def sm_count() -> int:
    """Streaming multiprocessors of the current device (venu_device_check)."""
    n, major, minor = C.c_int(0), C.c_int(0), C.c_int(0)
    check(lib().venu_device_check(C.byref(n), C.byref(major), C.byref(minor)))
    return int(n.value)


def generate_rtiow(seed: int = 0) -> np.ndarray:
    buf = np.zeros(600, SPHERE_DTYPE)
    n = lib().venu_scene_generate_rtiow(seed, ptr(buf), len(buf))
    return buf[:n].copy()


def generate_random(n: int, seed: int = 0, box_lo=(-100.0, 0.0, -100.0), box_hi=(100.0, 20.0, 100.0),
                    rmin: float = 0.01, rmax: float = 0.5) -> np.ndarray:
    out = np.zeros(n, SPHERE_DTYPE)
    lo = np.asarray(box_lo, np.float32)
    hi = np.asarray(box_hi, np.float32)
    check(lib().venu_scene_generate_random(n, seed, ptr(lo), ptr(hi), rmin, rmax, ptr(out)))
    return out


class Scene:
    """Core/Scene.h: the default constructor builds the RTIOW final scene."""

    def __init__(self, seed: int = 0, spheres=None):
        if spheres is None:
            self.spheres = generate_rtiow(seed)
        elif isinstance(spheres, np.ndarray):
            self.spheres = np.ascontiguousarray(spheres, SPHERE_DTYPE)
        else:
            self.spheres = spheres_to_array(spheres)

    @classmethod
    def random(cls, n: int, seed: int = 0, **kw) -> "Scene":
        return cls(spheres=generate_random(n, seed, **kw))

    @property
    def m_spheres(self):
        return array_to_spheres(self.spheres)

    @property
    def m_aabbs(self) -> np.ndarray:
        c = self.spheres["center"]
        r = np.abs(self.spheres["radius"])[:, None]
        return np.concatenate([c - r, c + r], axis=1)

    @property
    def m_indices(self) -> np.ndarray:
        return np.arange(len(self.spheres), dtype=np.uint32)

    def __len__(self) -> int:
        return len(self.spheres)


# ---------------------------------------------------------------------------
# Camera (Core/camera.h, Core/Camera.cpp)
# ---------------------------------------------------------------------------
class Camera:
    m_defaultForward = (0.0, 0.0, -1.0)

    def __init__(self, origin=(0.0, 0.0, 0.0), vfov: float = 45.0, aspect: float = 1.6,
                 aperture: float = 0.0, focalLength: float = 1.0):
        self.m_position = np.asarray(origin, np.float32)
        self.m_forward = np.asarray(self.m_defaultForward, np.float32)
        self.m_vfov = np.float32(vfov)
        self.m_aspect = np.float32(aspect)
        self.m_aperture = np.float32(aperture)
        self.m_focalLength = np.float32(focalLength)
        self.m_changed = True
        self._update_uvw()

    @staticmethod
    def _normalize(d):
        d = np.asarray(d, np.float32)
        dot = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
        return (d * (np.float32(1.0) / np.sqrt(dot))).astype(np.float32)

    def SetForward(self, direction) -> None:
        self.m_forward = self._normalize(direction)
        self.m_changed = True

    def GetLensRadius(self) -> float:
        return float(self.m_aperture * np.float32(0.5))

    def GetPosition(self):
        return self.m_position.copy()

    def GetFocalLength(self) -> float:
        return float(self.m_focalLength)

    def SetFocalLength(self, length: float) -> None:
        if self.m_focalLength != np.float32(length):
            self.m_focalLength = np.float32(length)
            self.m_changed = True

    def MoveForward(self, speed: float) -> None:
        self.m_position = (self.m_position + self.m_forward * np.float32(speed)).astype(np.float32)
        self.m_changed = True

    # Core/camera.h:42-78.  As in the reference, the u/v/w axes used here are
    # those of the last UVWFrame (constructor, params() or UVWFrame()).
    def MoveRight(self, speed: float) -> None:
        self.m_position = (self.m_position + self._normalize(self.m_u) * np.float32(speed)).astype(np.float32)
        self.m_changed = True

    def MoveUp(self, speed: float) -> None:
        self.m_position = (self.m_position + self._normalize(self.m_v) * np.float32(speed)).astype(np.float32)
        self.m_changed = True

    def _rotate(self, axis, degrees: float) -> None:
        f = np.ascontiguousarray(self.m_forward, np.float32)
        a = np.ascontiguousarray(axis, np.float32)
        out = np.zeros(3, np.float32)
        lib().venu_camera_rotate(ptr(f), ptr(a), float(degrees), ptr(out))
        self.m_forward = out
        self.m_changed = True

    def Pitch(self, speed: float) -> None:
        self._rotate(self.m_u, speed)

    def Yaw(self, speed: float) -> None:
        self._rotate(self.m_v, speed)

    def Roll(self, speed: float) -> None:
        self._rotate(self.m_w, speed)

    def Changed(self) -> bool:
        c = self.m_changed
        self.m_changed = False
        return c

    def params(self) -> np.ndarray:
        """The venu_camera record (Params origin/u/v/w/lens_radius)."""
        cam = np.zeros(1, CAMERA_DTYPE)
        e = np.ascontiguousarray(self.m_position, np.float32)
        f = np.ascontiguousarray(self.m_forward, np.float32)
        lib().venu_camera_frame(ptr(e), ptr(f), float(self.m_vfov), float(self.m_aspect),
                                float(self.m_aperture), float(self.m_focalLength), ptr(cam))
        self.m_u, self.m_v, self.m_w = cam[0]["u"].copy(), cam[0]["v"].copy(), cam[0]["w"].copy()
        return cam

    def _update_uvw(self) -> None:
        self.params()

    def UVWFrame(self):
        self.params()
        return self.m_u.copy(), self.m_v.copy(), self.m_w.copy()

    @staticmethod
    def look_at(eye, lookat, vfov, aspect, aperture, focal) -> np.ndarray:
        cam = np.zeros(1, CAMERA_DTYPE)
        e = np.asarray(eye, np.float32)
        l = np.asarray(lookat, np.float32)
        lib().venu_camera_look_at(ptr(e), ptr(l), float(vfov), float(aspect), float(aperture),
                                  float(focal), ptr(cam))
        return cam


# ---------------------------------------------------------------------------
# Device scene (LBVH) and closest-hit queries
# ---------------------------------------------------------------------------
class DeviceScene:
    """A venu_scene: spheres uploaded and the LBVH built on the device."""

    def __init__(self, spheres, stream=None):
        arr = spheres.spheres if isinstance(spheres, Scene) else np.ascontiguousarray(spheres, SPHERE_DTYPE)
        self.spheres = arr
        h = C.c_void_p()
        check(lib().venu_scene_create(ptr(arr), len(arr), _stream_handle(stream), C.byref(h)))
        self.handle = h

    @classmethod
    def from_device(cls, spheres_dev, n: int, stream=None) -> "DeviceScene":
        self = cls.__new__(cls)
        self.spheres = None
        h = C.c_void_p()
        check(lib().venu_scene_create_device(ptr(spheres_dev), n, _stream_handle(stream), C.byref(h)))
        self.handle = h
        return self

    def update(self, spheres, stream=None) -> None:
        """Moving spheres: the same count in the same order, new centres /
        radii / materials; the LBVH is refit, not rebuilt (venu_scene_update)."""
        arr = spheres.spheres if isinstance(spheres, Scene) else np.ascontiguousarray(spheres, SPHERE_DTYPE)
        check(lib().venu_scene_update(self.handle, ptr(arr), len(arr), _stream_handle(stream)))
        self.spheres = arr

    def update_device(self, spheres_dev, n: int, stream=None) -> None:
        """As update(), from a device buffer of venu_sphere records (asynchronous)."""
        check(lib().venu_scene_update_device(self.handle, ptr(spheres_dev), n, _stream_handle(stream)))
        self.spheres = None

    def info(self) -> dict:
        si = SceneInfo()
        check(lib().venu_scene_info_get(self.handle, C.byref(si)))
        return dict(num_spheres=si.num_spheres, num_nodes=si.num_nodes, device_bytes=si.device_bytes,
                    bounds=np.array(si.bounds[:], np.float32), build_ms=si.build_ms,
                    num_wide_nodes=si.num_wide_nodes, wide_ms=si.wide_ms)

    def export_bvh(self) -> dict:
        n = self.info()["num_spheres"]
        keys = np.zeros(n, np.uint32)
        ids = np.zeros(n, np.uint32)
        nodes = np.zeros(max(n - 1, 1), NODE_DTYPE)
        check(lib().venu_scene_export_bvh(self.handle, ptr(keys), ptr(ids), ptr(nodes)))
        return dict(keys=keys, ids=ids, nodes=nodes[: max(n - 1, 0)])

    def trace(self, rays, tmin: float = 0.001, tmax: float = 1e16, stream=None):
        """rays: (n, 6) float32 CUDA tensor -> (t, id, front) CUDA tensors."""
        torch = _torch()
        rays = rays.contiguous()
        n = rays.shape[0]
        t = torch.empty(n, dtype=torch.float32, device=rays.device)
        idv = torch.empty(n, dtype=torch.int32, device=rays.device)
        front = torch.empty(n, dtype=torch.int32, device=rays.device)
        check(lib().venu_trace(self.handle, ptr(rays), n, tmin, tmax, ptr(t), ptr(idv), ptr(front),
                               _stream_handle(stream)))
        return t, idv, front

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().venu_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# The plain wavefront renderer
# ---------------------------------------------------------------------------
class Wavefront:
    """A venu_renderer (queues sized for `max_paths` paths per wave)."""

    def __init__(self, max_paths: int = 0, count: bool = False, profile: bool = False):
        h = C.c_void_p()
        flags = (_lib.RENDERER_COUNT if count else 0) | (_lib.RENDERER_PROFILE if profile else 0)
        check(lib().venu_renderer_create(max_paths, flags, C.byref(h)))
        self.handle = h

    def render(self, scene: DeviceScene, camera: np.ndarray, width: int, height: int, spp: int,
               accum, subframe: int = 0, max_depth: int = 4, reset: bool = False,
               image_f=None, image8=None, stream=None) -> None:
        o = RenderOpts(width, height, spp, subframe, max_depth, _lib.FLAG_RESET_ACCUM if reset else 0)
        cam = np.ascontiguousarray(camera, CAMERA_DTYPE)
        check(lib().venu_render(self.handle, scene.handle, ptr(cam), C.byref(o), ptr(accum), ptr(image_f),
                                ptr(image8), _stream_handle(stream)))

    def set_tuning(self, **kw) -> None:
        """Launch shapes / traversal variant (venu_tuning); unspecified fields keep their value."""
        cur = self.tuning()
        cur.update(kw)
        t = Tuning(*(int(cur[f]) for f in TUNING_FIELDS))
        check(lib().venu_renderer_set_tuning(self.handle, C.byref(t)))

    def tuning(self) -> dict:
        t = Tuning()
        check(lib().venu_renderer_get_tuning(self.handle, C.byref(t)))
        return {f: int(getattr(t, f)) for f in TUNING_FIELDS}

    def stats(self) -> dict:
        s = RenderStats()
        check(lib().venu_renderer_stats(self.handle, C.byref(s)))
        return dict(segments=s.segments, paths=s.paths, waves=s.waves, kernel_launches=s.kernel_launches,
                    nodes_visited=s.nodes_visited, spheres_tested=s.spheres_tested,
                    traverse_ms=s.traverse_ms, shade_ms=s.shade_ms, traverse_launches=s.traverse_launches,
                    shade_launches=s.shade_launches, lane_steps=s.lane_steps, warp_steps=s.warp_steps)

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().venu_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_ppm(path: str, rgba8, width: int, height: int) -> None:
    """Binary PPM of a host RGBA8 image in the renderer's pixel order (row 0 =
    bottom): the headless stand-in for the reference's GL display."""
    a = np.ascontiguousarray(np.asarray(rgba8, np.uint8).reshape(-1))
    if a.size != 4 * width * height:
        raise ValueError("write_ppm: image size does not match width x height x 4")
    check(lib().venu_image_write_ppm(os.fsencode(path), ptr(a), width, height))


def write_pfm(path: str, rgbaf, width: int, height: int) -> None:
    """PFM (RGB float32, little-endian) of a host RGBA32F image."""
    a = np.ascontiguousarray(np.asarray(rgbaf, np.float32).reshape(-1))
    if a.size != 4 * width * height:
        raise ValueError("write_pfm: image size does not match width x height x 4")
    check(lib().venu_image_write_pfm(os.fsencode(path), ptr(a), width, height))


def new_accum(width: int, height: int, device="cuda"):
    torch = _torch()
    return torch.zeros((height * width, _lib.ACCUM_FLOATS), dtype=torch.float32, device=device)


# ---------------------------------------------------------------------------
# CUDAOutputBuffer (CUDA_DEVICE mode) and Renderer (Core/Renderer.h:22-97)
# ---------------------------------------------------------------------------
class CUDAOutputBuffer:
    """Device pixel buffer (Core/CUDAOutputBuffer.h, CUDA_DEVICE mode only:
    there is no GL interop).  Holds sRGB RGBA8 and linear RGBA32F images."""

    def __init__(self, width: int, height: int, device="cuda"):
        self.m_device = device
        self.resize(width, height)

    def resize(self, width: int, height: int) -> None:
        torch = _torch()
        self.m_width = max(1, int(width))
        self.m_height = max(1, int(height))
        self.pixels = torch.zeros((self.m_height, self.m_width, 4), dtype=torch.uint8, device=self.m_device)
        self.pixels_f = torch.zeros((self.m_height, self.m_width, 4), dtype=torch.float32, device=self.m_device)

    def width(self) -> int:
        return self.m_width

    def height(self) -> int:
        return self.m_height

    def map(self):
        return self.pixels

    def unmap(self) -> None:
        _torch().cuda.current_stream().synchronize()

    def getHostPointer(self) -> np.ndarray:
        return self.pixels.cpu().numpy()

    def getHostFloat(self) -> np.ndarray:
        return self.pixels_f.cpu().numpy()

    def writePPM(self, path: str) -> None:
        write_ppm(path, self.getHostPointer(), self.m_width, self.m_height)

    def writePFM(self, path: str) -> None:
        write_pfm(path, self.getHostFloat(), self.m_width, self.m_height)


class Renderer:
    """Renderer::Init / Draw / Cleanup over the wavefront kernels.

    Draw renders `samples_per_pixel` samples per pixel (16, as
    Core/Renderer.h:53) seeded with tea<4>(pixel, subframe_index) and adds
    them to a Kahan-compensated accumulator; a camera change resets it and
    restarts subframe_index at 1, as Core/Renderer.h:37-54 does.
    """

    def __init__(self, samples_per_pixel: int = 16, max_depth: int = 4, max_paths: int = 0):
        self.samples_per_pixel = samples_per_pixel
        self.max_depth = max_depth
        self.max_paths = max_paths
        self.scene = None
        self.wave = None
        self.accum = None
        self.subframe_index = 0

    def Init(self, scene: Scene, ptxSource: str | None = None) -> None:
        """ptxSource is accepted for signature parity and ignored (no PTX JIT)."""
        self.scene = DeviceScene(scene)
        self.wave = Wavefront(self.max_paths)
        self._scene_changed = False

    def Update(self, scene: Scene) -> None:
        """Moving spheres (no reference counterpart): the same spheres
        re-posed; the LBVH is refit and the progressive accumulation restarts."""
        self.scene.update(scene)
        self._scene_changed = True

    def Draw(self, camera: Camera, outputBuffer: CUDAOutputBuffer) -> None:
        W, H = outputBuffer.width(), outputBuffer.height()
        reset = False
        scene_changed, self._scene_changed = getattr(self, "_scene_changed", False), False
        if camera.Changed() or scene_changed or self.accum is None or self.accum.shape[0] != W * H:
            self.accum = new_accum(W, H, outputBuffer.m_device)
            self.subframe_index = 0
            reset = True
        self.subframe_index += 1
        self.wave.render(self.scene, camera.params(), W, H, self.samples_per_pixel, self.accum,
                         subframe=self.subframe_index, max_depth=self.max_depth, reset=reset,
                         image_f=outputBuffer.pixels_f, image8=outputBuffer.pixels)
        outputBuffer.unmap()

    def Cleanup(self) -> None:
        if self.wave is not None:
            self.wave.close()
        if self.scene is not None:
            self.scene.close()
        self.wave = self.scene = self.accum = None


# ---------------------------------------------------------------------------
# Batched / served rendering: many jobs in one shared path pool
# ---------------------------------------------------------------------------
def _camera_c(camera: np.ndarray) -> "_lib.CameraC":
    # CAMERA_DTYPE and venu_camera have the same 52-byte layout
    c = np.ascontiguousarray(camera, CAMERA_DTYPE).reshape(-1)[:1]
    return _lib.CameraC.from_buffer_copy(c.tobytes())


def _policy(policy) -> int:
    if isinstance(policy, bool):
        return _lib.POLICY_SHORTEST_FIRST if policy else _lib.POLICY_FIFO
    return _lib.POLICIES[policy]


class Batch:
    """A venu_batch: jobs admitted with submit(), advanced together by run(),
    finished ones accumulated and released by collect()."""

    def __init__(self, pool_paths: int = 0, max_jobs: int = 256, graph: bool = True):
        h = C.c_void_p()
        check(lib().venu_batch_create(pool_paths, max_jobs, 0 if graph else _lib.BATCH_NO_GRAPH, C.byref(h)))
        self.handle = h
        self.max_jobs = max_jobs

    def set_tuning(self, **kw) -> None:
        base = dict(traverse_variant=2, refill_min=8, traverse_block=256, traverse_blocks_per_sm=0,
                    shade_block=256, shade_blocks_per_sm=0, in_place_factor=1)
        base.update(kw)
        t = Tuning(*(int(base[f]) for f in TUNING_FIELDS))
        check(lib().venu_batch_set_tuning(self.handle, C.byref(t)))

    @staticmethod
    def job_bytes(width: int, height: int, spp: int) -> int:
        return int(lib().venu_batch_job_bytes(width, height, spp))

    def submit(self, scene: DeviceScene, camera: np.ndarray, width: int, height: int, spp: int, accum,
               subframe: int = 1, max_depth: int = 50, reset: bool = True, image_f=None, image8=None,
               stream=None) -> int:
        d = _lib.JobDesc()
        d.scene = scene.handle.value
        d.camera = _camera_c(camera)
        d.opts = RenderOpts(width, height, spp, subframe, max_depth, _lib.FLAG_RESET_ACCUM if reset else 0)
        d.accum = ptr(accum).value
        d.image_f = ptr(image_f).value if image_f is not None else None
        d.image8 = ptr(image8).value if image8 is not None else None
        jid = C.c_uint32()
        check(lib().venu_batch_submit(self.handle, C.byref(d), _stream_handle(stream), C.byref(jid)))
        return int(jid.value)

    def submit_many(self, jobs, stream=None) -> list:
        """Admits several jobs with one call (venu_batch_submit_many): each a
        dict of submit()'s arguments (scene, camera, width, height, spp,
        accum, and optionally subframe, max_depth, reset, image_f, image8).
        All or nothing; returns the job ids in order."""
        n = len(jobs)
        arr = (_lib.JobDesc * max(1, n))()
        for d, j in zip(arr, jobs):
            d.scene = j["scene"].handle.value
            d.camera = _camera_c(j["camera"])
            d.opts = RenderOpts(j["width"], j["height"], j["spp"], j.get("subframe", 1), j.get("max_depth", 50),
                                _lib.FLAG_RESET_ACCUM if j.get("reset", True) else 0)
            d.accum = ptr(j["accum"]).value
            d.image_f = ptr(j["image_f"]).value if j.get("image_f") is not None else None
            d.image8 = ptr(j["image8"]).value if j.get("image8") is not None else None
        ids = (C.c_uint32 * max(1, n))()
        check(lib().venu_batch_submit_many(self.handle, arr, n, _stream_handle(stream), ids))
        return [int(ids[k]) for k in range(n)]

    def run(self, max_iterations: int = 0, stop_on_finish: bool = False, stream=None) -> None:
        flags = _lib.RUN_STOP_ON_FINISH if stop_on_finish else 0
        check(lib().venu_batch_run(self.handle, max_iterations, flags, _stream_handle(stream)))

    def set_policy(self, policy) -> None:
        """Plan order: "fifo", "shortest_first" or "sequential" (a bool selects
        shortest_first / fifo)."""
        check(lib().venu_batch_set_policy(self.handle, _policy(policy)))

    def set_chunk(self, rays: int) -> None:
        """Rays traced per loop step (0: whole iterations)."""
        check(lib().venu_batch_set_chunk(self.handle, int(rays)))

    def interrupt(self, on: bool = True) -> None:
        """Ends a running run() at its next iteration boundary while set."""
        check(lib().venu_batch_interrupt(self.handle, 1 if on else 0))

    def collect(self, stream=None) -> list:
        ids = (C.c_uint32 * self.max_jobs)()
        n = C.c_uint32()
        check(lib().venu_batch_collect(self.handle, _stream_handle(stream), ids, self.max_jobs, C.byref(n)))
        return [int(ids[i]) for i in range(min(n.value, self.max_jobs))]

    def stats(self) -> dict:
        s = _lib.BatchStats()
        check(lib().venu_batch_stats_get(self.handle, C.byref(s)))
        return {f: int(getattr(s, f)) for f, _ in _lib.BatchStats._fields_ if f != "reserved"}

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().venu_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A venu_server: requests are admitted FIFO under an HBM budget and
    rendered together in one shared path pool by the server's own thread."""

    def __init__(self, hbm_budget_bytes: int, pool_paths: int = 0, max_jobs: int = 64,
                 iterations_per_step: int = 8, shortest_first: bool = False, express_paths: int = 0):
        h = C.c_void_p()
        check(lib().venu_server_create(int(hbm_budget_bytes), pool_paths, max_jobs, iterations_per_step,
                                       C.byref(h)))
        self.handle = h
        if shortest_first:
            self.set_policy("shortest_first")
        if express_paths:
            self.set_express(express_paths)

    def end_session(self, session: int) -> None:
        check(lib().venu_server_end_session(self.handle, session))

    def set_express(self, max_paths: int) -> None:
        """Requests of at most max_paths paths run in the express lane (0: off)."""
        check(lib().venu_server_set_express(self.handle, int(max_paths)))

    def set_policy(self, policy) -> None:
        """Plan order of the bulk lane: "fifo", "shortest_first" or "sequential"."""
        check(lib().venu_server_set_policy(self.handle, _policy(policy)))

    def submit(self, camera: np.ndarray, width: int, height: int, spp: int, spheres=None, scene_key: int = 0,
               subframe: int = 1, max_depth: int = 50, tag: int = 0, session: int = 0, reset: bool = False) -> int:
        """session != 0: add to that progressive session's accumulator (reset=True
        restarts it); the image returned is the running mean."""
        r = _lib.Request()
        arr = None
        if spheres is not None:
            arr = np.ascontiguousarray(spheres, SPHERE_DTYPE)
            r.spheres = arr.ctypes.data
            r.num_spheres = len(arr)
        r.scene_key = scene_key
        r.camera = _camera_c(camera)
        r.opts = RenderOpts(width, height, spp, subframe, max_depth, _lib.FLAG_RESET_ACCUM if reset else 0)
        r.tag = tag
        r.session = session
        rid = C.c_uint64()
        check(lib().venu_server_submit(self.handle, C.byref(r), C.byref(rid)))
        return int(rid.value)

    def wait(self, request_id: int, timeout_s: float = 600.0, release: bool = True) -> dict:
        res = _lib.Result()
        check(lib().venu_server_wait(self.handle, request_id, timeout_s, C.byref(res)))
        image = None
        if res.image8:
            n = res.width * res.height * 4
            image = np.ctypeslib.as_array((C.c_uint8 * n).from_address(res.image8)).copy().reshape(
                res.height, res.width, 4)
        out = dict(request_id=res.request_id, tag=res.tag, status=res.status, image=image, t_submit=res.t_submit,
                   t_admit=res.t_admit, t_done=res.t_done, latency_ms=1000.0 * (res.t_done - res.t_submit))
        if release:
            lib().venu_server_release(self.handle, request_id)
        return out

    def cancel(self, request_id: int) -> None:
        check(lib().venu_server_cancel(self.handle, request_id))

    def inject(self, what: int) -> None:
        check(lib().venu_server_inject(self.handle, what))

    def stats(self) -> dict:
        s = _lib.ServerStats()
        check(lib().venu_server_stats_get(self.handle, C.byref(s)))
        return {f: getattr(s, f) for f, _ in _lib.ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().venu_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
