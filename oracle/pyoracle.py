"""ctypes binding for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
reference arm, always as the checker, never as the thing measured or shipped.

``Oracle`` wraps oracle/_build/libvenu_oracle.so (the C++ restatement of the
reference's Core/RayTracer.cu path tracer, see venu_oracle.h).  ``RefBuild``
wraps oracle/_ref/libvenu_ref.so: the reference's own Core/RayTracer.cu
compiled for the host (only where the reference sources are present).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libvenu_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvenu_ref.so")

SPHERE_DTYPE = np.dtype([
    ("center", "<f4", (3,)), ("radius", "<f4"), ("albedo", "<f4", (3,)),
    ("fuzz", "<f4"), ("ir", "<f4"), ("material", "<u4"), ("pad", "<u4", (2,)),
])
assert SPHERE_DTYPE.itemsize == 48
CAMERA_DTYPE = np.dtype([
    ("origin", "<f4", (3,)), ("u", "<f4", (3,)), ("v", "<f4", (3,)),
    ("w", "<f4", (3,)), ("lens_radius", "<f4"),
])
NODE_DTYPE = np.dtype([("lo", "<f4", (3,)), ("left", "<i4"), ("hi", "<f4", (3,)), ("right", "<i4")])

MODE_REF = 0
MODE_GB300 = 1
MODE_REF_BVH = 2  # the reference's arithmetic, closest hit through the host LBVH


class _Opts(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in (
        "width", "height", "spp", "subframe_index", "max_depth", "mode", "nthreads",
        "row_begin", "row_end")]


def build(ref_root: str | None = None, with_ref: bool = False) -> None:
    """Compile the oracle and, if asked, the reference build (from ref_root,
    else the recipe's own REF_ROOT; skipped where no checkout is there)."""
    cmd = ["make", "-s", "-C", HERE, "all"]
    subprocess.run(cmd, check=True)
    if with_ref:
        extra = [f"REF_ROOT={ref_root}"] if ref_root else []
        subprocess.run(["make", "-s", "-C", HERE, "ref"] + extra, check=True)


def _p(a, t=C.c_void_p):
    return None if a is None else C.cast(a.ctypes.data, t)


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        self.L = L
        L.vo_tea4.restype = C.c_uint32
        L.vo_tea4.argtypes = [C.c_uint32, C.c_uint32]
        L.vo_scene_rtiow.restype = C.c_uint32
        L.vo_scene_random.restype = C.c_uint32
        L.vo_render.restype = C.c_uint64
        L.vo_render_refit.restype = C.c_uint64

    # RNG ---------------------------------------------------------------
    def tea4(self, a: int, b: int) -> int:
        return int(self.L.vo_tea4(a, b))

    def rnd_stream(self, seed: int, n: int):
        out = np.zeros(n, np.float32)
        st = np.zeros(n, np.uint32)
        self.L.vo_rnd_stream(C.c_uint32(seed), C.c_uint32(n), _p(out), _p(st))
        return out, st

    # scenes --------------------------------------------------------------
    def scene_rtiow(self, seed: int = 0) -> np.ndarray:
        buf = np.zeros(600, SPHERE_DTYPE)
        n = self.L.vo_scene_rtiow(C.c_uint32(seed), _p(buf), C.c_uint32(len(buf)))
        return buf[:n].copy()

    def scene_random(self, n: int, seed: int, box_lo=(-100, 0, -100), box_hi=(100, 20, 100),
                     rmin=0.01, rmax=0.5) -> np.ndarray:
        out = np.zeros(n, SPHERE_DTYPE)
        lo = np.asarray(box_lo, np.float32)
        hi = np.asarray(box_hi, np.float32)
        self.L.vo_scene_random(C.c_uint32(n), C.c_uint32(seed), _p(lo), _p(hi),
                               C.c_float(rmin), C.c_float(rmax), _p(out))
        return out

    def camera(self, eye, lookat, vfov, aspect, aperture, focal) -> np.ndarray:
        cam = np.zeros(1, CAMERA_DTYPE)
        e = np.asarray(eye, np.float32)
        l = np.asarray(lookat, np.float32)
        self.L.vo_camera_look_at(_p(e), _p(l), C.c_float(vfov), C.c_float(aspect),
                                 C.c_float(aperture), C.c_float(focal), _p(cam))
        return cam

    # LBVH ----------------------------------------------------------------
    def lbvh(self, spheres: np.ndarray):
        n = len(spheres)
        keys = np.zeros(n, np.uint32)
        ids = np.zeros(n, np.uint32)
        nodes = np.zeros(max(n - 1, 1), NODE_DTYPE)
        bounds = np.zeros(6, np.float32)
        depth = np.zeros(1, np.uint32)
        self.L.vo_lbvh_build(_p(spheres), C.c_uint32(n), _p(keys), _p(ids), _p(nodes),
                             _p(bounds), _p(depth))
        return dict(keys=keys, ids=ids, nodes=nodes[: max(n - 1, 0)], bounds=bounds,
                    depth=int(depth[0]))

    def lbvh_refit(self, spheres_build: np.ndarray, spheres_new: np.ndarray):
        """Nodes of the LBVH built on spheres_build, moved to spheres_new and
        refit (same topology, slot order and hoisted set)."""
        n = len(spheres_build)
        assert len(spheres_new) == n
        nodes = np.zeros(max(n - 1, 1), NODE_DTYPE)
        self.L.vo_lbvh_refit(_p(spheres_build), _p(spheres_new), C.c_uint32(n), _p(nodes))
        return nodes[: max(n - 1, 0)]

    # closest hit -----------------------------------------------------------
    def trace_fp64(self, spheres, rays, tmin=0.001, tmax=1e16):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        idv = np.zeros(n, np.int32)
        t = np.zeros(n, np.float64)
        disc = np.zeros(n, np.float64)
        t2 = np.zeros(n, np.float64)
        self.L.vo_trace_fp64(_p(spheres), C.c_uint32(len(spheres)), _p(rays), C.c_uint32(n),
                             C.c_float(tmin), C.c_float(tmax), _p(idv), _p(t), _p(disc), _p(t2))
        return idv, t, disc, t2

    def trace_bvh(self, spheres, rays, tmin=0.001, tmax=1e16):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        idv = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        front = np.zeros(n, np.uint32)
        nv = np.zeros(n, np.uint32)
        ns = np.zeros(n, np.uint32)
        self.L.vo_trace_bvh(_p(spheres), C.c_uint32(len(spheres)), _p(rays), C.c_uint32(n),
                            C.c_float(tmin), C.c_float(tmax), _p(idv), _p(t), _p(front),
                            _p(nv), _p(ns))
        return idv, t, front, nv, ns

    def trace_stack_depth(self, spheres, rays, tmin=0.001, tmax=1e16):
        """Per ray, the deepest traversal stack of the GB300 LBVH walk."""
        rays = np.ascontiguousarray(rays, np.float32)
        out = np.zeros(len(rays), np.uint32)
        self.L.vo_trace_bvh_stack(_p(spheres), C.c_uint32(len(spheres)), _p(rays), C.c_uint32(len(rays)),
                                  C.c_float(tmin), C.c_float(tmax), _p(out))
        return out

    def trace_ref(self, spheres, rays, tmin=0.001, tmax=1e16):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        idv = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        self.L.vo_trace_ref(_p(spheres), C.c_uint32(len(spheres)), _p(rays), C.c_uint32(n),
                            C.c_float(tmin), C.c_float(tmax), _p(idv), _p(t))
        return idv, t

    # render --------------------------------------------------------------
    def render(self, spheres, cam, width, height, spp, subframe=0, max_depth=4,
               mode=MODE_GB300, accum=None, nthreads=0, rows=None, want_samples=False, built_from=None):
        """Returns dict(accum, image_f, image8, segments, samples, nodes, spheres).

        GB300 mode: accum is (H*W, 8) float32 {sum.rgb, n, comp.rgb, 0}, updated
        in place (zeros = reset).  REF mode: accum is (H*W, 4) {mean.rgb, 1}.
        built_from: spheres the LBVH was built on before being refit to
        `spheres` (moving spheres); None = built on `spheres`.
        """
        npx = width * height
        if accum is None:
            accum = np.zeros((npx, 8 if mode == MODE_GB300 else 4), np.float32)
        image_f = np.zeros((npx, 4), np.float32)
        image8 = np.zeros((npx, 4), np.uint8)
        r0, r1 = (0, 0) if rows is None else rows
        nrows = height if rows is None else (r1 - r0)
        samples = np.zeros((spp, nrows * width, 3), np.float32) if want_samples else None
        o = _Opts(width, height, spp, subframe, max_depth, mode, nthreads, r0, r1)
        nv = np.zeros(1, np.uint64)
        ns = np.zeros(1, np.uint64)
        if built_from is not None:
            assert len(built_from) == len(spheres)
        segs = self.L.vo_render_refit(_p(built_from), _p(spheres), C.c_uint32(len(spheres)), _p(cam), C.byref(o),
                                      _p(accum), _p(image_f), _p(image8), _p(samples), _p(nv), _p(ns))
        return dict(accum=accum, image_f=image_f, image8=image8, segments=int(segs),
                    samples=samples, nodes=int(nv[0]), spheres=int(ns[0]))

    def srgb_pow(self, x) -> np.ndarray:
        """x^(1/2.4) by the GB300 arithmetic's power routine (x in [2^-126, 1])."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1)
        out = np.empty_like(x)
        self.L.vo_srgb_pow(_p(x), C.c_uint64(len(x)), _p(out))
        return out

    def make_color_gb300(self, rgb) -> np.ndarray:
        rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
        out = np.zeros((len(rgb), 4), np.uint8)
        self.L.vo_make_color_gb300(_p(rgb), C.c_uint32(len(rgb)), _p(out))
        return out

    def make_color(self, rgb) -> np.ndarray:
        rgb = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
        out = np.zeros((len(rgb), 4), np.uint8)
        self.L.vo_make_color(_p(rgb), C.c_uint32(len(rgb)), _p(out))
        return out


class RefBuild:
    """The reference's own Core/RayTracer.cu compiled for the host."""

    def __init__(self, path: str = REF_SO):
        self.L = C.CDLL(path)
        self.L.vr_tea4.restype = C.c_uint32
        self.L.vr_tea4.argtypes = [C.c_uint32, C.c_uint32]

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def tea4(self, a, b):
        return int(self.L.vr_tea4(a, b))

    def rnd_stream(self, seed, n):
        out = np.zeros(n, np.float32)
        st = np.zeros(n, np.uint32)
        self.L.vr_rnd_stream(C.c_uint32(seed), C.c_uint32(n), _p(out), _p(st))
        return out, st

    def render(self, spheres, cam, width, height, spp, subframe=0, accum=None, nthreads=0):
        npx = width * height
        if accum is None:
            accum = np.zeros((npx, 4), np.float32)
        image8 = np.zeros((npx, 4), np.uint8)
        c = np.concatenate([cam["origin"][0], cam["u"][0], cam["v"][0], cam["w"][0],
                            [cam["lens_radius"][0]]]).astype(np.float32)
        self.L.vr_render(_p(spheres), C.c_uint32(len(spheres)), _p(c), C.c_uint32(width),
                         C.c_uint32(height), C.c_uint32(spp), C.c_uint32(subframe), _p(accum),
                         _p(image8), C.c_uint32(nthreads))
        return dict(accum=accum, image8=image8)
