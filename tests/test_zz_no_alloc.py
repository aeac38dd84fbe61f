"""venu_lbvh_build_noalloc: the LBVH build for callers that cannot allocate
device memory (an engine that owns all HBM through its own pool, or a
per-frame rebuild that cannot take cudaMalloc's device synchronisation).

It must produce exactly what venu_scene_create builds (the tolerance of every
LBVH test here: bit-exact), call after call, although all calls share one
fixed scratch array that keeps the previous call's contents.  The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_SPHERES = 65536  # VENU_NOALLOC_MAX_SPHERES


def _fn(venu):
    L = venu.lib()
    f = L.venu_lbvh_build_noalloc
    f.argtypes = [C.c_void_p, C.c_uint32] + [C.c_void_p] * 6
    f.restype = C.c_int
    return f


def _build_noalloc(venu, torch, spheres):
    f = _fn(venu)
    n = len(spheres)
    dev_sph = torch.from_numpy(spheres.view(np.uint8).reshape(-1).copy()).cuda()
    # outputs deliberately filled with garbage: nothing may depend on them
    nodes = torch.full((max(n - 1, 1) * 8,), 7.0, dtype=torch.float32, device="cuda")
    sph = torch.full((n * 4,), 7.0, dtype=torch.float32, device="cuda")
    mat = torch.full((n * 4,), 7.0, dtype=torch.float32, device="cuda")
    meta = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    morton = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = f(C.c_void_p(dev_sph.data_ptr()), n, C.c_void_p(nodes.data_ptr()), C.c_void_p(sph.data_ptr()),
           C.c_void_p(mat.data_ptr()), C.c_void_p(meta.data_ptr()), C.c_void_p(morton.data_ptr()), stream)
    assert st == 0, venu.lib().venu_last_error()
    torch.cuda.synchronize()
    return dict(nodes=nodes.cpu().numpy()[: 8 * (n - 1)], sph=sph.cpu().numpy().reshape(n, 4),
                mat=mat.cpu().numpy().reshape(n, 4), meta=meta.cpu().numpy().view(np.uint32),
                morton=morton.cpu().numpy().view(np.uint32))


def test_noalloc_matches_scene_create(venu, cuda):
    torch = cuda
    scenes = [venu.generate_rtiow(0), venu.generate_random(20_000, 3), venu.generate_random(MAX_SPHERES, 4)]
    # consecutive calls: sizes go up, then back down to the first scene
    for sp in scenes + scenes[:1]:
        got = _build_noalloc(venu, torch, sp)
        want = venu.DeviceScene(sp).export_bvh()
        assert np.array_equal(got["morton"], want["keys"])
        assert np.array_equal(got["meta"] & 0x3FFFFFFF, want["ids"])
        assert got["nodes"].tobytes() == want["nodes"].tobytes()
        ids = want["ids"]
        assert np.array_equal(got["sph"][:, :3], sp["center"][ids])
        assert np.array_equal(got["sph"][:, 3], sp["radius"][ids])
        assert np.array_equal(got["mat"][:, :3], sp["albedo"][ids])
        assert np.array_equal(got["meta"] >> 30, sp["material"][ids])


def test_noalloc_rejects_too_large(venu, cuda):
    f = _fn(venu)
    st = f(None, MAX_SPHERES + 1, None, None, None, None, None, None)
    assert st == 8  # VENU_ERR_TOO_LARGE
    assert b"65536" in venu.lib().venu_last_error()
