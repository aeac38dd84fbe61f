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


def _build_noalloc(venu, torch, spheres, with_nodes=True):
    f = _fn(venu)
    n = len(spheres)
    dev_sph = torch.from_numpy(spheres.view(np.uint8).reshape(-1).copy()).cuda()
    # outputs deliberately filled with garbage: nothing may depend on them
    nodes = torch.full((max(n - 1, 1) * 8,), 7.0, dtype=torch.float32, device="cuda")
    nodes_ptr = C.c_void_p(nodes.data_ptr()) if with_nodes else None
    sph = torch.full((n * 4,), 7.0, dtype=torch.float32, device="cuda")
    mat = torch.full((n * 4,), 7.0, dtype=torch.float32, device="cuda")
    meta = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    morton = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = f(C.c_void_p(dev_sph.data_ptr()), n, nodes_ptr, C.c_void_p(sph.data_ptr()),
           C.c_void_p(mat.data_ptr()), C.c_void_p(meta.data_ptr()), C.c_void_p(morton.data_ptr()), stream)
    assert st == 0, venu.lib().venu_last_error()
    torch.cuda.synchronize()
    return dict(nodes=nodes.cpu().numpy()[: 8 * (n - 1)], sph=sph.cpu().numpy().reshape(n, 4),
                mat=mat.cpu().numpy().reshape(n, 4), meta=meta.cpu().numpy().view(np.uint32),
                morton=morton.cpu().numpy().view(np.uint32))


def _edge_scenes(venu):
    """The LBVH edge cases of the allocating build's tests: 1 and 2 spheres,
    many equal Morton codes, nine more r=1000 spheres spread far apart, and
    seventy in a row."""
    rt = venu.generate_rtiow(0)
    dups = venu.generate_random(3000, 4)
    dups["center"][100:900] = dups["center"][100]
    many = venu.generate_rtiow(0)[:9].copy()
    many["center"][:, 0] = np.arange(9) * 3000.0 - 12000.0
    many["center"][:, 1] = -1000.0
    many["radius"] = 1000.0
    many = np.concatenate([rt, many])
    too_many = np.repeat(rt[:1], 70)
    too_many["center"][:, 0] = np.arange(70) * 2500.0 - 80000.0
    too_many = np.concatenate([rt, too_many])
    return {"n1": rt[:1].copy(), "n2": rt[:2].copy(), "dups": dups, "many_huge": many, "too_many_huge": too_many}


def _check(venu, got, sp):
    want = venu.DeviceScene(sp).export_bvh()
    assert np.array_equal(got["morton"], want["keys"])
    assert np.array_equal(got["meta"] & 0x3FFFFFFF, want["ids"])
    assert got["nodes"].tobytes() == want["nodes"].tobytes()
    ids = want["ids"]
    assert np.array_equal(got["sph"][:, :3], sp["center"][ids])
    assert np.array_equal(got["sph"][:, 3], sp["radius"][ids])
    assert np.array_equal(got["mat"][:, :3], sp["albedo"][ids])
    assert np.array_equal(got["meta"] >> 30, sp["material"][ids])
    return want


def test_noalloc_matches_scene_create(venu, cuda):
    torch = cuda
    scenes = [venu.generate_rtiow(0), venu.generate_random(20_000, 3), venu.generate_random(MAX_SPHERES, 4)]
    # consecutive calls: sizes go up, then back down to the first scene
    for sp in scenes + scenes[:1]:
        _check(venu, _build_noalloc(venu, torch, sp), sp)


def test_noalloc_edge_scenes(venu, cuda):
    torch = cuda
    edge = _edge_scenes(venu)
    # n = 1 has no internal node: the nodes output may be NULL
    _check(venu, _build_noalloc(venu, torch, edge["n1"], with_nodes=False), edge["n1"])
    hoisted = {}
    for name in ("n2", "dups", "many_huge", "too_many_huge", "n1"):
        want = _check(venu, _build_noalloc(venu, torch, edge[name]), edge[name])
        words = want["nodes"]["left"].tolist() + want["nodes"]["right"].tolist()
        hoisted[name] = sum(1 for w in words if (w & 0xC0000000) == 0xC0000000)
    # the ground sphere of a small scene is hoisted (its leaf carries both
    # flags); spread-out huge spheres are not
    assert hoisted["n2"] == 1 and hoisted["dups"] == 1 and hoisted["many_huge"] == 0


def test_noalloc_rejects_too_large(venu, cuda):
    f = _fn(venu)
    st = f(None, MAX_SPHERES + 1, None, None, None, None, None, None)
    assert st == 8  # VENU_ERR_TOO_LARGE
    assert b"65536" in venu.lib().venu_last_error()
