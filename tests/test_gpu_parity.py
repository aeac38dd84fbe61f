"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Bars:
  * LBVH (Morton codes, sorted order, Karras topology, node boxes): bit-exact;
  * closest hit for arbitrary rays: bit-exact against the oracle's FP32
    traversal; sphere id equal and t within 1e-5 relative of the FP64
    brute-force oracle for well-conditioned rays (not within ~0.6 degrees of
    tangency, no second sphere within 1e-4 relative);
  * rendering: the accumulator (Kahan sums, sample counts), the float image
    and the segment count are bit-exact against the oracle's GB300 arithmetic,
    at several wave shapes; sRGB bytes within 1 (powf differs by an ulp
    between the device and host libm).
"""
import os

import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


def _dev_scene(venu, spheres):
    return venu.DeviceScene(spheres)


def test_device_is_sm103(venu, cuda):
    import ctypes as C

    sms, ma, mi = C.c_int(), C.c_int(), C.c_int()
    st = venu.lib().venu_device_check(C.byref(sms), C.byref(ma), C.byref(mi))
    assert st == 0, venu.lib().venu_last_error()
    assert (ma.value, mi.value) == (10, 3)
    assert sms.value >= 100


@pytest.mark.parametrize("case", ["rtiow", "n1", "n2", "n3", "rand1k", "rand100k", "dups"])
def test_lbvh_bit_exact(venu, oracle, cuda, case):
    if case == "rtiow":
        sp = oracle.scene_rtiow(0)
    elif case.startswith("n"):
        sp = oracle.scene_rtiow(1)[: int(case[1:])]
    elif case == "rand1k":
        sp = oracle.scene_random(1000, 1)
    elif case == "rand100k":
        sp = oracle.scene_random(100_000, 2)
    else:
        sp = oracle.scene_random(3000, 4)
        sp["center"][100:900] = sp["center"][100]  # many equal Morton codes
    ds = _dev_scene(venu, sp)
    got = ds.export_bvh()
    want = oracle.lbvh(sp)
    assert np.array_equal(got["keys"], want["keys"])
    assert np.array_equal(got["ids"], want["ids"])
    assert got["nodes"].tobytes() == want["nodes"].tobytes()
    info = ds.info()
    assert info["num_spheres"] == len(sp)
    assert np.array_equal(info["bounds"], want["bounds"]) or len(sp) == 0


def test_lbvh_golden(venu, cuda):
    g = np.load(GOLDEN)
    sp = g["scene"].reshape(-1).view(pyoracle.SPHERE_DTYPE)
    got = _dev_scene(venu, sp).export_bvh()
    assert np.array_equal(got["keys"], g["bvh_keys"])
    assert np.array_equal(got["ids"], g["bvh_ids"])
    assert got["nodes"].view(np.uint8).tobytes() == g["bvh_nodes"].tobytes()


def _random_rays(n, seed, lo=(-12, 0.01, -12), hi=(14, 4, 12)):
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(lo[i], hi[i], n) for i in range(3)], 1)
    d = rng.normal(size=(n, 3))
    return np.concatenate([o, d], 1).astype(np.float32)


@pytest.mark.parametrize("scene", ["rtiow", "rand50k"])
def test_trace_matches_oracle(venu, oracle, cuda, scene):
    torch = cuda
    if scene == "rtiow":
        sp = oracle.scene_rtiow(0)
        rays = _random_rays(30000, 5)
    else:
        sp = oracle.scene_random(50_000, 6)
        rays = _random_rays(30000, 7, lo=(-100, 0, -100), hi=(100, 25, 100))
    ds = _dev_scene(venu, sp)
    t, idv, front = ds.trace(torch.from_numpy(rays).cuda())
    t, idv, front = t.cpu().numpy(), idv.cpu().numpy(), front.cpu().numpy()
    ob, tb, fb, _, _ = oracle.trace_bvh(sp, rays)
    assert np.array_equal(idv, ob)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
    assert np.array_equal(front.astype(np.uint32), fb)
    # FP64 brute force: closest sphere and 1e-5 relative t
    id64, t64, disc, t2 = oracle.trace_fp64(sp, rays)
    well = (id64 >= 0) & (disc > 1e-4) & (t2 > t64 * (1 + 1e-4))
    assert well.sum() > 1000
    assert np.array_equal(idv[well], id64[well])
    rel = np.abs(t[well].astype(np.float64) - t64[well]) / t64[well]
    assert rel.max() < 1e-5, rel.max()
    assert ((idv < 0) == (id64 < 0)).mean() > 0.999


def test_trace_secondary_rays(venu, oracle, cuda):
    """Rays leaving sphere surfaces (the hard case for the quadratic)."""
    torch = cuda
    sp = oracle.scene_rtiow(0)
    rays = _random_rays(30000, 8)
    ds = _dev_scene(venu, sp)
    t, idv, _ = ds.trace(torch.from_numpy(rays).cuda())
    t, idv = t.cpu().numpy(), idv.cpu().numpy()
    h = idv >= 0
    p = rays[h, :3] + rays[h, 3:] * t[h, None]
    d = np.random.default_rng(9).normal(size=p.shape)
    rays2 = np.concatenate([p, d], 1).astype(np.float32)
    t2, id2, _ = ds.trace(torch.from_numpy(rays2).cuda())
    t2, id2 = t2.cpu().numpy(), id2.cpu().numpy()
    ob, tb, _, _, _ = oracle.trace_bvh(sp, rays2)
    assert np.array_equal(id2, ob) and np.array_equal(t2.view(np.uint32), tb.view(np.uint32))
    id64, t64, disc, tsec = oracle.trace_fp64(sp, rays2)
    well = (id64 >= 0) & (disc > 1e-4) & (tsec > t64 * (1 + 1e-4))
    assert np.array_equal(id2[well], id64[well])
    assert (np.abs(t2[well].astype(np.float64) - t64[well]) / t64[well]).max() < 1e-5


def test_trace_near_axis_parallel_rays(venu, oracle, cuda):
    """Directions with components exactly zero or tiny (1/d up to 1e20) take
    the per-axis slab margins: GPU equals the oracle bit for bit, and every
    ray's closest hit is the FP64 brute force's."""
    torch = cuda
    from tests.test_oracle import _axis_rays

    sp = oracle.scene_random(50_000, 6)
    rays = _axis_rays(4000, 3)
    ds = _dev_scene(venu, sp)
    t, idv, front = ds.trace(torch.from_numpy(rays).cuda())
    t, idv, front = t.cpu().numpy(), idv.cpu().numpy(), front.cpu().numpy()
    ob, tb, fb, _, _ = oracle.trace_bvh(sp, rays)
    assert np.array_equal(idv, ob)
    assert np.array_equal(t.view(np.uint32), tb.view(np.uint32))
    assert np.array_equal(front.astype(np.uint32), fb)


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_render_wide_scene_every_variant(venu, oracle, cuda, variant):
    """A 20k-sphere field 200 units wide seen from inside: among its ~300k
    segments about one in 10^4 has a direction component small enough for
    the per-axis slab margins, in every traversal variant (the dynamic-fetch
    kernel traces those rays on their own).  Accumulator and box / sphere
    test counts equal the oracle's."""
    torch = cuda
    sp = oracle.scene_random(20_000, 11)
    W, H, spp, depth = 64, 48, 16, 8
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    wf = venu.Wavefront(1 << 16, count=True)
    wf.set_tuning(traverse_variant=variant, refill_min=8, traverse_block=128, shade_block=256)
    accum = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, accum, subframe=3, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    st = wf.stats()
    want = oracle.render(sp, cam, W, H, spp, subframe=3, max_depth=depth, mode=pyoracle.MODE_GB300)
    assert np.array_equal(accum.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
    assert st["segments"] == want["segments"]
    assert st["nodes_visited"] == want["nodes"] and st["spheres_tested"] == want["spheres"]


def _render_gpu(venu, cuda, sp, cam, W, H, spp, subframe, depth, max_paths=0, accum=None, reset=True):
    torch = cuda
    ds = _dev_scene(venu, sp)
    wf = venu.Wavefront(max_paths)
    if accum is None:
        accum = venu.new_accum(W, H)
    img_f = torch.zeros((H * W, 4), dtype=torch.float32, device="cuda")
    img8 = torch.zeros((H * W, 4), dtype=torch.uint8, device="cuda")
    wf.render(ds, cam, W, H, spp, accum, subframe=subframe, max_depth=depth, reset=reset, image_f=img_f,
              image8=img8)
    torch.cuda.synchronize()
    st = wf.stats()
    return accum.cpu().numpy(), img_f.cpu().numpy(), img8.cpu().numpy(), st


@pytest.mark.parametrize("depth", [1, 4, 50])
def test_render_bit_exact(venu, oracle, cuda, depth):
    sp = oracle.scene_rtiow(0)
    W, H, spp = 48, 27, 4
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    acc, img_f, img8, st = _render_gpu(venu, cuda, sp, cam, W, H, spp, 1, depth)
    want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))
    assert np.array_equal(img_f.view(np.uint32), want["image_f"].view(np.uint32))
    assert np.array_equal(img8, want["image8"])
    assert st["segments"] == want["segments"]
    assert st["paths"] == W * H * spp


def test_render_golden(venu, cuda):
    g = np.load(GOLDEN)
    sp = g["scene"].reshape(-1).view(pyoracle.SPHERE_DTYPE)
    cam = g["camera"].view(pyoracle.CAMERA_DTYPE)
    W, H, spp = (int(x) for x in g["wh_spp"])
    for depth in (4, 50):
        acc, _, _, st = _render_gpu(venu, cuda, sp, cam, W, H, spp, 1, depth)
        assert np.array_equal(acc.view(np.uint32), g[f"gb_d{depth}_accum"].view(np.uint32))
        assert st["segments"] == int(g[f"gb_d{depth}_segments"][0])


@pytest.mark.parametrize("max_paths", [997, 3 * 40 * 30, 40 * 30 * 7 + 5])
def test_render_wave_shapes(venu, oracle, cuda, max_paths):
    """Waves of P < npix pixels, of k < spp samples, and a single wave all
    give the same bits (per-pixel sample order is preserved)."""
    sp = oracle.scene_rtiow(2)
    W, H, spp = 40, 30, 7
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    acc, _, _, st = _render_gpu(venu, cuda, sp, cam, W, H, spp, 3, 8, max_paths=max_paths)
    want = oracle.render(sp, cam, W, H, spp, subframe=3, max_depth=8, mode=pyoracle.MODE_GB300)
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))
    assert st["segments"] == want["segments"]


def test_progressive_accumulation(venu, oracle, cuda):
    """Renderer::Draw twice (subframes 1 and 2) == the oracle accumulating the
    same subframes into one Kahan buffer."""
    sp = oracle.scene_rtiow(0)
    W, H = 32, 20
    cam_np = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    scene = venu.Scene(spheres=sp)
    r = venu.Renderer(samples_per_pixel=3, max_depth=6)
    r.Init(scene)
    cam = venu.Camera((13, 2, 3), 20.0, W / H, 0.1, 10.0)
    cam.SetForward(np.float32([0, 0, 0]) - np.float32([13, 2, 3]))
    assert cam.params().tobytes() == cam_np.tobytes()
    out = venu.CUDAOutputBuffer(W, H)
    r.Draw(cam, out)
    r.Draw(cam, out)
    acc = r.accum.cpu().numpy()
    want = oracle.render(sp, cam_np, W, H, 3, subframe=1, max_depth=6, mode=pyoracle.MODE_GB300)
    want = oracle.render(sp, cam_np, W, H, 3, subframe=2, max_depth=6, mode=pyoracle.MODE_GB300,
                         accum=want["accum"])
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))
    assert np.array_equal(out.getHostFloat().reshape(-1, 4).view(np.uint32), want["image_f"].view(np.uint32))
    # camera change resets the accumulation (Core/Renderer.h:37-45)
    cam.MoveForward(0.1)
    r.Draw(cam, out)
    assert float(r.accum[:, 3].max()) == 3.0
    r.Cleanup()


def test_render_random_scene(venu, oracle, cuda):
    sp = oracle.scene_random(20_000, 12)
    W, H, spp = 64, 36, 2
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    acc, _, _, st = _render_gpu(venu, cuda, sp, cam, W, H, spp, 0, 50)
    want = oracle.render(sp, cam, W, H, spp, subframe=0, max_depth=50, mode=pyoracle.MODE_GB300)
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))
    assert st["segments"] == want["segments"]


def test_empty_and_tiny_scenes(venu, oracle, cuda):
    W, H = 16, 9
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    for n in (0, 1, 2):
        sp = oracle.scene_rtiow(0)[:n]
        acc, _, _, st = _render_gpu(venu, cuda, sp, cam, W, H, 2, 0, 10)
        want = oracle.render(sp, cam, W, H, 2, subframe=0, max_depth=10, mode=pyoracle.MODE_GB300)
        assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))


@pytest.mark.parametrize("tuning", [
    dict(traverse_variant=0, refill_min=32, traverse_block=64, shade_block=128),
    dict(traverse_variant=1, refill_min=1, traverse_block=256, shade_block=64),
    dict(traverse_variant=1, refill_min=16, traverse_block=128, shade_block=512, traverse_blocks_per_sm=2),
    dict(traverse_variant=2, refill_min=8, traverse_block=128, shade_block=256),
    dict(traverse_variant=2, refill_min=8, traverse_block=256, shade_block=256, traverse_blocks_per_sm=1),
    dict(traverse_variant=3, refill_min=8, traverse_block=128, shade_block=256),
    dict(traverse_variant=3, refill_min=32, traverse_block=256, shade_block=128, traverse_blocks_per_sm=2),
    dict(traverse_variant=4, refill_min=32, traverse_block=128, shade_block=256),
    dict(traverse_variant=4, refill_min=32, traverse_block=64, shade_block=256, traverse_blocks_per_sm=3),
    dict(traverse_variant=5, refill_min=8, traverse_block=128, shade_block=256),
    dict(traverse_variant=5, refill_min=1, traverse_block=256, shade_block=128, traverse_blocks_per_sm=2),
    dict(traverse_variant=2, refill_min=32, traverse_block=128, shade_block=256, in_place_factor=8),
    dict(traverse_variant=4, refill_min=32, traverse_block=64, shade_block=256, in_place_factor=16),
])
def test_render_tunings_bit_exact(venu, oracle, cuda, tuning):
    """Launch shapes and traversal variants change speed, never bits."""
    torch = cuda
    sp = oracle.scene_rtiow(0)
    W, H, spp, depth = 40, 24, 3, 12
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    wf = venu.Wavefront(1500)
    wf.set_tuning(**tuning)
    assert {k: wf.tuning()[k] for k in tuning} == tuning
    accum = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, accum, subframe=2, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    want = oracle.render(sp, cam, W, H, spp, subframe=2, max_depth=depth, mode=pyoracle.MODE_GB300)
    assert np.array_equal(accum.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
    assert wf.stats()["segments"] == want["segments"]


def test_tuning_rejects_bad_values(venu, cuda):
    wf = venu.Wavefront(1000)
    with pytest.raises(venu.VenuError):
        wf.set_tuning(traverse_block=96)
    with pytest.raises(venu.VenuError):
        wf.set_tuning(refill_min=0)


def _edge_scene(oracle, case):
    sp = oracle.scene_rtiow(0).copy()
    if case == "hollow_glass":  # RTIOW's hollow bubble: a negative radius inside the glass sphere
        inner = sp[1:2].copy()
        inner["radius"] = -0.9
        sp = np.concatenate([sp, inner])
    elif case == "zero_radius":
        sp["radius"][10:40] = 0.0
    elif case == "duplicates":  # exact copies: equal hits resolved by the smaller slot
        sp = np.concatenate([sp, sp[4:60]])
    elif case == "many_huge":  # more huge spheres than are hoisted
        big = sp[:9].copy()
        big["center"][:, 0] = np.arange(9) * 3000.0 - 12000.0
        big["center"][:, 1] = -1000.0
        big["radius"] = 1000.0
        sp = np.concatenate([sp, big])
    elif case == "too_many_huge":  # more than 64 huge spheres: none hoisted
        big = np.repeat(sp[:1], 70)
        big["center"][:, 0] = np.arange(70) * 2500.0 - 80000.0
        sp = np.concatenate([sp, big])
    return sp


@pytest.mark.parametrize("case", ["hollow_glass", "zero_radius", "duplicates", "many_huge", "too_many_huge"])
def test_edge_scenes_bit_exact(venu, oracle, cuda, case):
    sp = _edge_scene(oracle, case)
    ds = _dev_scene(venu, sp)
    got, want = ds.export_bvh(), oracle.lbvh(sp)
    assert np.array_equal(got["ids"], want["ids"]) and got["nodes"].tobytes() == want["nodes"].tobytes()
    W, H, spp = 40, 24, 3
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    acc, _, _, st = _render_gpu(venu, cuda, sp, cam, W, H, spp, 1, 12)
    ref = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=12, mode=pyoracle.MODE_GB300)
    assert np.array_equal(acc.view(np.uint32), ref["accum"].view(np.uint32))
    assert st["segments"] == ref["segments"]


def _nested_scene(oracle, n, levels, rfrac, seed=5):
    """Spheres in nested cubes of half-size 50 * 2^-k (k = i mod levels),
    radius rfrac times that: overlapping boxes at every scale, so rays toward
    the centre push far children at many levels of the tree."""
    rng = np.random.default_rng(seed)
    sp = oracle.scene_random(n, 9)
    s = 50.0 * 2.0 ** (-(np.arange(n) % levels))
    sp["center"] = ((rng.random((n, 3)) * 2 - 1) * s[:, None]).astype(np.float32)
    sp["radius"] = (rfrac * s).astype(np.float32)
    return sp


# (spheres, levels, radius fraction, the stack entries the renderer keeps in
# shared memory for that scene size: 4 up to 4096 spheres, else 8)
DEEP = [(4000, 12, 0.5, 4), (6000, 10, 0.7, 8)]


@pytest.mark.parametrize("n,levels,rfrac,ks", DEEP)
@pytest.mark.parametrize("variant", [2, 3, 4, 5])
def test_deep_stack_spills_bit_exact(venu, oracle, cuda, n, levels, rfrac, ks, variant):
    """Scenes whose rays need more stack entries than the shared-memory ring
    holds: the spill to local memory and back keeps every result bit-exact,
    and no stack error is reported (stats() raises on one)."""
    sp = _nested_scene(oracle, n, levels, rfrac)
    rng = np.random.default_rng(1)
    eye = (150.0, 30.0, 150.0)  # outside every sphere
    o = np.tile(np.array(eye, np.float32), (4000, 1))
    tgt = (rng.random((4000, 3)) * 2 - 1) * rng.choice([0.01, 0.1, 1, 10, 30], size=(4000, 1))
    depth = oracle.trace_stack_depth(sp, np.concatenate([o, tgt - o], 1))
    assert depth.max() > ks  # the case reaches the spill path
    W, H, spp = 48, 27, 2
    cam = oracle.camera(eye, (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    torch = cuda
    ds = _dev_scene(venu, sp)
    wf = venu.Wavefront(0)
    wf.set_tuning(traverse_variant=variant, refill_min=8, traverse_block=128, shade_block=256)
    acc = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, acc, subframe=1, max_depth=6, reset=True)
    torch.cuda.synchronize()
    st = wf.stats()
    want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=6, mode=pyoracle.MODE_GB300)
    assert np.array_equal(acc.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
    assert st["segments"] == want["segments"]


@pytest.mark.parametrize("scene", ["rtiow", "random"])
def test_in_place_refill_bit_exact(venu, oracle, cuda, scene):
    """Launches with more rays than the grid has threads finished in place
    (in_place_factor 8: blocks take rays with an atomic, compact their
    survivors and refill finished threads between bounces) give the same
    accumulator and segment count as the oracle."""
    torch = cuda
    if scene == "rtiow":
        sp, eye = oracle.scene_rtiow(0), (13, 2, 3)
    else:
        sp, eye = oracle.scene_random(20_000, 3), (60, 15, 60)
    W, H, spp, depth = 400, 225, 4, 12  # 360 k paths: more than the grid's threads, fewer than 8x
    cam = oracle.camera(eye, (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
    for variant in (2, 4):
        wf = venu.Wavefront(0)
        wf.set_tuning(traverse_variant=variant, traverse_block=128, in_place_factor=8)
        acc = venu.new_accum(W, H)
        wf.render(ds, cam, W, H, spp, acc, subframe=1, max_depth=depth, reset=True)
        torch.cuda.synchronize()
        assert np.array_equal(acc.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
        assert wf.stats()["segments"] == want["segments"]


@pytest.mark.parametrize("variant,factor", [(2, 1), (4, 1), (2, 8)])
def test_wave_graph_matches_host_loop(venu, oracle, cuda, variant, factor):
    """The fused variants run each wave's bounce loop as one CUDA graph whose
    while node stops when a bounce leaves no rays; the profiling build
    launches every bounce from the host.  Both give the oracle's accumulator
    and segment count, and the graph runs only the bounces that have rays
    (at most one empty launch per wave) where the host launches all of
    max_depth.  Waves of part of the pixels keep the host loop."""
    torch = cuda
    sp = oracle.scene_rtiow(0)
    # (W, H, spp, depth, max_paths, launches with the graph against the host loop)
    cases = [(200, 120, 2, 50, 10_000, "=="),   # waves of 10 k of the 24 k pixels, one sample: host loop
             (64, 36, 2, 50, 0, "=="),           # 4.6 k paths, all finished in place by the first bounce
             (1280, 720, 4, 50, 0, "<"),         # one wave of 3.7 M paths: more than 8 per thread of any grid
             (320, 180, 6, 50, 120_000, "<=")]   # three waves of all pixels x 2 samples
    for W, H, spp, depth, max_paths, rel in cases:
        cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
        want = oracle.render(sp, cam, W, H, spp, subframe=2, max_depth=depth, mode=pyoracle.MODE_GB300)
        ds = venu.DeviceScene(sp)
        got = {}
        for profile in (False, True):
            wf = venu.Wavefront(max_paths, profile=profile)
            wf.set_tuning(traverse_variant=variant, traverse_block=128, in_place_factor=factor)
            acc = venu.new_accum(W, H)
            for _ in range(2):  # the second render reuses the graph
                wf.render(ds, cam, W, H, spp, acc, subframe=2, max_depth=depth, reset=True)
            torch.cuda.synchronize()
            st = wf.stats()
            assert np.array_equal(acc.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
            assert st["segments"] == want["segments"]
            got[profile] = st["kernel_launches"]
        # a wave the first bounce finishes in place stops after it either way
        ok = {"<": got[False] < got[True], "<=": got[False] <= got[True], "==": got[False] == got[True]}[rel]
        assert ok, (W, H, spp, got)
