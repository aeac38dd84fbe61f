"""GPU tests of moving spheres (venu_scene_update): the LBVH is refit in
place -- topology, slot order and hoisted set kept, boxes recomputed -- and
must equal the oracle's refit bit for bit; renders through the refit tree
must equal the oracle's renders (and those of a fresh build)."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _moved(spheres, seed, scale=1.0, radius=True, material=False):
    rng = np.random.default_rng(seed)
    out = spheres.copy()
    for a in range(3):
        out["center"][1:, a] += (rng.normal(size=len(out) - 1) * scale).astype(np.float32)
    if radius:
        out["radius"][1:] *= rng.uniform(0.5, 1.5, size=len(out) - 1).astype(np.float32)
    if material:
        out["material"][1:] = rng.integers(0, 3, size=len(out) - 1).astype(np.uint32)
    return out


def _render(venu, torch, ds, cam, W, H, spp, subframe, depth, variant=None):
    wf = venu.Wavefront(0, count=True)
    if variant is not None:
        wf.set_tuning(traverse_variant=variant)
    acc = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, acc, subframe=subframe, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    return acc.cpu().numpy(), wf.stats()


@pytest.mark.parametrize("case", ["rtiow", "rand20k"])
def test_refit_nodes_and_render(venu, oracle, cuda, case):
    torch = cuda
    if case == "rtiow":
        sp = oracle.scene_rtiow(0)
        mv = _moved(sp, 1, scale=0.3, material=True)
        eye = (13, 2, 3)
    else:
        sp = oracle.scene_random(20_000, 4)
        mv = _moved(sp, 2, scale=2.0)
        eye = (60, 15, 60)
    ds = venu.DeviceScene(sp)
    W, H, spp, depth = 40, 24, 3, 20
    cam = oracle.camera(eye, (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    info0 = ds.info()
    assert info0["num_wide_nodes"] == 0  # the 4-wide tree is built on first use by variant 4 or 5
    if case == "rtiow":
        # the update below then refits an existing 4-wide tree; rand20k builds
        # its 4-wide tree only after the update, from the refit binary tree
        _render(venu, torch, ds, cam, W, H, 1, 1, depth, variant=4)
        info1 = ds.info()
        assert info1["num_wide_nodes"] > 0 and info1["device_bytes"] > info0["device_bytes"]
    before = ds.export_bvh()
    ds.update(mv)
    got = ds.export_bvh()
    assert np.array_equal(got["ids"], before["ids"]) and np.array_equal(got["keys"], before["keys"])
    want_nodes = oracle.lbvh_refit(sp, mv)
    assert np.array_equal(got["nodes"].view(np.uint32), want_nodes.view(np.uint32))
    acc, st = _render(venu, torch, ds, cam, W, H, spp, 2, depth)
    want = oracle.render(mv, cam, W, H, spp, subframe=2, max_depth=depth, built_from=sp)
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))
    assert st["segments"] == want["segments"]
    assert st["nodes_visited"] == want["nodes"] and st["spheres_tested"] == want["spheres"]
    fresh = oracle.render(mv, cam, W, H, spp, subframe=2, max_depth=depth)
    assert np.array_equal(acc.view(np.uint32), fresh["accum"].view(np.uint32))
    # the 4-wide tree: refit with the binary one (rtiow) or built from it (rand20k)
    assert (ds.info()["num_wide_nodes"] > 0) == (case == "rtiow")
    acc4, st4 = _render(venu, torch, ds, cam, W, H, spp, 2, depth, variant=4)
    assert np.array_equal(acc4.view(np.uint32), want["accum"].view(np.uint32))
    assert st4["segments"] == want["segments"]
    assert ds.info()["num_wide_nodes"] > 0


def test_refit_round_trip_and_limits(venu, oracle, cuda):
    sp = oracle.scene_random(5000, 8)
    ds = venu.DeviceScene(sp)
    built = ds.export_bvh()["nodes"]
    for k in range(3):
        ds.update(_moved(sp, 10 + k, scale=4.0))
    ds.update(sp)  # back where it was built: the build's boxes again
    assert np.array_equal(ds.export_bvh()["nodes"].view(np.uint32), built.view(np.uint32))
    with pytest.raises(venu.VenuError):
        ds.update(sp[:-1])  # a different count needs a new scene
    tiny = venu.DeviceScene(sp[:1])
    tiny.update(_moved(sp[:2], 3)[:1])
    empty = venu.DeviceScene(sp[:0])
    empty.update(sp[:0])


def test_update_device_and_renderer_update(venu, oracle, cuda):
    torch = cuda
    sp = oracle.scene_rtiow(0)
    mv = _moved(sp, 6, scale=0.2)
    W, H = 32, 18
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    dev = torch.from_numpy(mv.view(np.uint8).copy()).cuda()
    ds.update_device(dev, len(mv))
    acc, _ = _render(venu, torch, ds, cam, W, H, 2, 1, 10)
    want = oracle.render(mv, cam, W, H, 2, subframe=1, max_depth=10, built_from=sp)
    assert np.array_equal(acc.view(np.uint32), want["accum"].view(np.uint32))

    # Renderer.Update restarts the progressive accumulation
    scene = venu.Scene()
    cam2 = venu.Camera((13.0, 2.0, 3.0), 20.0, W / H, 0.1, 10.0)
    cam2.SetForward((-13.0, -2.0, -3.0))
    r = venu.Renderer(samples_per_pixel=2, max_depth=6)
    r.Init(scene)
    out = venu.CUDAOutputBuffer(W, H)
    r.Draw(cam2, out)
    r.Draw(cam2, out)
    moved = _moved(scene.spheres, 7, scale=0.2)
    scene.spheres = moved
    r.Update(scene)
    r.Draw(cam2, out)
    assert r.subframe_index == 1
    want = oracle.render(moved, cam2.params(), W, H, 2, subframe=1, max_depth=6, built_from=oracle.scene_rtiow(0))
    assert np.array_equal(r.accum.cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
    r.Cleanup()
