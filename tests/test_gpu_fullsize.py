"""Parity at the benchmark's full sizes.  The oracle cannot render these
frames whole in seconds, so each is checked through properties of the whole
frame (every pixel has all its samples, values finite and non-negative, the
path count exact, the batch engine's accumulator identical bit for bit) and
bit-exactly against the oracle on sampled rows; the 1M-sphere LBVH is
compared whole."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _frame_properties(acc, W, H, spp, st):
    a = acc.cpu().numpy()
    assert (a[:, 3] == spp).all()  # every pixel received all its samples
    assert np.isfinite(a).all() and (a[:, :3] >= 0).all()
    assert st["paths"] == W * H * spp and st["segments"] >= st["paths"]
    return a


def _rows_match(oracle, a, sp, cam, W, H, spp, depth, rows):
    for r0 in rows:
        want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300,
                             rows=(r0, r0 + 1))
        got, ref = a[r0 * W:(r0 + 1) * W], want["accum"][r0 * W:(r0 + 1) * W]
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), f"row {r0}"


def test_rtiow_1920x1080_256spp(venu, oracle, cuda):
    torch = cuda
    W, H, spp, depth = 1920, 1080, 256, 50
    sp = oracle.scene_rtiow(0)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    wf = venu.Wavefront(0)
    acc = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, acc, subframe=1, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    a = _frame_properties(acc, W, H, spp, wf.stats())
    _rows_match(oracle, a, sp, cam, W, H, spp, depth, (0, 540, 1079))
    b = venu.Batch(pool_paths=16 << 20, max_jobs=1)
    acc2 = venu.new_accum(W, H)
    b.submit(ds, cam, W, H, spp, acc2, subframe=1, max_depth=depth)
    b.run()
    assert len(b.collect()) == 1
    torch.cuda.synchronize()
    assert torch.equal(acc, acc2)
    b.close()
    # the whole frame as one wave (the benchmark's shape, ~64 GB of queues)
    # against the default waves of 64 Mi paths: the same samples in the same
    # order, so the same bits
    wf.close()
    one = venu.Wavefront(W * H * spp)
    one.render(ds, cam, W, H, spp, acc2, subframe=1, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    st = one.stats()
    one.close()
    assert st["waves"] == 1 and st["paths"] == W * H * spp
    assert torch.equal(acc, acc2)


def test_renderer_wave_cap(venu, cuda):
    """max_paths up to 2^30 (queues are allocated by the first render, so
    creating the renderer costs nothing); above it, a clear error."""
    venu.Wavefront(1 << 30).close()
    with pytest.raises(venu.VenuError, match="2\\^30"):
        venu.Wavefront((1 << 30) + 1)


def test_random_1m_spheres_1080p_64spp(venu, oracle, cuda):
    torch = cuda
    W, H, spp, depth = 1920, 1080, 64, 50
    sp = oracle.scene_random(1_000_000, 42)
    ds = venu.DeviceScene(sp)
    got = ds.export_bvh()
    want = oracle.lbvh(sp)
    assert np.array_equal(got["keys"], want["keys"]) and np.array_equal(got["ids"], want["ids"])
    assert got["nodes"].tobytes() == want["nodes"].tobytes()
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    wf = venu.Wavefront(0)
    acc = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, acc, subframe=1, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    a = _frame_properties(acc, W, H, spp, wf.stats())
    _rows_match(oracle, a, sp, cam, W, H, spp, depth, (540,))


def test_mixed_64_scenes_batched_equals_plain(venu, cuda):
    """The 64-scene mixed workload: every job's accumulator from the shared
    pool equals its plain render bit for bit."""
    torch = cuda
    from venusaur_gb300 import workloads

    jobs = workloads.mixed_jobs(64)
    scenes = {}
    b = venu.Batch(pool_paths=16 << 20, max_jobs=64)
    wf = venu.Wavefront(16 << 20)
    plain, batch = [], []
    for j in jobs:
        key = (j["n"], j["scene_seed"])
        if key not in scenes:
            scenes[key] = venu.DeviceScene(venu.generate_random(j["n"], j["scene_seed"]))
        cam = venu.Camera.look_at(j["eye"], (0, 0, 0), 20.0, j["W"] / j["H"], 0.1, 10.0)
        a1, a2 = venu.new_accum(j["W"], j["H"]), venu.new_accum(j["W"], j["H"])
        wf.render(scenes[key], cam, j["W"], j["H"], j["spp"], a1, subframe=j["subframe"], max_depth=j["depth"])
        b.submit(scenes[key], cam, j["W"], j["H"], j["spp"], a2, subframe=j["subframe"], max_depth=j["depth"])
        plain.append(a1)
        batch.append(a2)
    b.run()
    assert len(b.collect()) == len(jobs)
    torch.cuda.synchronize()
    for i, (a1, a2) in enumerate(zip(plain, batch)):
        assert torch.equal(a1, a2), f"job {i}"
        assert int(a1[:, 3].min().item()) == jobs[i]["spp"]
