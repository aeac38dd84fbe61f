"""GPU tests of the render server (continuous batching under an HBM budget).
Failures are made on the host (injected allocation / build failures, a
cancelled request, a request larger than the budget); the GPU never faults."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _case(oracle, seed, W, H, spp, depth=6):
    sp = oracle.scene_rtiow(seed)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
    return sp, cam, want


def test_server_results_match_oracle(venu, oracle, cuda):
    srv = venu.Server(hbm_budget_bytes=1 << 30, pool_paths=2000, max_jobs=8, iterations_per_step=4)
    cases = [_case(oracle, s, W, H, spp) for s, W, H, spp in ((0, 32, 18, 2), (1, 20, 20, 3), (2, 16, 9, 1))]
    ids = []
    for i, (sp, cam, _) in enumerate(cases):
        ids.append(srv.submit(cam, *((32, 18, 2), (20, 20, 3), (16, 9, 1))[i], spheres=sp, max_depth=6, tag=i))
    # same scene key twice: the second request reuses the resident BVH
    sp0, cam0, want0 = cases[0]
    k1 = srv.submit(cam0, 32, 18, 2, spheres=sp0, scene_key=77, max_depth=6)
    k2 = srv.submit(cam0, 32, 18, 2, spheres=None, scene_key=77, max_depth=6)
    for i, rid in enumerate(ids):
        r = srv.wait(rid)
        assert r["status"] == 0 and r["tag"] == i
        want = cases[i][2]["image8"].reshape(r["image"].shape)
        assert np.array_equal(r["image"], want)
    for rid in (k1, k2):
        r = srv.wait(rid, timeout_s=float("inf"))  # no limit: clamped to 1e9 s, not an overflow
        assert r["status"] == 0
        assert np.array_equal(r["image"], want0["image8"].reshape(r["image"].shape))
    st = srv.stats()
    assert st["completed"] == 5 and st["failed"] == 0 and st["p99_ms"] >= st["p50_ms"] > 0
    srv.close()


def test_server_budget_fifo_and_faults(venu, oracle, cuda):
    sp, cam, want = _case(oracle, 0, 24, 16, 2)
    # the server's admission estimate: job, image and accumulator, and the
    # scene at 240 bytes per sphere + 4096 (binary and 8-wide trees)
    job = venu.Batch.job_bytes(24, 16, 2) + 24 * 16 * 36 + 485 * 240 + 4096
    # room for about one job at a time: requests queue and run in order
    srv = venu.Server(hbm_budget_bytes=job + 40000, pool_paths=1000, max_jobs=4, iterations_per_step=2)
    too_big = srv.submit(cam, 2000, 2000, 64, spheres=sp)
    assert srv.wait(too_big)["status"] == 3  # VENU_ERR_OOM: can never fit the budget
    ra = srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6))
    assert ra["status"] == 0
    assert np.array_equal(ra["image"], want["image8"].reshape(ra["image"].shape))
    # injected allocation failure: that request fails, the next one runs
    srv.inject(venu._lib.INJECT_ALLOC)
    assert srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6))["status"] == 3
    # FIFO under the budget: c is admitted before d; d can be cancelled while it waits
    c = srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6)
    d = srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6)
    try:
        srv.cancel(d)
        cancelled = True
    except venu.VenuError:
        cancelled = False  # already admitted
    rc, rd = srv.wait(c), srv.wait(d)
    assert rc["status"] == 0
    if cancelled:
        assert rd["status"] == 7  # VENU_ERR_CANCELLED
    else:
        assert rd["status"] == 0 and rd["t_admit"] >= rc["t_admit"]
    # injected BVH build failure
    srv.inject(venu._lib.INJECT_SCENE)
    assert srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6))["status"] == 2
    assert srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp, max_depth=6))["status"] == 0
    st = srv.stats()
    assert st["failed"] == 3 + (1 if cancelled else 0)
    srv.close()


def test_server_rejects_malformed(venu, oracle, cuda):
    srv = venu.Server(hbm_budget_bytes=1 << 28, max_jobs=2)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, 1.0, 0.1, 10.0)
    with pytest.raises(venu.VenuError):
        srv.submit(cam, 1, 1, 1, spheres=oracle.scene_rtiow(0))
    with pytest.raises(venu.VenuError):
        srv.submit(cam, 8, 8, 1, spheres=oracle.scene_rtiow(0), max_depth=0)
    srv.close()


def test_server_shortest_first(venu, oracle, cuda):
    """Shortest-first plan order: same images, every request completes."""
    srv = venu.Server(hbm_budget_bytes=1 << 30, pool_paths=1500, max_jobs=8, iterations_per_step=64,
                      shortest_first=True)
    big = _case(oracle, 0, 48, 32, 8)
    small = _case(oracle, 1, 12, 8, 1)
    rb = srv.submit(big[1], 48, 32, 8, spheres=big[0], max_depth=6)
    rs = srv.submit(small[1], 12, 8, 1, spheres=small[0], max_depth=6)
    for rid, (_, _, want) in ((rb, big), (rs, small)):
        r = srv.wait(rid)
        assert r["status"] == 0
        assert np.array_equal(r["image"], want["image8"].reshape(r["image"].shape))
    srv.set_policy(False)
    r = srv.wait(srv.submit(small[1], 12, 8, 1, spheres=small[0], max_depth=6))
    assert r["status"] == 0
    srv.close()


def test_server_express_lane(venu, oracle, cuda):
    """Requests at or below the express threshold run in the second pool;
    every image is the same as the oracle's whichever lane rendered it."""
    srv = venu.Server(hbm_budget_bytes=1 << 30, pool_paths=3000, max_jobs=8, iterations_per_step=64,
                      express_paths=12 * 8 * 2)
    cases = [(_case(oracle, 0, 48, 32, 6), (48, 32, 6)), (_case(oracle, 1, 12, 8, 2), (12, 8, 2)),
             (_case(oracle, 2, 40, 24, 4), (40, 24, 4)), (_case(oracle, 3, 12, 8, 1), (12, 8, 1))]
    ids = [srv.submit(c[1], *wh, spheres=c[0], max_depth=6) for c, wh in cases]
    for rid, (c, _) in zip(ids, cases):
        r = srv.wait(rid)
        assert r["status"] == 0
        assert np.array_equal(r["image"], c[2]["image8"].reshape(r["image"].shape))
    st = srv.stats()
    assert st["completed"] == 4 and st["failed"] == 0
    assert st["segments"] == sum(c[2]["segments"] for c, _ in cases)
    srv.close()


def test_server_progressive_session(venu, oracle, cuda):
    """Requests of one session add to its resident accumulator (the running
    mean of Renderer::Draw); a reset or a new size restarts it; end_session
    frees it.  Images equal the oracle's progressive accumulation."""
    srv = venu.Server(hbm_budget_bytes=1 << 30, pool_paths=2000, max_jobs=8, iterations_per_step=8,
                      express_paths=1000)
    sp = oracle.scene_rtiow(0)
    W, H, spp, depth = 24, 16, 2, 6
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    acc = None
    ids = []
    for sub in (1, 2, 3):
        ids.append(srv.submit(cam, W, H, spp, spheres=sp, scene_key=5, max_depth=depth, subframe=sub, session=42))
    for sub, rid in zip((1, 2, 3), ids):
        want = oracle.render(sp, cam, W, H, spp, subframe=sub, max_depth=depth, mode=pyoracle.MODE_GB300, accum=acc)
        acc = want["accum"]
        r = srv.wait(rid)
        assert r["status"] == 0
        assert np.array_equal(r["image"], want["image8"].reshape(r["image"].shape))
    # an explicit reset restarts the session at subframe 7
    r = srv.wait(srv.submit(cam, W, H, spp, scene_key=5, max_depth=depth, subframe=7, session=42, reset=True))
    want = oracle.render(sp, cam, W, H, spp, subframe=7, max_depth=depth, mode=pyoracle.MODE_GB300)
    assert np.array_equal(r["image"], want["image8"].reshape(r["image"].shape))
    # ending the session: the next request of that id starts from zero
    srv.end_session(42)
    r = srv.wait(srv.submit(cam, W, H, spp, scene_key=5, max_depth=depth, subframe=2, session=42))
    want = oracle.render(sp, cam, W, H, spp, subframe=2, max_depth=depth, mode=pyoracle.MODE_GB300)
    assert np.array_equal(r["image"], want["image8"].reshape(r["image"].shape))
    assert srv.stats()["failed"] == 0
    srv.close()


def test_server_lru_eviction_counted(venu, oracle, cuda):
    """A budget with room for one resident scene and one small job: a second
    keyed scene evicts the first (least recently used, unreferenced), the
    first's key is then no longer resident (a request relying on it fails
    with VENU_ERR_INVALID and succeeds when the spheres are sent again), and
    the server counts the evictions and the peak of resident bytes."""
    sp0, cam, want0 = _case(oracle, 0, 24, 16, 2)
    sp1, _, want1 = _case(oracle, 1, 24, 16, 2)
    job = venu.Batch.job_bytes(24, 16, 2) + 24 * 16 * 36
    scene = 488 * 240 + 4096  # the server's estimate of an RTIOW scene, above its built size
    srv = venu.Server(hbm_budget_bytes=job + scene + 1024, pool_paths=1000, max_jobs=4, iterations_per_step=2)
    r = srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp0, scene_key=1, max_depth=6))
    assert r["status"] == 0 and np.array_equal(r["image"], want0["image8"].reshape(r["image"].shape))
    r = srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp1, scene_key=2, max_depth=6))
    assert r["status"] == 0 and np.array_equal(r["image"], want1["image8"].reshape(r["image"].shape))
    st = srv.stats()
    assert st["evictions"] >= 1
    assert 0 < st["peak_resident_bytes"] <= st["budget_bytes"]
    r = srv.wait(srv.submit(cam, 24, 16, 2, spheres=None, scene_key=1, max_depth=6))
    assert r["status"] == 1  # VENU_ERR_INVALID: key 1 was evicted
    r = srv.wait(srv.submit(cam, 24, 16, 2, spheres=sp0, scene_key=1, max_depth=6))
    assert r["status"] == 0 and np.array_equal(r["image"], want0["image8"].reshape(r["image"].shape))
    assert srv.stats()["evictions"] >= 2
    srv.close()
