"""GPU tests of the batched/served engine (venu_batch_*): jobs of different
scenes, sizes, sample counts and depths share one path pool; each job's
accumulator must equal the oracle's (and venu_render's) bit for bit, whether
it ran alone or in the mix, in one graph launch or in chunks."""
import numpy as np
import pytest

from oracle import pyoracle

pytestmark = pytest.mark.gpu


def _jobs(oracle):
    return [
        dict(scene=oracle.scene_rtiow(0), eye=(13, 2, 3), W=40, H=24, spp=3, depth=8, sub=1),
        dict(scene=oracle.scene_random(3000, 5), eye=(60, 15, 60), W=33, H=17, spp=5, depth=50, sub=2),
        dict(scene=oracle.scene_rtiow(3), eye=(13, 2, 3), W=16, H=9, spp=1, depth=4, sub=7),
        dict(scene=oracle.scene_rtiow(0)[:2], eye=(13, 2, 3), W=8, H=6, spp=4, depth=3, sub=1),
    ]


def _want(oracle, j):
    cam = oracle.camera(j["eye"], (0, 0, 0), 20.0, j["W"] / j["H"], 0.1, 10.0)
    r = oracle.render(j["scene"], cam, j["W"], j["H"], j["spp"], subframe=j["sub"], max_depth=j["depth"],
                      mode=pyoracle.MODE_GB300)
    return cam, r


def _submit_all(venu, torch, batch, oracle, jobs):
    out = []
    for j in jobs:
        cam, want = _want(oracle, j)
        ds = venu.DeviceScene(j["scene"])
        acc = venu.new_accum(j["W"], j["H"])
        img = torch.zeros((j["W"] * j["H"], 4), dtype=torch.float32, device="cuda")
        jid = batch.submit(ds, cam, j["W"], j["H"], j["spp"], acc, subframe=j["sub"], max_depth=j["depth"],
                           image_f=img)
        out.append(dict(id=jid, ds=ds, acc=acc, img=img, want=want))
    return out


@pytest.mark.parametrize("pool,graph", [(0, True), (700, True), (700, False)])
def test_batch_matches_oracle(venu, oracle, cuda, pool, graph):
    torch = cuda
    b = venu.Batch(pool_paths=pool, max_jobs=8, graph=graph)
    sub = _submit_all(venu, torch, b, oracle, _jobs(oracle))
    b.run()
    done = b.collect()
    torch.cuda.synchronize()
    assert sorted(done) == sorted(s["id"] for s in sub)
    total_segments = 0
    for s in sub:
        assert np.array_equal(s["acc"].cpu().numpy().view(np.uint32), s["want"]["accum"].view(np.uint32))
        assert np.array_equal(s["img"].cpu().numpy().view(np.uint32), s["want"]["image_f"].view(np.uint32))
        total_segments += s["want"]["segments"]
    st = b.stats()
    assert st["segments"] == total_segments
    assert st["active_jobs"] == 0 and st["resident_bytes"] == 0
    if graph:
        assert st["graph_launches"] == 1


def test_batch_chunked_runs_and_late_admission(venu, oracle, cuda):
    """Continuous batching: jobs arrive while others are in flight; runs of a
    few iterations interleave with admission and collection."""
    torch = cuda
    b = venu.Batch(pool_paths=500, max_jobs=8)
    jobs = _jobs(oracle)
    first = _submit_all(venu, torch, b, oracle, jobs[:2])
    b.run(max_iterations=2)
    finished = b.collect()
    late = _submit_all(venu, torch, b, oracle, jobs[2:])
    allsub = first + late
    for _ in range(500):
        b.run(max_iterations=4)
        finished += b.collect()
        if len(finished) == len(allsub):
            break
    torch.cuda.synchronize()
    assert sorted(finished) == sorted(s["id"] for s in allsub)
    for s in allsub:
        assert np.array_equal(s["acc"].cpu().numpy().view(np.uint32), s["want"]["accum"].view(np.uint32))


def test_batch_equals_plain_render(venu, oracle, cuda):
    """The same job alone through venu_render and in a batch mix."""
    torch = cuda
    sp = oracle.scene_random(20000, 9)
    W, H, spp = 48, 32, 4
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    a1 = venu.new_accum(W, H)
    wf = venu.Wavefront(3000)
    wf.render(ds, cam, W, H, spp, a1, subframe=4, max_depth=50, reset=True)
    b = venu.Batch(pool_paths=4000, max_jobs=4)
    a2 = venu.new_accum(W, H)
    other = _submit_all(venu, torch, b, oracle, _jobs(oracle)[:1])
    b.submit(ds, cam, W, H, spp, a2, subframe=4, max_depth=50)
    b.run()
    b.collect()
    torch.cuda.synchronize()
    assert np.array_equal(a1.cpu().numpy().view(np.uint32), a2.cpu().numpy().view(np.uint32))
    assert np.array_equal(other[0]["acc"].cpu().numpy().view(np.uint32), other[0]["want"]["accum"].view(np.uint32))


def test_batch_limits(venu, oracle, cuda):
    b = venu.Batch(pool_paths=1000, max_jobs=1)
    sp = oracle.scene_rtiow(0)
    ds = venu.DeviceScene(sp)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, 1.0, 0.1, 10.0)
    acc = venu.new_accum(8, 8)
    b.submit(ds, cam, 8, 8, 1, acc)
    with pytest.raises(venu.VenuError):
        b.submit(ds, cam, 8, 8, 1, acc)  # max_jobs reached
    with pytest.raises(venu.VenuError):
        venu.Batch(pool_paths=1000, max_jobs=0)
    b.run()
    assert len(b.collect()) == 1


def test_batch_stop_on_finish(venu, oracle, cuda):
    """Each run with stop_on_finish ends right after some job completes; the
    jobs are handed out one run at a time and stay exact."""
    torch = cuda
    b = venu.Batch(pool_paths=600, max_jobs=8)
    sub = _submit_all(venu, torch, b, oracle, _jobs(oracle))
    got = []
    for _ in range(64):
        b.run(max_iterations=0, stop_on_finish=True)
        fin = b.collect()
        assert fin, "a run with stop_on_finish returned without finishing a job"
        got += fin
        if len(got) == len(sub):
            break
    assert sorted(got) == sorted(s["id"] for s in sub)
    torch.cuda.synchronize()
    for s in sub:
        assert np.array_equal(s["acc"].cpu().numpy().view(np.uint32), s["want"]["accum"].view(np.uint32))


def _one(venu, torch, oracle, b, scene, eye, W, H, spp, depth, sub=1):
    cam, want = _want(oracle, dict(scene=scene, eye=eye, W=W, H=H, spp=spp, depth=depth, sub=sub))
    ds = venu.DeviceScene(scene)
    acc = venu.new_accum(W, H)
    jid = b.submit(ds, cam, W, H, spp, acc, subframe=sub, max_depth=depth)
    return dict(id=jid, ds=ds, acc=acc, want=want)


@pytest.mark.parametrize("policy", ["fifo", "shortest_first", "sequential"])
def test_batch_policy(venu, oracle, cuda, policy):
    """A small job submitted behind a large one: shortest-first generates its
    paths at once (it finishes within a few iterations); FIFO only after the
    large job's paths are all generated; sequential only after the large job
    has finished.  Results are exact whatever the order."""
    torch = cuda
    b = venu.Batch(pool_paths=4096, max_jobs=4)
    b.set_policy(policy)
    sp = oracle.scene_rtiow(0)
    big = _one(venu, torch, oracle, b, sp, (13, 2, 3), 64, 64, 16, 4)
    small = _one(venu, torch, oracle, b, sp, (13, 2, 3), 8, 6, 1, 4)
    b.run(stop_on_finish=True)
    first = b.collect()
    it = b.stats()["iterations"]
    if policy == "shortest_first":
        assert first == [small["id"]] and it <= 8
    elif policy == "fifo":
        # 65536 paths through a 4096-path pool (>= 16 iterations) before the
        # small job's paths are generated
        assert first == [big["id"]] and it >= 16
    else:
        assert first == [big["id"]]  # the small job cannot start before the big one is done
    b.run()
    rest = b.collect()
    torch.cuda.synchronize()
    assert sorted(first + rest) == sorted([big["id"], small["id"]])
    for j in (big, small):
        assert np.array_equal(j["acc"].cpu().numpy().view(np.uint32), j["want"]["accum"].view(np.uint32))


@pytest.mark.parametrize("policy", ["fifo", "shortest_first", "sequential"])
def test_batch_many_jobs_policy(venu, oracle, cuda, policy):
    """70 jobs (more than one warp of the plan kernel, which hands out the
    free slots 32 jobs at a time) in a pool that holds a few of them: every
    result exact; under the sequential policy the jobs finish strictly in
    submission order."""
    torch = cuda
    b = venu.Batch(pool_paths=512, max_jobs=80)
    b.set_policy(policy)
    scenes = [oracle.scene_rtiow(k) for k in range(4)]
    jobs = []
    for k in range(70):
        W, H, spp = 8 + (k % 3) * 4, 6, 1 + (k * 7) % 3
        jobs.append(_one(venu, torch, oracle, b, scenes[k % 4], (13, 2, 3), W, H, spp, 4, sub=1 + k % 5))
    order = []
    for _ in range(400):
        b.run(stop_on_finish=True)
        order += b.collect()
        if len(order) == len(jobs):
            break
    torch.cuda.synchronize()
    assert sorted(order) == sorted(j["id"] for j in jobs)
    if policy == "sequential":
        assert order == [j["id"] for j in jobs]
    for j in jobs:
        assert np.array_equal(j["acc"].cpu().numpy().view(np.uint32), j["want"]["accum"].view(np.uint32))


def test_batch_submit_many(venu, oracle, cuda):
    """One call admits 44 jobs (two seed-table groups of at most 32): every
    result exact.  All or nothing: a call with one invalid job, or with more
    jobs than free slots, admits none."""
    torch = cuda
    b = venu.Batch(pool_paths=2048, max_jobs=48)
    scenes = [oracle.scene_rtiow(k) for k in range(3)]
    dev = [venu.DeviceScene(sp) for sp in scenes]
    specs, wants = [], []
    for k in range(44):
        W, H, spp, depth, sub = 6 + (k % 4) * 3, 5, 1 + k % 3, 4, 1 + k % 4
        cam, want = _want(oracle, dict(scene=scenes[k % 3], eye=(13, 2, 3), W=W, H=H, spp=spp, depth=depth, sub=sub))
        specs.append(dict(scene=dev[k % 3], camera=cam, width=W, height=H, spp=spp, subframe=sub, max_depth=depth,
                          accum=venu.new_accum(W, H)))
        wants.append(want)
    bad = dict(specs[0], width=1)
    with pytest.raises(venu.VenuError):
        b.submit_many(specs[:3] + [bad])
    assert b.stats()["active_jobs"] == 0
    with pytest.raises(venu.VenuError):
        b.submit_many(specs + specs[:5])  # 49 jobs, 48 slots
    assert b.stats()["active_jobs"] == 0
    ids = b.submit_many(specs)
    assert len(set(ids)) == 44 and b.stats()["active_jobs"] == 44
    b.run()
    assert sorted(b.collect()) == sorted(ids)
    torch.cuda.synchronize()
    for spec, want in zip(specs, wants):
        assert np.array_equal(spec["accum"].cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))


def test_batch_interrupt(venu, oracle, cuda):
    """While the interrupt flag is set a run ends after one iteration;
    cleared, the run goes to the end.  Results are exact."""
    torch = cuda
    b = venu.Batch(pool_paths=2048, max_jobs=2)
    j = _one(venu, torch, oracle, b, oracle.scene_rtiow(0), (13, 2, 3), 40, 30, 4, 8)
    b.interrupt(True)
    b.run()
    assert b.collect() == []
    assert b.stats()["iterations"] == 1
    b.run()
    assert b.stats()["iterations"] == 2
    b.interrupt(False)
    b.run()
    assert b.collect() == [j["id"]]
    torch.cuda.synchronize()
    assert np.array_equal(j["acc"].cpu().numpy().view(np.uint32), j["want"]["accum"].view(np.uint32))


@pytest.mark.parametrize("chunk", [1, 100, 7777])
def test_batch_chunked_steps(venu, oracle, cuda, chunk):
    """Iterations split into steps of `chunk` rays: the same accumulators;
    stop-on-finish, step caps and interrupts act at step boundaries."""
    torch = cuda
    b = venu.Batch(pool_paths=3000, max_jobs=8)
    b.set_chunk(chunk)
    sub = _submit_all(venu, torch, b, oracle, _jobs(oracle))
    got = []
    b.interrupt(True)
    b.run()
    assert b.stats()["iterations"] == 1  # one step, then the interrupt
    b.interrupt(False)
    for _ in range(100000):
        b.run(max_iterations=37, stop_on_finish=True)
        got += b.collect()
        if len(got) == len(sub):
            break
    assert sorted(got) == sorted(s["id"] for s in sub)
    torch.cuda.synchronize()
    total = 0
    for s in sub:
        assert np.array_equal(s["acc"].cpu().numpy().view(np.uint32), s["want"]["accum"].view(np.uint32))
        total += s["want"]["segments"]
    assert b.stats()["segments"] == total
