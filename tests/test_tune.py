"""The autotuner: its candidate space (CPU) and, on the GPU, that both tuners
return settings from their spaces and that a tuned render is bit-identical
to an untuned one (tuning changes speed only)."""
import numpy as np
import pytest

from venusaur_gb300 import tune


def test_candidate_space():
    c = list(tune.candidates())
    # variant 1 x refill {4,8,16} x traverse block {64,128,256} x shade {128,256},
    # variants 0, 3 and 5 x traverse block x shade block, variants 2 and 4 x
    # traverse block x in-place factor
    assert len(c) == 3 * 3 * 2 + 3 * 3 * 2 + 2 * 3 * 2
    assert len({tuple(sorted(x.items())) for x in c}) == len(c)
    for x in c:
        assert x["traverse_variant"] in (0, 1, 2, 3, 4, 5)
        if x["traverse_variant"] != 1:
            assert x["refill_min"] == 32
        if x["traverse_variant"] in (2, 4):
            assert x["shade_block"] == 256
        else:
            assert x["in_place_factor"] == 1
    small = list(tune.candidates({"traverse_variant": (2,), "traverse_block": (128,), "in_place_factor": (1,)}))
    assert len(small) == 1
    v5 = list(tune.candidates({"traverse_variant": (5,)}))
    assert len(v5) == 3 * 2 and all(x["traverse_variant"] == 5 for x in v5)


@pytest.mark.gpu
def test_autotune_render_and_jobs(venu, oracle, cuda):
    torch = cuda
    W, H, spp, depth = 64, 36, 2, 12
    sp = oracle.scene_rtiow(0)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    ds = venu.DeviceScene(sp)
    space = {"traverse_variant": (0, 2), "refill_min": (8,), "traverse_block": (64, 256), "shade_block": (256,),
             "in_place_factor": (1,)}
    best, mp, res = tune.autotune(ds, cam, W, H, spp, depth, space=space, max_paths=(1 << 20,))
    assert mp == 1 << 20 and len(res) == 4
    assert best in [{k: v for k, v in r.items() if k in best} for r in res]

    wf = venu.Wavefront(1 << 20)
    plain = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, plain, subframe=3, max_depth=depth, reset=True)
    wf.set_tuning(**best)
    tuned = venu.new_accum(W, H)
    wf.render(ds, cam, W, H, spp, tuned, subframe=3, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    assert torch.equal(plain, tuned)

    rnd = venu.DeviceScene(oracle.scene_random(3000, 5))
    jobs = [dict(scene=ds, camera=cam, W=W, H=H, spp=spp, depth=depth, subframe=1),
            dict(scene=rnd, camera=oracle.camera((60, 15, 60), (0, 0, 0), 20.0, 1.0, 0.1, 10.0), W=48, H=48,
                 spp=3, depth=depth, subframe=2)]
    pools, blocks = (1 << 20, 2 << 20), (128, 256)
    p_best, b_best, res = tune.autotune_jobs(jobs, pools=pools, blocks=blocks, space=space)
    assert len(res) == 4 + len(pools) * len(blocks)
    assert b_best["pool_paths"] in pools and b_best["traverse_block"] in blocks
    assert p_best["traverse_variant"] in (0, 2)
    b = venu.Batch(pool_paths=b_best["pool_paths"], max_jobs=2)
    b.set_tuning(traverse_variant=2, traverse_block=b_best["traverse_block"])
    accs = [venu.new_accum(j["W"], j["H"]) for j in jobs]
    for j, a in zip(jobs, accs):
        b.submit(j["scene"], j["camera"], j["W"], j["H"], j["spp"], a, subframe=j["subframe"], max_depth=depth)
    b.run()
    assert len(b.collect()) == 2
    torch.cuda.synchronize()
    want = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth)
    assert np.array_equal(accs[0].cpu().numpy().view(np.uint32), want["accum"].view(np.uint32))
