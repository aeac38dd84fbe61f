"""Autotuner for the wavefront renderer's launch shapes.

Times candidate venu_tuning settings (traversal variant, refill threshold,
block shapes, resident blocks per SM) and queue sizes (paths in flight) on a
reduced copy of the caller's workload -- the same scene, camera, resolution
and depth with fewer samples per pixel -- and returns the fastest.  Results
never change the image (every setting is bit-identical); only speed differs.
"""
from __future__ import annotations

import itertools
import math

from .core import DeviceScene, Wavefront, new_accum

DEFAULT_SPACE = {
    "traverse_variant": (0, 1, 2, 3, 4, 5),
    "refill_min": (4, 8, 16),
    "traverse_block": (64, 128, 256),
    "shade_block": (128, 256),
    "in_place_factor": (1, 8),
}


def candidates(space=None):
    space = dict(DEFAULT_SPACE, **(space or {}))
    seen = set()
    for v, r, tb, sb, f in itertools.product(space["traverse_variant"], space["refill_min"],
                                             space["traverse_block"], space["shade_block"],
                                             space["in_place_factor"]):
        # the refill threshold matters to the dynamic-fetch variant only, the
        # shade block to the variants with a separate shade kernel only, the
        # in-place factor to the variants that are fused on every bounce only
        key = (v, r if v == 1 else 32, tb, sb if v not in (2, 4) else 256, f if v in (2, 4) else 1)
        if key in seen:
            continue
        seen.add(key)
        yield dict(traverse_variant=v, refill_min=key[1], traverse_block=tb, traverse_blocks_per_sm=0,
                   shade_block=key[3], shade_blocks_per_sm=0, in_place_factor=key[4])


def time_render(wf: Wavefront, scene: DeviceScene, cam, W, H, spp, depth, accum, reps=2):
    import torch

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    wf.render(scene, cam, W, H, spp, accum, subframe=1, max_depth=depth, reset=True)  # warm
    ev0.record()
    for i in range(reps):
        wf.render(scene, cam, W, H, spp, accum, subframe=2 + i, max_depth=depth, reset=True)
    ev1.record()
    torch.cuda.synchronize()
    segs = wf.stats()["segments"]
    ms = ev0.elapsed_time(ev1) / reps
    return segs / (ms / 1000.0), ms


def autotune(scene: DeviceScene, cam, W, H, spp, depth, space=None, max_paths=(8 << 20,), tune_spp=None,
             reps=2, log=None, finalists=3, final_reps=6):
    """Returns (best_tuning: dict, best_max_paths: int, results: list).

    Every candidate is timed once (reps renders) on the reduced copy; then
    every candidate (when one render of the full workload takes at most
    about 50 ms) or the `finalists` fastest are timed again -- on the full
    workload when one render of it takes at most about 0.3 s (a short
    render repeated until each timing covers ~20 ms), else with final_reps
    renders of the reduced copy -- and the fastest of those wins,
    so that run-to-run noise and the reduced copy's smaller waves decide
    less."""
    tune_spp = tune_spp or max(1, min(spp, 8))
    accum = new_accum(W, H)
    results = []
    for mp in max_paths:
        wf = Wavefront(mp)
        for cand in candidates(space):
            wf.set_tuning(**cand)
            rate, ms = time_render(wf, scene, cam, W, H, tune_spp, depth, accum, reps)
            results.append(dict(cand, max_paths=mp, segments_per_s=rate, ms=ms))
            if log:
                log(results[-1])
        wf.close()
    ranked = sorted(results, key=lambda r: -r["segments_per_s"])
    # the finalists on the full workload when a render of it is short (the
    # reduced copy has the same scene but smaller waves, which can favour
    # other launch shapes: every candidate when a render takes at most
    # ~50 ms, the `finalists` fastest up to ~300 ms), else on the reduced
    # copy again
    full_ms = ranked[0]["ms"] * spp / tune_spp
    if full_ms <= 50.0:
        # a short render is repeated until each candidate's timing covers
        # ~20 ms: three renders of a 0.7 ms frame left the pick to launch
        # jitter (400x225x16: 128- or 256-thread blocks from run to run,
        # 5.46 against 5.37 G segments/s)
        final_spp, reps_final = spp, max(3, min(64, int(math.ceil(20.0 / max(full_ms, 1e-3)))))
    elif full_ms <= 300.0:
        final_spp, reps_final = spp, 3
        ranked = ranked[:max(1, finalists)]
    else:
        final_spp, reps_final = tune_spp, final_reps
        ranked = ranked[:max(1, finalists)]
    best = None
    for r in ranked:
        cand = {k: r[k] for k in r if k not in ("max_paths", "segments_per_s", "ms")}
        wf = Wavefront(r["max_paths"])
        wf.set_tuning(**cand)
        rate, ms = time_render(wf, scene, cam, W, H, final_spp, depth, accum, reps_final)
        wf.close()
        r["final_segments_per_s"] = rate
        r["final_spp"] = final_spp
        if best is None or rate > best[0]:
            best = (rate, cand, r["max_paths"])
    return best[1], best[2], results


def _time(fn) -> float:
    import torch

    fn()  # warm
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    fn()
    ev1.record()
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1)


def autotune_jobs(jobs, pools=(16 << 20, 32 << 20, 64 << 20), blocks=(64, 128, 256), space=None, log=None):
    """Tunes both ways of rendering a set of jobs on (a reduced copy of) it.

    jobs: list of dicts {scene: DeviceScene, camera, W, H, spp, depth,
    subframe}.  Returns (plain_tuning, batch_tuning, results):
    plain_tuning -- the venu_tuning fields that render the jobs fastest one
    by one; batch_tuning -- the batch engine's pool size and block shape
    that render them fastest together in one pool (the batch always traces
    and shades in one kernel).  Results never change any image.
    """
    from .core import Batch

    results = []
    accs = [new_accum(j["W"], j["H"]) for j in jobs]
    cands = list(candidates(space))
    wf = Wavefront(max(min(128 << 20, max(j["W"] * j["H"] * j["spp"] for j in jobs)), 1 << 20))

    def plain():
        for j, a in zip(jobs, accs):
            wf.render(j["scene"], j["camera"], j["W"], j["H"], j["spp"], a, subframe=j["subframe"],
                      max_depth=j["depth"], reset=True)

    best_plain = None
    for cand in cands:
        wf.set_tuning(**cand)
        ms = _time(plain)
        results.append(dict(cand, method="plain", ms=ms))
        if log:
            log(results[-1])
        if best_plain is None or ms < best_plain[0]:
            best_plain = (ms, dict(cand))
    wf.close()

    best_batch = None
    for pool in pools:
        b = Batch(pool_paths=pool, max_jobs=len(jobs))
        for tb in blocks:
            b.set_tuning(traverse_variant=2, traverse_block=tb)

            def batched():
                b.submit_many([dict(scene=j["scene"], camera=j["camera"], width=j["W"], height=j["H"], spp=j["spp"],
                                    accum=a, subframe=j["subframe"], max_depth=j["depth"]) for j, a in zip(jobs, accs)])
                b.run()
                b.collect()

            ms = _time(batched)
            results.append(dict(method="batched", pool_paths=pool, traverse_block=tb, ms=ms))
            if log:
                log(results[-1])
            if best_batch is None or ms < best_batch[0]:
                best_batch = (ms, dict(pool_paths=pool, traverse_block=tb))
        b.close()
    return best_plain[1], best_batch[1], results


def compare(scene: DeviceScene, cam, W, H, spp, depth=50, variants=(2, 3, 4, 5), blocks=(128, 256), reps=3,
            factors=(1, 8)):
    """Times every traversal variant x block shape on one render (the mean
    of `reps` renders after a warm-up) and, per variant, a counting render:
    box and sphere tests per segment, traversal steps per segment and the
    SIMD utilisation of the traversal loop.  Also checks that every setting
    gives the same accumulator.  Returns a list of dicts."""
    import torch

    out, ref = [], None
    accum = new_accum(W, H)
    for v in variants:
        for tb in blocks:
            for f in (factors if v in (2, 4) else (1,)):
                wf = Wavefront(min(1 << 30, W * H * spp))
                wf.set_tuning(traverse_variant=v, traverse_block=tb, in_place_factor=f)
                rate, ms = time_render(wf, scene, cam, W, H, spp, depth, accum, reps)
                same = None
                if ref is None:
                    ref = accum.clone()
                else:
                    same = bool(torch.equal(ref, accum))
                wf.close()
                out.append(dict(traverse_variant=v, traverse_block=tb, in_place_factor=f, segments_per_s=rate, ms=ms,
                                identical=same))
        wf = Wavefront(min(1 << 30, W * H * spp), count=True)
        wf.set_tuning(traverse_variant=v, traverse_block=blocks[0])
        wf.render(scene, cam, W, H, spp, accum, subframe=1 + reps, max_depth=depth, reset=True)
        torch.cuda.synchronize()
        st = wf.stats()
        wf.close()
        seg = max(1, st["segments"])
        out.append(dict(traverse_variant=v, counting=True, boxes_per_segment=st["nodes_visited"] / seg,
                        spheres_per_segment=st["spheres_tested"] / seg, steps_per_segment=st["lane_steps"] / seg,
                        simd_utilization=st["lane_steps"] / max(1, 32 * st["warp_steps"])))
    return out


def main(argv=None) -> None:
    """python -m venusaur_gb300.tune --scene rtiow|random [--n N --seed S]
    --width W --height H --spp K [--variants 2,3,4,5] [--blocks 128,256]:
    prints compare()'s rows as JSON lines (one GPU, the current device)."""
    import argparse
    import json

    from .core import Camera, generate_random, generate_rtiow

    ap = argparse.ArgumentParser(prog="python -m venusaur_gb300.tune")
    ap.add_argument("--scene", choices=("rtiow", "random"), default="rtiow")
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--spp", type=int, default=8)
    ap.add_argument("--depth", type=int, default=50)
    ap.add_argument("--variants", default="2,3,4,5")
    ap.add_argument("--blocks", default="128,256")
    ap.add_argument("--factors", default="1,8", help="in-place factors tried with the fused variants")
    a = ap.parse_args(argv)
    sp = generate_rtiow(a.seed) if a.scene == "rtiow" else generate_random(a.n, a.seed)
    eye = (13.0, 2.0, 3.0) if a.scene == "rtiow" else (60.0, 15.0, 60.0)
    cam = Camera.look_at(eye, (0.0, 0.0, 0.0), 20.0, a.width / a.height, 0.1, 10.0)
    ds = DeviceScene(sp)
    for row in compare(ds, cam, a.width, a.height, a.spp, a.depth, [int(x) for x in a.variants.split(",")],
                       [int(x) for x in a.blocks.split(",")], factors=[int(x) for x in a.factors.split(",")]):
        print(json.dumps(row), flush=True)
    info = ds.info()  # after the renders: variants 4 and 5 build the 4-wide tree on first use
    print(json.dumps(dict(scene=a.scene, spheres=len(sp), width=a.width, height=a.height, spp=a.spp,
                          build_ms=info["build_ms"], wide_nodes=info["num_wide_nodes"], wide_ms=info["wide_ms"])))


if __name__ == "__main__":
    main()
