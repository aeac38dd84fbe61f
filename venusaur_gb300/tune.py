"""Autotuner for the wavefront renderer's launch shapes.

Times candidate venu_tuning settings (traversal variant, refill threshold,
block shapes, resident blocks per SM) and queue sizes (paths in flight) on a
reduced copy of the caller's workload -- the same scene, camera, resolution
and depth with fewer samples per pixel -- and returns the fastest.  Results
never change the image (every setting is bit-identical); only speed differs.
"""
from __future__ import annotations

import itertools

from .core import DeviceScene, Wavefront, new_accum

DEFAULT_SPACE = {
    "traverse_variant": (0, 1, 2, 3, 4, 5),
    "refill_min": (4, 8, 16),
    "traverse_block": (64, 128, 256),
    "shade_block": (128, 256),
}


def candidates(space=None):
    space = dict(DEFAULT_SPACE, **(space or {}))
    seen = set()
    for v, r, tb, sb in itertools.product(space["traverse_variant"], space["refill_min"],
                                          space["traverse_block"], space["shade_block"]):
        # the refill threshold matters to the dynamic-fetch variants only, the
        # shade block to the variants with a separate shade kernel only
        key = (v, r if v == 1 else 32, tb, sb if v not in (2, 4) else 256)
        if key in seen:
            continue
        seen.add(key)
        yield dict(traverse_variant=v, refill_min=key[1], traverse_block=tb, traverse_blocks_per_sm=0,
                   shade_block=key[3], shade_blocks_per_sm=0)


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

    Every candidate is timed once (reps renders); the `finalists` fastest are
    timed again with final_reps renders each and the fastest of those wins,
    so that run-to-run noise between close candidates decides less."""
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
    ranked = sorted(results, key=lambda r: -r["segments_per_s"])[:max(1, finalists)]
    best = None
    for r in ranked:
        cand = {k: r[k] for k in r if k not in ("max_paths", "segments_per_s", "ms")}
        wf = Wavefront(r["max_paths"])
        wf.set_tuning(**cand)
        rate, ms = time_render(wf, scene, cam, W, H, tune_spp, depth, accum, final_reps)
        wf.close()
        r["final_segments_per_s"] = rate
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
