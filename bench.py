"""Benchmark: path segments/s of the RTIOW path tracer on GB300.

Headline workload (`--config c2`): the RTIOW final scene (485 spheres, seed
0), 1920x1080, 256 spp, max depth 50, FP32 Kahan accumulation, rendered by
the plain single-scene wavefront method.  One step = one full render (Draw)
of that image.  Inputs are synthetic (the seeded scene generator); the
working set of the ray queues (>1.5 GB) is far larger than L2, so no explicit
L2 flush is done between steps.

Reported keys (one JSON line on rank 0):
  value      segments/s with the scene resident (device-timed, CUDA events)
  e2e        the same metric through the public C ABI from host memory:
             scene upload + LBVH build + render + image download per step
  roofline   the traversal kernel: algorithmic bytes per launch / its
             event-timed duration against the measured HBM copy bandwidth,
             the measured SIMD utilisation of its traversal loop, its FP32
             rate, and (when the kernel sources match the ones the ncu
             figures were taken on) DRAM bytes per segment
  configs    the other single-GPU configurations: c1 (400x225x16) and c3
             (1M spheres, 1080p x 64, with the LBVH build time and bytes
             fetched per ray segment)
  cpu_baseline  the reference's arithmetic (its intersection and shading
             programs restated on the host, closest hit through the host LBVH)
             on a fixed sample of the workload, every host thread
  batched / batched_small_jobs / served   plain vs batched vs served methods

`--impl reference` times the same host restatement of the reference's
arithmetic on the same fixed sample each step and prints its line; it loads
nothing of the product library.  With torchrun (N>1) each rank renders its
own replica (no collective on the data path); rank 0 prints the aggregate.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    "c1": dict(workload="RTIOW final scene, 400x225, 16 spp, depth 50, plain wavefront", scene="rtiow",
               W=400, H=225, spp=16, depth=50, eye=(13, 2, 3)),
    "c2": dict(workload="RTIOW final scene, 1920x1080, 256 spp, depth 50, plain wavefront", scene="rtiow",
               W=1920, H=1080, spp=256, depth=50, eye=(13, 2, 3)),
    "c3": dict(workload="1M-sphere scene (200x20x200 box), 1920x1080, 64 spp, depth 50, plain wavefront",
               scene="random1m", W=1920, H=1080, spp=64, depth=50, eye=(60, 15, 60)),
}
# The fixed CPU sample of each configuration: rows [r0, r1) of the image at
# `spp` samples per pixel, subframe 1.  The cpu_baseline leg and every step of
# the reference arm render exactly this sample.
CPU_SAMPLE = {
    "c1": dict(rows=(0, 225), spp=16),
    "c2": dict(rows=(540, 1080), spp=64),
    "c3": dict(rows=(540, 548), spp=8),
}
METRIC = "path segments/s on 1 GB300 (batched/served vs plain); p50/p99 render latency"
UNIT = "segments/s"
# the renderer's largest wave (venu_renderer_create) and the batch engine's
# largest pool (venu_batch_create)
MAX_WAVE_PATHS = 1 << 30
MAX_POOL_PATHS = 1 << 28

# Sources of the plain renderer's kernels: the ncu figures below hold only
# while these files are byte-identical to the ones they were taken on.
KERNEL_SOURCES = ("venusaur_gb300/csrc/venu_device.cuh", "venusaur_gb300/csrc/render_kernels.cuh",
                  "venusaur_gb300/csrc/render.cu")
# ncu figures of the dominant kernel, per (config, traverse variant), summed
# over every launch of one render of a reduced case of the same scene (fewer
# samples per pixel: the per-segment traffic does not depend on the sample
# count).  dram_b_per_seg = (dram__bytes_read.sum + dram__bytes_write.sum) /
# segments; lanes_per_inst = smsp__thread_inst_executed_per_inst_executed.ratio
# (active lanes per issued instruction, all instructions).  `sha` is
# kernel_sources_sha() of the captured build.  Each figure is summed over the
# k_trace_shade (and, for variant 3, k_traverse) launches of two renders of
# `bench.py --config <c> --spp <s> --profile-render --tuning <variant>`
# (c2: 4 spp, c3: 2 spp, c1: its own 16 spp; "/f8": in_place_factor 8;
# traverse_block 256 for c2/v2, c3/v2 and c3/v3, 128 for the others)
# under ncu --metrics
# dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum,
# smsp__inst_executed.sum,smsp__thread_inst_executed.sum.
NCU_FIGURES = {"sha": "7ec4d38e57e4d468", "commit": "4264606", "figures": {
    "c2/v2": {"dram_b_per_seg": 62.6, "lanes_per_inst": 15.87, "warp_inst_per_seg": 82.1},
    "c2/v4": {"dram_b_per_seg": 63.86, "lanes_per_inst": 17.82, "warp_inst_per_seg": 84.3},
    "c1/v2": {"dram_b_per_seg": 38.26, "lanes_per_inst": 14.14, "warp_inst_per_seg": 104.0},
    "c1/v2/f8": {"dram_b_per_seg": 25.28, "lanes_per_inst": 14.96, "warp_inst_per_seg": 108.5},
    "c1/v4": {"dram_b_per_seg": 41.31, "lanes_per_inst": 16.01, "warp_inst_per_seg": 104.6},
    "c1/v4/f8": {"dram_b_per_seg": 26.64, "lanes_per_inst": 16.92, "warp_inst_per_seg": 110.1},
    "c3/v3": {"dram_b_per_seg": 62.21, "lanes_per_inst": 6.58, "warp_inst_per_seg": 657.5},
    "c3/v2": {"dram_b_per_seg": 127.3, "lanes_per_inst": 6.41, "warp_inst_per_seg": 721.7},
    "c3/v5": {"dram_b_per_seg": 60.63, "lanes_per_inst": 8.48, "warp_inst_per_seg": 630.0},
}}


def kernel_sources_sha() -> str:
    """Hash of the kernel code: the sources with comments removed and
    whitespace collapsed, so that only a change of code invalidates the ncu
    figures."""
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, f), encoding="utf-8") as fh:
            code = fh.read()
        code = re.sub(r"/\*.*?\*/", " ", code, flags=re.S)
        code = re.sub(r"//[^\n]*", " ", code)
        h.update(" ".join(code.split()).encode())
    return h.hexdigest()[:16]


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_scene(venu, kind):
    if kind == "rtiow":
        return venu.generate_rtiow(0)
    if kind == "random1m":
        return venu.generate_random(1_000_000, 1)
    raise ValueError(kind)


def oracle_scene(O, cfg):
    """The same scene and camera from the oracle's own generators (equal to
    the product's byte for byte), so a CPU leg needs nothing of the product."""
    sp = O.scene_rtiow(0) if cfg["scene"] == "rtiow" else O.scene_random(1_000_000, 1)
    cam = O.camera(cfg["eye"], (0, 0, 0), 20.0, cfg["W"] / cfg["H"], 0.1, 10.0)
    return sp, cam


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_run(O, spheres, cam, cfg, name, mode, nthreads, repeats=1):
    """Renders the fixed CPU sample of configuration `name` `repeats` times
    on the host; returns (segments/s, seconds, segments, description)."""
    from oracle import pyoracle

    smp = CPU_SAMPLE[name]
    (r0, r1), spp = smp["rows"], smp["spp"]
    W, H, depth = cfg["W"], cfg["H"], cfg["depth"]
    segs, secs = 0, 0.0
    for _ in range(repeats):
        t0 = time.perf_counter()
        res = O.render(spheres, cam, W, H, spp, subframe=1, max_depth=depth, mode=mode, nthreads=nthreads,
                       rows=(r0, r1))
        secs += time.perf_counter() - t0
        segs += res["segments"]
    arith = {pyoracle.MODE_REF_BVH: "reference", pyoracle.MODE_GB300: "gb300", pyoracle.MODE_REF: "reference"}[mode]
    desc = (f"rows [{r0},{r1}) x {W} px x {spp} spp (depth {depth}, subframe 1) of the {W}x{H} workload, "
            f"{arith} arithmetic")
    return segs / secs, secs, segs, desc


REF_ARITH = ("the reference's intersection, closest-hit and miss programs (Core/RayTracer.cu:163-449: half-b "
             "quadratic, double-precision dielectric, pow() Schlick, recursive attenuation) restated on the host "
             "and bit-exact with the reference's own RayTracer.cu compiled for the host; closest hit through "
             "the host LBVH in place of OptiX's traversal")


def rmse_vs_reference(venu, torch, O, ds, spheres, cam, W, H, depth, spp=16):
    """Per-pixel RMSE of the GPU image against the reference's arithmetic
    (the oracle's REF mode: the reference's own RayTracer.cu semantics --
    double-precision dielectric, pow() Schlick, half-b quadratic,
    brute-force closest hit -- pinned bit-exactly to the reference's code
    compiled for the host) at the same seeds on the middle row, beside the
    seed-to-seed noise of the same estimate."""
    from oracle import pyoracle

    row = H // 2
    acc = venu.new_accum(W, H)
    wf = venu.Wavefront(0)
    wf.render(ds, cam, W, H, spp, acc, subframe=0, max_depth=depth, reset=True)
    a = acc.cpu().numpy()[row * W:(row + 1) * W]
    gpu = a[:, :3] / a[:, 3:4]
    wf.render(ds, cam, W, H, spp, acc, subframe=7, max_depth=depth, reset=True)
    b = acc.cpu().numpy()[row * W:(row + 1) * W]
    other_seeds = b[:, :3] / b[:, 3:4]
    wf.close()
    ref = O.render(spheres, cam, W, H, spp, subframe=0, max_depth=depth, mode=pyoracle.MODE_REF,
                   rows=(row, row + 1))["accum"][row * W:(row + 1) * W, :3]
    rmse = float(np.sqrt(((gpu - ref) ** 2).mean()))
    noise = float(np.sqrt(((other_seeds - ref) ** 2).mean()))
    return {"value": rmse, "seed_noise": noise,
            "sample": f"row {row}, {W} px x {spp} spp, depth {depth}, subframe 0 (same seeds); seed_noise: "
                      "the same against subframe 7",
            "against": "the reference's arithmetic (oracle REF mode, bit-exact with the reference's own "
                       "RayTracer.cu built for the host)"}


def run_single_job(venu, torch, tuning, ds, cam, W, H, spp, depth, segs_step, subframe, pool):
    """The same render as one job of the batch engine: one pool of paths
    regenerated continuously (no waves, no tails), one graph launch.  The
    accumulator must equal the plain renderer's bit for bit."""
    b = venu.Batch(pool_paths=pool, max_jobs=1)
    if tuning:
        b.set_tuning(**tuning)
    acc_b, acc_p = venu.new_accum(W, H), venu.new_accum(W, H)
    wf = venu.Wavefront(pool)
    if tuning:
        wf.set_tuning(**tuning)
    wf.render(ds, cam, W, H, spp, acc_p, subframe=subframe, max_depth=depth, reset=True)
    wf.close()

    def one():
        b.submit(ds, cam, W, H, spp, acc_b, subframe=subframe, max_depth=depth, reset=True)
        b.run()
        assert len(b.collect()) == 1

    one()  # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    one()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    same = bool(torch.equal(acc_b, acc_p))
    b.close()
    return {"value": segs_step / (ms / 1000.0), "unit": UNIT, "ms": ms, "identical_accumulator": same,
            "method": "the headline render as one job of the batch engine: continuous path regeneration in a "
                      f"{pool >> 20} Mi-path pool, one graph launch (includes its seed-table kernel)"}


def profile_mixed(venu, torch, args):
    """A few steps of the mixed workload for a profiler: its first 12 jobs
    (2.3 GB of seed tables and sample slots) admitted to a 16 Mi-path pool,
    the host-driven loop, the given launch shapes."""
    from venusaur_gb300 import workloads

    jobs = workloads.mixed_jobs(64)[:12]
    b = venu.Batch(pool_paths=16 << 20, max_jobs=len(jobs), graph=False)
    b.set_tuning(**(json.loads(args.tuning) if args.tuning else dict(traverse_variant=2, traverse_block=256)))
    scenes, keep = {}, []
    for j in jobs:
        key = (j["n"], j["scene_seed"])
        if key not in scenes:
            scenes[key] = venu.DeviceScene(venu.generate_random(j["n"], j["scene_seed"]))
        cam = venu.Camera.look_at(j["eye"], (0, 0, 0), 20.0, j["W"] / j["H"], 0.1, 10.0)
        acc = venu.new_accum(j["W"], j["H"])
        keep.append(acc)
        b.submit(scenes[key], cam, j["W"], j["H"], j["spp"], acc, subframe=j["subframe"], max_depth=j["depth"])
    b.run(max_iterations=args.profile_mixed)
    torch.cuda.synchronize()
    print(json.dumps({"profile_mixed": b.stats()}))


def batch_ceiling(venu, torch, wf, jobs, cams, scenes, sat_paths=64 << 20):
    """What batching can recover on this job set at most, with these kernels:
    every job rendered alone by the plain method (device time, CUDA events),
    against the time its segments take at the rate the plain method reaches
    on the same scene, camera and resolution when the GPU is saturated (the
    job re-rendered with its samples per pixel raised to at least `sat_paths`
    paths).  A batcher that ran every job at its scene's saturated rate would
    take sum(ideal); plain takes sum(alone): their ratio bounds the speed-up
    of any batching of these jobs."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    alone_ms, ideal_ms, rows = 0.0, 0.0, []
    for j, cam in zip(jobs, cams):
        W, H = j["W"], j["H"]
        acc = venu.new_accum(W, H)
        ds = scenes[j["key"]]

        def once(spp, sub):
            e0.record()
            wf.render(ds, cam, W, H, spp, acc, subframe=sub, max_depth=j["depth"], reset=True)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1), wf.stats()["segments"]

        once(j["spp"], j["subframe"])  # warm
        t_ms, segs = once(j["spp"], j["subframe"])
        sat_spp = max(j["spp"], -(-sat_paths // (W * H)))
        st_ms, st_segs = once(sat_spp, j["subframe"])
        rate = st_segs / st_ms
        alone_ms += t_ms
        ideal_ms += segs / rate
        rows.append((W * H * j["spp"], t_ms, segs / rate))
        del acc
    rows.sort()
    half = len(rows) // 2
    return {"plain_alone_ms": alone_ms, "ideal_ms": ideal_ms, "max_speedup": alone_ms / ideal_ms,
            "smaller_half": {"plain_alone_ms": sum(r[1] for r in rows[:half]),
                             "ideal_ms": sum(r[2] for r in rows[:half])},
            "larger_half": {"plain_alone_ms": sum(r[1] for r in rows[half:]),
                            "ideal_ms": sum(r[2] for r in rows[half:])},
            "method": "each job alone by the plain method vs its segments at its scene's saturated plain rate "
                      f"(same scene, camera and resolution, spp raised to >= {sat_paths >> 20} Mi paths)"}


def profile_render(venu, torch, cfg, args):
    """One warm-up render and one render of the configuration (for a
    profiler's launch list: the second render's launches follow the first's)."""
    W, H, spp, depth = cfg["W"], cfg["H"], cfg["spp"], cfg["depth"]
    ds = venu.DeviceScene(make_scene(venu, cfg["scene"]))
    cam = venu.Camera.look_at(cfg["eye"], (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    # the profiling build launches every bounce from the host (ncu does not
    # profile kernels of graphs with conditional nodes, which the fused
    # variants otherwise run each wave's bounce loop as); the kernels and
    # their work are the same
    wf = venu.Wavefront(int(min(MAX_WAVE_PATHS, W * H * spp)), profile=True)
    wf.set_tuning(**(json.loads(args.tuning) if args.tuning else dict(traverse_variant=2, traverse_block=128)))
    acc = venu.new_accum(W, H)
    out = []
    for sub in (1, 2):
        wf.render(ds, cam, W, H, spp, acc, subframe=sub, max_depth=depth, reset=True)
        torch.cuda.synchronize()
        st = wf.stats()
        out.append({"segments": st["segments"], "paths": st["paths"], "kernel_launches": st["kernel_launches"]})
    print(json.dumps({"profile_render": cfg["workload"], "tuning": wf.tuning(), "renders": out,
                      "kernel_sources_sha": kernel_sources_sha()}))


def run_batched(venu, torch, tuning, max_paths, n_jobs=64, small=False, autotune=True):
    """The plain method (one venu_render per job, in sequence) against the
    batched engine (all jobs in one shared pool, one graph launch) on the
    mixed-scene workload (or, small=True, on many small RTIOW renders).
    BVHs are built before timing (resident scenes)."""
    from venusaur_gb300 import workloads

    jobs = workloads.small_jobs() if small else workloads.mixed_jobs(n_jobs)
    scenes = {}
    for j in jobs:
        key = ("rtiow", j["rtiow_seed"]) if small else (j["n"], j["scene_seed"])
        j["key"] = key
        if key not in scenes:
            sp = venu.generate_rtiow(j["rtiow_seed"]) if small else venu.generate_random(j["n"], j["scene_seed"])
            scenes[key] = venu.DeviceScene(sp)
    cams = [venu.Camera.look_at(j["eye"], (0, 0, 0), 20.0, j["W"] / j["H"], 0.1, 10.0) for j in jobs]
    # launch shapes for both methods, and the batch pool size, from the
    # autotuner on a reduced copy of this job set (every 4th job, at most
    # 16 spp: ~80 Mi paths of the mixed set, more than the largest pool):
    # each method gets its own best settings
    if autotune:
        from venusaur_gb300 import tune

        red = [dict(scene=scenes[j["key"]], camera=c, W=j["W"], H=j["H"], spp=min(j["spp"], 16), depth=j["depth"],
                    subframe=j["subframe"]) for j, c in list(zip(jobs, cams))[::4]]
        tuning, batch_tuning, _ = tune.autotune_jobs(red, pools=(16 << 20, 32 << 20, 64 << 20, 128 << 20))
    else:
        batch_tuning = {"pool_paths": min(max_paths, MAX_POOL_PATHS), "traverse_block": 256}
    acc_plain = [venu.new_accum(j["W"], j["H"]) for j in jobs]
    acc_batch = [venu.new_accum(j["W"], j["H"]) for j in jobs]
    img_plain = [torch.empty((j["W"] * j["H"], 4), dtype=torch.uint8, device="cuda") for j in jobs]
    img_batch = [torch.empty((j["W"] * j["H"], 4), dtype=torch.uint8, device="cuda") for j in jobs]
    wf = venu.Wavefront(128 << 20)
    if tuning:
        wf.set_tuning(**tuning)
    b = venu.Batch(pool_paths=batch_tuning["pool_paths"], max_jobs=len(jobs))
    b.set_tuning(traverse_variant=2, traverse_block=batch_tuning["traverse_block"])

    def plain(rep):
        segs = 0
        for j, cam, acc, img in zip(jobs, cams, acc_plain, img_plain):
            wf.render(scenes[j["key"]], cam, j["W"], j["H"], j["spp"], acc, subframe=j["subframe"],
                      max_depth=j["depth"], reset=True, image8=img)
        return segs

    def batched(rep):
        b.submit_many([dict(scene=scenes[j["key"]], camera=cam, width=j["W"], height=j["H"], spp=j["spp"],
                            accum=acc, subframe=j["subframe"], max_depth=j["depth"], image8=img)
                       for j, cam, acc, img in zip(jobs, cams, acc_batch, img_batch)])
        b.run()
        done = b.collect()
        assert len(done) == len(jobs)

    def timed(fn):
        fn(-1)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        fn(0)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), 1000 * (time.perf_counter() - t0)

    seg0 = b.stats()["segments"]
    b_ms, b_wall = timed(batched)
    segs = (b.stats()["segments"] - seg0) // 2
    p_ms, p_wall = timed(plain)
    same_all = all(torch.equal(acc_plain[i], acc_batch[i]) for i in range(len(jobs)))
    ceiling = None if small else batch_ceiling(venu, torch, wf, jobs, cams, scenes)
    desc = (f"{len(jobs)} RTIOW scenes (seeds 0..{len(jobs) - 1}), 256x144, 4 spp, depth 50" if small else
            f"{n_jobs} scenes, spheres log-uniform 100..200000, resolutions {{256x256, 512x512, 640x360, "
            f"1024x1024}}, spp {{4, 16, 64}}, depth 50 (seeded)")
    return {
        "workload": desc,
        "paths": workloads.paths(jobs), "segments": int(segs),
        "plain": {"value": segs / (p_ms / 1000), "ms": p_ms, "wall_ms": p_wall,
                  "method": "venu_render per job, in sequence (waves of up to 128 Mi paths)",
                  "tuning": tuning},
        "batched": {"value": segs / (b_ms / 1000), "ms": b_ms, "wall_ms": b_wall,
                    "method": "one shared path pool, one graph launch", "tuning": batch_tuning},
        "speedup": p_ms / b_ms,
        "identical_accumulators": bool(same_all),
        "ceiling": ceiling,
    }


def run_served(venu, torch, tuning, n_sessions=40, util=0.8, budget=150 << 30):
    """Serving the progressive-session workload: sessions of requests of 8, 8,
    16, 32, 64 spp (each submitted when the previous image is back,
    accumulated on the device) on scenes from the 1M-sphere distribution (100..1M
    spheres, one scene per session, its BVH built when its first request is
    admitted and kept resident for the rest), four resolutions, depth 50.

    Each method's capacity is measured at saturation (every session starting
    at once); each then serves a Poisson stream of session starts at `util`
    of its own capacity.  Methods: the render server (continuous batching,
    150 GB HBM budget; one lane FIFO, and an express lane for requests of
    at most 4 Mi paths ahead of a sequential bulk lane), and the plain
    method serving requests one at a time in arrival order.  A last run
    serves the server's stream under a budget small enough to bind, so that
    admission waits and scenes are evicted (an evicted scene is sent again
    by its session's next request)."""
    import heapq

    from venusaur_gb300 import workloads
    from venusaur_gb300._lib import lib

    base = workloads.serving_sessions(n_sessions)
    spheres = [venu.generate_random(s["n"], s["scene_seed"]) for s in base]
    cams = [venu.Camera.look_at(s["eye"], (0, 0, 0), 20.0, s["W"] / s["H"], 0.1, 10.0) for s in base]
    n_req = sum(len(s["steps"]) for s in base)

    def pct(lat):
        lat = np.asarray(lat)
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max())}

    def serve(srv, arrivals):
        """Drives the server: one thread per session, requests in order."""
        lat, first, segs0 = [], [], srv.stats()["segments"]
        failed = [0]
        lock = threading.Lock()
        start = time.perf_counter()

        def session(i):
            s = base[i]
            dt = start + arrivals[i] - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            sub = 1
            for k, spp in enumerate(s["steps"]):
                kw = dict(scene_key=i + 1, session=i + 1, subframe=sub, max_depth=s["depth"], reset=(k == 0))
                rid = srv.submit(cams[i], s["W"], s["H"], spp, spheres=spheres[i] if k == 0 else None, **kw)
                r = srv.wait(rid)
                if r["status"] == 1 and k > 0:  # its scene was evicted: send it again
                    rid = srv.submit(cams[i], s["W"], s["H"], spp, spheres=spheres[i], **kw)
                    r = srv.wait(rid)
                with lock:
                    if r["status"] != 0:
                        failed[0] += 1
                    lat.append(r["latency_ms"])
                    if k == 0:
                        first.append(r["latency_ms"])
                sub += spp
            srv.end_session(i + 1)

        ths = [threading.Thread(target=session, args=(i,)) for i in range(len(base))]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        makespan = time.perf_counter() - start
        st = srv.stats()
        out = pct(lat)
        out.update({"p50_ms_first": float(np.percentile(first, 50)), "requests": len(lat), "failed": failed[0],
                    "makespan_s": makespan, "value": (st["segments"] - segs0) / makespan, "unit": UNIT,
                    "evictions": int(st["evictions"]), "admission_waits": int(st["admission_waits"]),
                    "peak_resident_gb": st["peak_resident_bytes"] / 2**30, "budget_gb": st["budget_bytes"] / 2**30})
        return out

    def new_server(kind, budget_bytes):
        if kind == "fifo":
            return venu.Server(budget_bytes, pool_paths=64 << 20, max_jobs=256, iterations_per_step=64)
        srv = venu.Server(budget_bytes, pool_paths=64 << 20, max_jobs=256, iterations_per_step=64,
                          express_paths=4 << 20)
        srv.set_policy("sequential")
        return srv

    wf = venu.Wavefront(128 << 20)
    if tuning:
        wf.set_tuning(**tuning)

    def serve_plain(arrivals):
        """The plain method: one request at a time, in the order they become
        ready (a session's next request when its previous image is back);
        each session's BVH built on its first request, its accumulator kept."""
        ready = [(arrivals[i], i, i, 0) for i in range(len(base))]
        heapq.heapify(ready)
        seq = len(base)
        dscenes, accs, sub = {}, {}, [1] * len(base)
        lat, first, segs = [], [], 0
        start = time.perf_counter()
        while ready:
            t_ready, _, i, k = heapq.heappop(ready)
            now = time.perf_counter() - start
            if now < t_ready:
                time.sleep(t_ready - now)
            s = base[i]
            if k == 0:
                dscenes[i] = venu.DeviceScene(spheres[i])
                accs[i] = venu.new_accum(s["W"], s["H"])
            img = torch.empty((s["W"] * s["H"], 4), dtype=torch.uint8, device="cuda")
            spp = s["steps"][k]
            wf.render(dscenes[i], cams[i], s["W"], s["H"], spp, accs[i], subframe=sub[i], max_depth=s["depth"],
                      reset=(k == 0), image8=img)
            img.cpu()
            segs += wf.stats()["segments"]
            sub[i] += spp
            t_done = time.perf_counter() - start
            lat.append(1000.0 * (t_done - t_ready))
            if k == 0:
                first.append(lat[-1])
            if k + 1 < len(s["steps"]):
                heapq.heappush(ready, (t_done, seq, i, k + 1))
                seq += 1
            else:
                del dscenes[i], accs[i]
        makespan = time.perf_counter() - start
        out = pct(lat)
        out.update({"p50_ms_first": float(np.percentile(first, 50)), "requests": len(lat), "failed": 0,
                    "makespan_s": makespan, "value": segs / makespan, "unit": UNIT})
        return out

    unit = workloads.serving_sessions(n_sessions, rate_per_s=1.0)
    unit_arr = [s["arrival"] for s in unit]
    burst = [0.0] * len(base)
    out = {}
    # capacities at saturation
    cap = {}
    for kind in ("fifo", "express"):
        srv = new_server(kind, budget)
        r = serve(srv, burst)
        srv.close()
        cap[kind] = {"sessions_per_s": len(base) / r["makespan_s"], "requests_per_s": n_req / r["makespan_s"],
                     "value": r["value"], "p99_ms": r["p99_ms"], "peak_resident_gb": r["peak_resident_gb"]}
    r = serve_plain(burst)
    cap["plain"] = {"sessions_per_s": len(base) / r["makespan_s"], "requests_per_s": n_req / r["makespan_s"],
                    "value": r["value"], "p99_ms": r["p99_ms"]}
    out["capacity"] = cap
    # streams at util of each method's own capacity
    for kind in ("fifo", "express"):
        lam = util * cap[kind]["sessions_per_s"]
        srv = new_server(kind, budget)
        out[f"server_{kind}"] = serve(srv, [t / lam for t in unit_arr])
        out[f"server_{kind}"]["sessions_per_s"] = lam
        srv.close()
    lam_p = util * cap["plain"]["sessions_per_s"]
    out["plain"] = serve_plain([t / lam_p for t in unit_arr])
    out["plain"]["sessions_per_s"] = lam_p
    # the plain method's stream through both servers as well: the same
    # offered load for every method
    for kind in ("fifo", "express"):
        srv = new_server(kind, budget)
        out[f"server_{kind}_at_plain_load"] = serve(srv, [t / lam_p for t in unit_arr])
        srv.close()
    # a budget that binds: room for the largest request (its job, image and
    # scene) and every session's accumulator, plus a quarter
    need = max(int(lib().venu_batch_job_bytes(s["W"], s["H"], spp)) + s["W"] * s["H"] * 36 + 240 * s["n"] + 4096
               for s in base for spp in s["steps"])
    accs = sum(s["W"] * s["H"] * 32 for s in base)
    tight = int(1.25 * (need + accs))
    lam = util * cap["express"]["sessions_per_s"]
    srv = new_server("express", tight)
    out["server_express_tight_budget"] = serve(srv, [t / lam for t in unit_arr])
    srv.close()
    wf.close()
    out["workload"] = (f"{n_sessions} progressive sessions ({n_req} requests of 8, 8, 16, 32, 64 spp, 128 "
                       "accumulated), scenes from the 1M-sphere distribution (sphere counts log-uniform "
                       "100..1000000, one per session), resolutions {256x256, 512x512, 640x360, 1024x1024}, depth "
                       f"50; Poisson session starts at {int(100 * util)} % of each method's capacity measured at "
                       f"saturation; HBM budget 150 GB (tight run: {tight / 2**30:.2f} GB)")
    return out


def run_reference(args, cfg):
    """The reference arm: the reference's arithmetic on the host cores (the
    oracle's REF_BVH mode), the fixed CPU sample of the configuration per
    step.  It builds its scene and camera with the oracle's own generators and
    loads nothing of the product library.  Under torchrun only rank 0 works."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import pyoracle

    pyoracle.build()
    O = pyoracle.Oracle()
    spheres, cam = oracle_scene(O, cfg)
    nt = os.cpu_count() or 1
    times, segs = [], 0
    for i in range(args.warmup + args.steps):
        rate, dt, s, sample = cpu_run(O, spheres, cam, cfg, args.config, pyoracle.MODE_REF_BVH, nt)
        if i >= args.warmup:
            times.append(dt)
            segs += s
    value = segs / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": cfg["workload"], "cpu_sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port", "arithmetic": "reference",
                         "sample": sample, "what": REF_ARITH},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure_plain(venu, torch, rep, name, cfg, args, steps, warmup, headline):
    """The plain single-scene method on one configuration: autotuned launch
    shapes, `warmup` untimed renders, `steps` renders timed with CUDA events,
    then deterministic replays of the last step for the roofline (events
    around every traversal launch; a counting build for box and sphere tests
    and the traversal loop's SIMD utilisation).  Returns (block, state)."""
    W, H, spp, depth = cfg["W"], cfg["H"], cfg["spp"], cfg["depth"]
    spheres = make_scene(venu, cfg["scene"])
    cam = venu.Camera.look_at(cfg["eye"], (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    stream = torch.cuda.current_stream()
    ds = venu.DeviceScene(spheres)
    tuning, tune_log = None, []
    # Wave size: every path of the render in flight (the renderer takes up
    # to 2^30 paths, ~120 B each: the 1080p x 256 frame is one wave of
    # 530.8 M paths, ~64 GB of queues and slots): fewer waves, fewer tails
    # (measured on RTIOW 1080p x 256: 16 Mi 8.6, 32 Mi 9.8, 64 Mi 10.3,
    # 128 Mi 10.7 G segments/s; later, with the primary rays made in the
    # kernel, 128 Mi 11.07, 256 Mi 11.27; two waves of 2^28 against one
    # 11.94 -> 12.01).
    max_paths = args.max_paths or int(min(MAX_WAVE_PATHS, W * H * spp))
    if args.tuning:
        tuning = json.loads(args.tuning)
    elif not args.no_autotune:
        from venusaur_gb300 import tune

        tuning, _, tune_log = tune.autotune(ds, cam, W, H, spp, depth, max_paths=(max_paths,))
    wf = venu.Wavefront(max_paths)
    if tuning:
        wf.set_tuning(**tuning)
    accum = venu.new_accum(W, H)
    img8 = torch.zeros((H * W, 4), dtype=torch.uint8, device="cuda")

    def step(i):
        wf.render(ds, cam, W, H, spp, accum, subframe=1 + i, max_depth=depth, reset=True, image8=img8)

    for i in range(warmup):
        step(i)
    torch.cuda.synchronize()
    clocks = ClockSampler(rep.local) if headline else None
    if clocks:
        clocks.start()
    rep.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        step(warmup + i)
    e1.record(stream)
    torch.cuda.synchronize()
    rep.barrier()
    clk = clocks.stop() if clocks else None
    # per-step stats are those of the last render; every step renders the
    # same workload (only the seed differs), so counts are per step
    st = wf.stats()
    segs_step = st["segments"]
    # replicas: segments of every rank over the slowest rank's time
    total_segs, secs, value = rep.throughput(segs_step * steps, e0.elapsed_time(e1) / 1000.0)
    ms = 1000.0 * secs

    # --- roofline of the traversal kernel -----------------------------------
    last_sub = 1 + warmup + steps - 1
    acc2 = venu.new_accum(W, H)
    wfp = venu.Wavefront(max_paths, profile=True)
    if tuning:
        wfp.set_tuning(**tuning)
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    wfp.render(ds, cam, W, H, spp, acc2, subframe=last_sub, max_depth=depth, reset=True)
    p1.record(stream)
    torch.cuda.synchronize()
    prof_ms = p0.elapsed_time(p1)
    stp = wfp.stats()
    wfp.close()
    wfc = venu.Wavefront(max_paths, count=True)
    if tuning:
        wfc.set_tuning(**tuning)
    wfc.render(ds, cam, W, H, spp, acc2, subframe=last_sub, max_depth=depth, reset=True)
    torch.cuda.synchronize()
    sc = wfc.stats()
    wfc.close()
    del acc2
    nodes, sph = sc["nodes_visited"], sc["spheres_tested"]
    segs_c, paths_c = sc["segments"], sc["paths"]
    cur = wf.tuning()
    variant = (tuning or {}).get("traverse_variant", cur["traverse_variant"])
    factor = (tuning or {}).get("in_place_factor", cur.get("in_place_factor", 1)) or 1
    # variants 2 and 4 trace and shade in one kernel on every bounce (4 over
    # the 4-wide tree); 3 and 5 only on the primary bounce, then k_traverse
    # (5 over the 4-wide tree); 0 and 1 always run k_traverse
    fused = variant in (2, 4)
    # Algorithmic bytes of the dominant kernel per render, by the per-segment
    # figure: 32 B per node (box) tested + 16 B per sphere tested + the ray
    # state queue traffic: 112 B per segment for the fused traverse+shade
    # kernel (28 B ray write + read -- the depth word also carries the slot
    # of the sphere the ray leaves --, 12 B hit write + read, 16 B
    # throughput/seed/pixel read + write), 40 B for the separate traversal
    # kernel (28 B ray read, 12 B hit write).  The fused kernel makes the
    # primary rays itself from a 4-byte seed per path: 32 B for those
    # segments (4 B seed write + read, 12 B hit, 16 B throughput/seed/pixel
    # write after the bounce).
    trav_bytes = nodes * 32 + sph * 16
    if fused:
        kernel = "k_trace_shade" if variant == 2 else "k_trace_shade_wide"
        kbytes = trav_bytes + paths_c * 32 + (segs_c - paths_c) * 112
    elif variant in (3, 5):  # fused primary bounce, separate traversal after it
        kernel = "k_trace_shade (primary) + k_traverse" + (" (4-wide tree)" if variant == 5 else "")
        kbytes = trav_bytes + paths_c * 32 + (segs_c - paths_c) * 40
    else:
        kernel = "k_traverse"
        kbytes = trav_bytes + segs_c * 40
    nl = max(1, stp["traverse_launches"])
    per_launch_bytes = kbytes / nl
    avg_launch_s = stp["traverse_ms"] / nl / 1000.0
    achieved = per_launch_bytes / avg_launch_s / 1e9
    peak, peak_kind = load_peaks()
    # FP32 view (per-segment estimate): 20 flop per box, 25 per sphere, 60
    # per shade, 30 per camera ray (made in the fused kernel); peak = SMs x
    # 128 FP32 lanes x 2 (FMA) x the highest SM clock seen (else 2070 MHz)
    kflops = nodes * 20 + sph * 25 + (segs_c * 60 + paths_c * 30 if fused else 0)
    sm_mhz = (clk or {}).get("sm_max_mhz") or 2070.0
    fp32_peak = venu.sm_count() * 128 * 2 * sm_mhz * 1e6 / 1e12
    fp32_tflops = kflops / (stp["traverse_ms"] / 1000.0) / 1e12
    simd = sc["lane_steps"] / max(1, 32 * sc["warp_steps"])
    sha = kernel_sources_sha()
    fig_key = f"{name}/v{variant}" + (f"/f{factor}" if fused and factor > 1 else "")
    fig = NCU_FIGURES["figures"].get(fig_key) if NCU_FIGURES["sha"] == sha else None
    traffic = dram_frac = None
    if fig is not None:
        traffic = fig["dram_b_per_seg"] * segs_c / nl
        dram_frac = traffic / avg_launch_s / 1e9 / peak
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "peak_kind": peak_kind, "traffic": traffic, "kernel": kernel,
        "frac_kind": "algorithmic bytes (32 B per box test, 16 B per sphere test, queue traffic) per launch / "
                     "event time; the node set is served from L1/L2, so this is not DRAM throughput",
        "bytes_per_segment": kbytes / max(1, segs_c),
        "nodes_per_segment": nodes / max(1, segs_c), "spheres_per_segment": sph / max(1, segs_c),
        "simd_utilization": simd,
        "simd_utilization_kind": "traversal steps summed over lanes / (32 x steps issued per warp), counting "
                                 "build of the same render (live)",
        "dram_bytes_per_segment": fig["dram_b_per_seg"] if fig else None,
        "dram_frac": dram_frac,
        "lanes_per_inst_ncu": fig["lanes_per_inst"] if fig else None,
        "warp_inst_per_segment_ncu": fig["warp_inst_per_seg"] if fig else None,
        "ncu_kernel_sources_sha": NCU_FIGURES["sha"], "ncu_commit": NCU_FIGURES["commit"],
        "kernel_sources_sha": sha,
        "ncu_figures_key": fig_key,
        "ncu_note": None if fig else ("no ncu figures for these kernel sources and this variant: traffic, "
                                      "dram_frac and lanes_per_inst_ncu are null"),
        # the kernel's launches over the whole profiled render (the same
        # render with an event pair around every launch)
        "kernel_share": stp["traverse_ms"] / max(1e-9, prof_ms),
        "profiled_render_ms": prof_ms,
        "fp32_tflops": fp32_tflops, "fp32_peak_tflops": fp32_peak, "fp32_frac": fp32_tflops / fp32_peak,
    }
    block = {
        "workload": cfg["workload"], "value": value, "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
        "warmup": warmup, "segments_per_step": segs_step, "paths_per_step": st["paths"],
        "spheres": int(len(spheres)), "width": W, "height": H, "spp": spp, "max_depth": depth,
        "tuning": dict(wf.tuning(), max_paths=max_paths), "autotune_candidates": len(tune_log),
        "lbvh": {"build_ms": ds.info()["build_ms"], "device_bytes": ds.info()["device_bytes"]},
        "gpu_launches": st["kernel_launches"] * steps,
        "roofline": roofline,
    }
    state = dict(wf=wf, ds=ds, spheres=spheres, cam=cam, accum=accum, img8=img8, tuning=tuning,
                 max_paths=max_paths, segs_step=segs_step, total_segs=total_segs, clocks=clk, stream=stream)
    return block, state


def measure_e2e(venu, torch, rep, cfg, state, steps):
    """The headline metric through the C ABI from pinned host memory: scene
    upload + LBVH build + render + image download every step."""
    import ctypes as C

    from venusaur_gb300._lib import RenderOpts, check, lib, ptr

    W, H, spp, depth = cfg["W"], cfg["H"], cfg["spp"], cfg["depth"]
    spheres, cam, accum, img8 = state["spheres"], state["cam"], state["accum"], state["img8"]
    host_sph = torch.from_numpy(spheres.view(np.uint8)).pin_memory()
    host_img = torch.empty((H * W, 4), dtype=torch.uint8).pin_memory()
    wf_plain = venu.Wavefront(state["max_paths"])
    if state["tuning"]:
        wf_plain.set_tuning(**state["tuning"])
    cam_np = np.ascontiguousarray(cam)
    h = C.c_void_p(state["stream"].cuda_stream)

    def e2e_step(i):
        sc_h = C.c_void_p()
        check(lib().venu_scene_create(ptr(host_sph), len(spheres), h, C.byref(sc_h)))
        o = RenderOpts(W, H, spp, 1 + i, depth, 1)
        check(lib().venu_render(wf_plain.handle, sc_h, ptr(cam_np), C.byref(o), ptr(accum), None, ptr(img8), h))
        host_img.copy_(img8, non_blocking=True)
        torch.cuda.synchronize()
        lib().venu_scene_destroy(sc_h)

    e2e_step(0)
    rep.barrier()
    t0 = time.perf_counter()
    for i in range(steps):
        e2e_step(i + 1)
    t1 = time.perf_counter()
    e2e_s = rep.max(t1 - t0)
    wf_plain.close()
    return {"value": state["total_segs"] / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(spheres.nbytes),
            "d2h_bytes_per_step": int(H * W * 4), "ms_per_step": 1000 * e2e_s / steps}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="venu", choices=["venu", "reference"])
    ap.add_argument("--config", default="c2", choices=sorted(CONFIGS))
    ap.add_argument("--max-paths", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0, help="override the config's samples per pixel (small profiling cases)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default launch shapes")
    ap.add_argument("--tuning", default="", help="JSON launch shapes to use instead of the autotuner's")
    ap.add_argument("--profile-mixed", type=int, default=0, metavar="STEPS",
                    help="only run STEPS loop steps of the first 12 jobs of the mixed workload (~4 GB on the "
                         "device) through the batch engine's host-driven loop (ncu cannot profile kernels "
                         "inside conditional graphs) and exit")
    ap.add_argument("--no-batched", action="store_true", help="skip the mixed-scene batched/plain comparison")
    ap.add_argument("--profile-render", action="store_true",
                    help="only render the configuration once (after one warm-up render) with the launch shapes of "
                         "--tuning (default: variant 2, 128-thread blocks) and print its segment count: the "
                         "case the ncu figures of the roofline are taken on")
    ap.add_argument("--no-configs", action="store_true", help="skip the other configurations' blocks")
    args = ap.parse_args()
    cfg = dict(CONFIGS[args.config])
    if args.spp:
        cfg["spp"] = args.spp
        cfg["workload"] = cfg["workload"].replace(f"{CONFIGS[args.config]['spp']} spp", f"{args.spp} spp")
    if args.impl == "reference":
        run_reference(args, cfg)
        return
    from venusaur_gb300.replicas import Replicas

    rep = Replicas()
    world, rank, local = rep.world, rep.rank, rep.local

    import torch

    torch.cuda.set_device(local)
    import venusaur_gb300 as venu
    from venusaur_gb300 import build as vb

    vb.build()
    if args.profile_mixed:
        profile_mixed(venu, torch, args)
        return
    if args.profile_render:
        profile_render(venu, torch, cfg, args)
        return
    # CPU baseline first, on an idle host (rank 0, single process only): the
    # reference's arithmetic on the fixed sample of this configuration, every
    # host thread; the GB300-arithmetic port on the same sample beside it.
    cpu_baseline = cpu_gb300 = None
    O = None
    if not args.no_cpu and world == 1:
        from oracle import pyoracle

        pyoracle.build()
        O = pyoracle.Oracle()
        nt = os.cpu_count() or 1
        o_sph, o_cam = oracle_scene(O, cfg)
        cpu_run(O, o_sph, o_cam, CONFIGS["c1"], "c1", pyoracle.MODE_REF_BVH, nt)  # thread start-up, page-in
        rate, dt, segs, sample = cpu_run(O, o_sph, o_cam, cfg, args.config, pyoracle.MODE_REF_BVH, nt, repeats=3)
        cpu_baseline = {"value": rate, "unit": UNIT, "cores": nt, "kind": "port", "arithmetic": "reference",
                        "sample": sample + " (3 runs)", "seconds": dt, "what": REF_ARITH}
        rate, dt, segs, sample = cpu_run(O, o_sph, o_cam, cfg, args.config, pyoracle.MODE_GB300, nt)
        cpu_gb300 = {"value": rate, "unit": UNIT, "cores": nt, "kind": "port", "arithmetic": "gb300",
                     "sample": sample, "seconds": dt,
                     "what": "the oracle's restatement of this library's own arithmetic over the same LBVH"}

    steps, warmup = args.steps, args.warmup
    block, state = measure_plain(venu, torch, rep, args.config, cfg, args, steps, warmup, headline=True)
    state["wf"].close()  # its queues (~64 GB for the headline) before the next renderer takes its own
    e2e = measure_e2e(venu, torch, rep, cfg, state, steps)
    others = {}
    if not args.no_configs and world == 1:
        for name in ("c1", "c2", "c3"):
            if name == args.config:
                continue
            if name == "c2" and args.config != "c2":
                continue  # the headline's own config only as headline
            b, st2 = measure_plain(venu, torch, rep, name, dict(CONFIGS[name]), args, min(steps, 5), 3,
                                   headline=False)
            st2["wf"].close()
            others[name] = b
            del st2
            torch.cuda.empty_cache()

    if rank != 0:
        return
    W, H = cfg["W"], cfg["H"]
    line = {
        "metric": METRIC, "value": block["value"], "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": block["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded RTIOW scene generator)",
        "config": {"workload": cfg["workload"], "width": W, "height": H, "spp": cfg["spp"],
                   "max_depth": cfg["depth"], "spheres": block["spheres"], "method": "plain single-scene wavefront",
                   "l2": "working set (ray queues > 1.5 GB) larger than L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "segments_per_step": block["segments_per_step"], "paths_per_step": block["paths_per_step"],
                   "tuning": block["tuning"], "autotune_candidates": block["autotune_candidates"],
                   "lbvh": block["lbvh"]},
        "gpu_launches": block["gpu_launches"],
        "clocks": state["clocks"],
        "e2e": e2e,
        "roofline": block["roofline"],
    }
    if others:
        line["configs"] = others
    if not args.no_batched and world == 1:
        ds, cam, tuning = state["ds"], state["cam"], state["tuning"]
        line["batched_single_job"] = run_single_job(venu, torch, tuning, ds, cam, W, H, cfg["spp"], cfg["depth"],
                                                    state["segs_step"], warmup + steps,
                                                    min(state["max_paths"], 256 << 20))
        retune = not (args.tuning or args.no_autotune)
        line["batched"] = run_batched(venu, torch, tuning, state["max_paths"], autotune=retune)
        line["batched_small_jobs"] = run_batched(venu, torch, tuning, state["max_paths"], small=True,
                                                 autotune=retune)
        line["served"] = run_served(venu, torch, tuning)
    if cpu_baseline is not None:
        line["cpu_baseline"] = cpu_baseline
        line["cpu_port_gb300"] = cpu_gb300
        line["rmse_vs_reference"] = rmse_vs_reference(venu, torch, O, state["ds"], state["spheres"], state["cam"],
                                                      W, H, cfg["depth"])
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
