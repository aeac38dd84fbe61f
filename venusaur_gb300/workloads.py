"""Seeded synthetic workloads for the batched and served measurements.

mixed_jobs(): independent scenes with sphere counts log-uniform in
[100, 200 000] (ground sphere + random spheres in a 200x20x200 box, the
random-scene generator), resolutions uniform from {256x256, 512x512,
640x360, 1024x1024}, samples per pixel uniform from {4, 16, 64}, depth 50,
camera at (60, 15, 60) looking at the origin (vfov 20, aperture 0.1, focus 10).

serving_jobs(): the same scene/resolution distribution with spp uniform from
{8, 16, 32, 64, 128} and Poisson arrival times.

serving_sessions(): progressive render sessions, each on its own scene drawn
from the 1M-sphere scene's distribution (the same generator, sphere counts
log-uniform in [100, 1 000 000]), one of the four resolutions, and five
requests of 8, 8, 16, 32 and 64 samples per pixel (8 to 128 accumulated),
each submitted when the previous one's image is back; sessions start with
Poisson arrivals.
"""
from __future__ import annotations

import math

import numpy as np

RESOLUTIONS = ((256, 256), (512, 512), (640, 360), (1024, 1024))
SPP_MIXED = (4, 16, 64)
SPP_SERVING = (8, 16, 32, 64, 128)
EYE = (60.0, 15.0, 60.0)


def _draw(rng, spp_set, nmin, nmax):
    n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
    W, H = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
    spp = int(spp_set[int(rng.integers(len(spp_set)))])
    return n, W, H, spp


def mixed_jobs(n_jobs: int = 64, seed: int = 0, nmin: int = 100, nmax: int = 200_000, depth: int = 50):
    rng = np.random.default_rng(seed)
    jobs = []
    for i in range(n_jobs):
        n, W, H, spp = _draw(rng, SPP_MIXED, nmin, nmax)
        jobs.append(dict(n=n, scene_seed=1000 + i, W=W, H=H, spp=spp, depth=depth, eye=EYE, subframe=1))
    return jobs


def serving_jobs(n_jobs: int, rate_per_s: float, seed: int = 1, nmin: int = 100, nmax: int = 200_000,
                 depth: int = 50, n_scenes: int = 16):
    """Requests with Poisson arrivals; scenes drawn from a pool of n_scenes so
    that resident BVHs are reused across requests."""
    rng = np.random.default_rng(seed)
    scene_pool = []
    for k in range(n_scenes):
        n, *_ = _draw(rng, SPP_SERVING, nmin, nmax)
        scene_pool.append(dict(n=n, scene_seed=5000 + k))
    t = 0.0
    jobs = []
    for i in range(n_jobs):
        t += float(rng.exponential(1.0 / rate_per_s))
        _, W, H, spp = _draw(rng, SPP_SERVING, nmin, nmax)
        sc = scene_pool[int(rng.integers(n_scenes))]
        jobs.append(dict(n=sc["n"], scene_seed=sc["scene_seed"], W=W, H=H, spp=spp, depth=depth, eye=EYE,
                         subframe=1, arrival=t))
    return jobs


def small_jobs(n_jobs: int = 128, W: int = 256, H: int = 144, spp: int = 4, depth: int = 50):
    """Many small renders of RTIOW scenes (seeds 0..n_jobs-1): the regime where
    one render per launch sequence leaves the GPU mostly idle."""
    return [dict(rtiow_seed=i, W=W, H=H, spp=spp, depth=depth, eye=(13.0, 2.0, 3.0), subframe=1)
            for i in range(n_jobs)]


def paths(jobs) -> int:
    return sum(j["W"] * j["H"] * j["spp"] for j in jobs)


SESSION_STEPS = (8, 8, 16, 32, 64)  # samples per request; 8, 16, 32, 64, 128 accumulated


def serving_sessions(n_sessions: int, rate_per_s: float = 0.0, seed: int = 5, nmin: int = 100,
                     nmax: int = 1_000_000, depth: int = 50):
    """Sessions with their start times.  The sessions themselves (scene,
    resolution) depend only on `seed`; the start times are the same unit
    Poisson draws scaled by 1 / rate_per_s (all at 0 when the rate is 0),
    so one set of sessions can be offered at several rates."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_sessions):
        n, W, H, _ = _draw(rng, SPP_SERVING, nmin, nmax)
        out.append(dict(n=n, scene_seed=7000 + i, W=W, H=H, steps=SESSION_STEPS, depth=depth, eye=EYE))
    gaps = np.random.default_rng(seed + 1).exponential(1.0, size=n_sessions)
    t = np.cumsum(gaps) - gaps[0]
    for s, ti in zip(out, t):
        s["arrival"] = float(ti / rate_per_s) if rate_per_s > 0 else 0.0
    return out


def session_paths(sessions) -> int:
    return sum(s["W"] * s["H"] * sum(s["steps"]) for s in sessions)
