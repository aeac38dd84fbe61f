"""CPU tests: the oracle against the reference's own code and golden vectors.

The oracle (oracle/venu_oracle.cpp) is pinned two ways:
  * against tests/golden/golden.npz, made from the reference's Core/random.cuh
    and Core/RayTracer.cu compiled for the host (tests/golden/make_golden.py);
  * live against that same reference build (oracle/_ref) where it exists.
"""
import os

import numpy as np
import pytest

from oracle import pyoracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


def _scene_cam(g):
    spheres = g["scene"].reshape(-1).view(pyoracle.SPHERE_DTYPE)
    cam = g["camera"].view(pyoracle.CAMERA_DTYPE)
    W, H, SPP = (int(x) for x in g["wh_spp"])
    return spheres, cam, W, H, SPP


def test_rng_known_answers(oracle, g):
    for (a, b), want in zip(g["rng_pairs"], g["rng_tea4"]):
        assert oracle.tea4(int(a), int(b)) == int(want)
    vals, states = oracle.rnd_stream(oracle.tea4(0, 1), 256)
    assert np.array_equal(vals.view(np.uint32), g["rng_rnd"].view(np.uint32))
    assert np.array_equal(states, g["rng_states"])
    # the value quoted for tea<4>(0,1) then rnd: LCG state 3617041482, 0.592472672
    assert int(states[0]) == 3617041482
    assert abs(float(vals[0]) - 0.592472672) < 1e-9


def test_ref_mode_matches_reference_golden(oracle, g):
    spheres, cam, W, H, SPP = _scene_cam(g)
    r = oracle.render(spheres, cam, W, H, SPP, subframe=0, max_depth=4, mode=pyoracle.MODE_REF)
    assert np.array_equal(r["accum"].view(np.uint32), g["ref_s0_accum"].view(np.uint32))
    assert np.abs(r["image8"].astype(int) - g["ref_s0_image8"].astype(int)).max() <= 1
    # progressive subframe: lerp with the previous accumulation buffer
    r3 = oracle.render(spheres, cam, W, H, 2, subframe=3, max_depth=4, mode=pyoracle.MODE_REF,
                       accum=g["ref_s3_prior"].copy())
    assert np.array_equal(r3["accum"].view(np.uint32), g["ref_s3_accum"].view(np.uint32))


def test_ref_bvh_mode_matches_reference_golden(oracle, g):
    """The reference's arithmetic with the closest hit found through the host
    LBVH (the timed CPU baseline) equals the brute force, and so the
    reference's own RayTracer.cu built for the host, bit for bit."""
    spheres, cam, W, H, SPP = _scene_cam(g)
    r = oracle.render(spheres, cam, W, H, SPP, subframe=0, max_depth=4, mode=pyoracle.MODE_REF_BVH)
    assert np.array_equal(r["accum"].view(np.uint32), g["ref_s0_accum"].view(np.uint32))
    r3 = oracle.render(spheres, cam, W, H, 2, subframe=3, max_depth=4, mode=pyoracle.MODE_REF_BVH,
                       accum=g["ref_s3_prior"].copy())
    assert np.array_equal(r3["accum"].view(np.uint32), g["ref_s3_accum"].view(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 3000])
def test_ref_bvh_mode_matches_brute_force(oracle, n):
    sp = oracle.scene_random(n, 7)
    W, H = 48, 27
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    a = oracle.render(sp, cam, W, H, 3, subframe=1, max_depth=50, mode=pyoracle.MODE_REF)
    b = oracle.render(sp, cam, W, H, 3, subframe=1, max_depth=50, mode=pyoracle.MODE_REF_BVH)
    assert a["segments"] == b["segments"]
    assert np.array_equal(a["accum"].view(np.uint32), b["accum"].view(np.uint32))
    if n > 2:
        assert b["spheres"] < a["segments"] * n // 10  # the LBVH prunes


def test_gb300_mode_golden(oracle, g):
    spheres, cam, W, H, SPP = _scene_cam(g)
    for depth in (4, 50):
        r = oracle.render(spheres, cam, W, H, SPP, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
        assert np.array_equal(r["accum"].view(np.uint32), g[f"gb_d{depth}_accum"].view(np.uint32))
        assert r["segments"] == int(g[f"gb_d{depth}_segments"][0])


def test_lbvh_golden(oracle, g):
    spheres, *_ = _scene_cam(g)
    b = oracle.lbvh(spheres)
    assert np.array_equal(b["keys"], g["bvh_keys"])
    assert np.array_equal(b["ids"], g["bvh_ids"])
    assert b["nodes"].view(np.uint8).tobytes() == g["bvh_nodes"].tobytes()


@pytest.mark.skipif(not pyoracle.RefBuild.available(), reason="reference build (oracle/_ref) not present")
def test_ref_mode_matches_reference_live(oracle):
    R = pyoracle.RefBuild()
    spheres = oracle.scene_rtiow(3)
    for (W, H, spp, sub) in ((40, 30, 3, 0), (17, 9, 5, 2)):
        cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
        prior = np.random.default_rng(W).random((W * H, 4)).astype(np.float32)
        a = oracle.render(spheres, cam, W, H, spp, subframe=sub, max_depth=4, mode=pyoracle.MODE_REF,
                          accum=prior.copy())
        b = R.render(spheres, cam, W, H, spp, subframe=sub, accum=prior.copy())
        assert np.array_equal(a["accum"].view(np.uint32), b["accum"].view(np.uint32))


def test_lbvh_structure(oracle):
    """Karras invariants: every slot is reached once; boxes contain children."""
    for n in (2, 3, 7, 100, 2000):
        sp = oracle.scene_random(n, 11) if n > 2 else oracle.scene_rtiow(0)[:n]
        b = oracle.lbvh(sp)
        keys, nodes = b["keys"], b["nodes"]
        assert np.all(np.diff(keys.astype(np.int64)) >= 0)
        assert sorted(b["ids"].tolist()) == list(range(n))
        seen_leaf, seen_int = set(), {0}
        stack = [0]
        while stack:
            i = stack.pop()
            for c in (int(nodes[i]["left"]), int(nodes[i]["right"])):
                if c < 0:
                    seen_leaf.add(c & 0x3FFFFFFF)  # bit 30 marks a hoisted leaf
                    k = c & 0x3FFFFFFF
                    s = sp[b["ids"][k]]
                    assert np.all(nodes[i]["lo"] <= s["center"] - abs(s["radius"]))
                    assert np.all(nodes[i]["hi"] >= s["center"] + abs(s["radius"]))
                else:
                    seen_int.add(c)
                    stack.append(c)
                    assert np.all(nodes[i]["lo"] <= nodes[c]["lo"])
                    assert np.all(nodes[i]["hi"] >= nodes[c]["hi"])
        assert seen_leaf == set(range(n)) and seen_int == set(range(n - 1))


def test_duplicate_keys_tiebreak(oracle):
    """Spheres sharing a Morton code keep index order (stable sort)."""
    sp = oracle.scene_random(64, 5)
    sp["center"][10:40] = sp["center"][10]
    b = oracle.lbvh(sp)
    same = [i for i in b["ids"] if 10 <= i < 40]
    assert same == sorted(same)


def test_bvh_traversal_matches_brute_force(oracle):
    """FP32 LBVH closest hit vs FP32/FP64 brute force on random rays."""
    rng = np.random.default_rng(1)
    sp = oracle.scene_rtiow(0)
    n = 20000
    o = np.stack([rng.uniform(-12, 14, n), rng.uniform(0.01, 4, n), rng.uniform(-12, 12, n)], 1)
    d = rng.normal(size=(n, 3))
    rays = np.concatenate([o, d], 1).astype(np.float32)
    idb, tb, front, nv, ns = oracle.trace_bvh(sp, rays)
    id64, t64, disc, t2 = oracle.trace_fp64(sp, rays)
    well = (id64 >= 0) & (disc > 1e-4) & (t2 > t64 * (1 + 1e-4))
    assert (idb == id64)[well].all()
    rel = np.abs(tb[well].astype(np.float64) - t64[well]) / t64[well]
    assert rel.max() < 1e-5, rel.max()
    assert ((idb == -1) == (id64 == -1)).mean() > 0.999


def _axis_rays(n, seed):
    """Rays inside a random-sphere field whose directions have one or two
    components exactly zero or tiny (down to 1e-30): the near-axis-parallel
    rays the slab test must cull as well as any other."""
    rng = np.random.default_rng(seed)
    o = np.stack([rng.uniform(-90, 90, n), rng.uniform(0.5, 19.5, n), rng.uniform(-90, 90, n)], 1)
    d = rng.normal(size=(n, 3))
    tiny = np.array([0.0, -0.0, 1e-30, -1e-12, 1e-9, 3e-7, -2e-6])
    for i in range(n):
        for a in rng.choice(3, size=1 + i % 2, replace=False):
            d[i, a] = tiny[(i // 2) % len(tiny)]
    return np.concatenate([o, d], 1).astype(np.float32)


def test_near_axis_parallel_rays(oracle):
    """A direction component at or near zero gives 1/d up to 1e20; its slab
    rounding margin must not switch off the culling on the other two axes
    (with one margin shared by all axes such a ray visited every node its
    slab met: tens of thousands in a 50k-sphere field)."""
    sp = oracle.scene_random(50_000, 6)
    rays = _axis_rays(4000, 3)
    idb, tb, front, nv, ns = oracle.trace_bvh(sp, rays)
    ok = oracle.trace_bvh(sp, _random_rays_like(rays, 4))[3]
    assert nv.max() < 8 * max(ok.max(), 1), (nv.max(), ok.max())
    assert nv.mean() < 3 * ok.mean()
    id64, t64, disc, t2 = oracle.trace_fp64(sp, rays)
    well = (id64 >= 0) & (disc > 1e-4) & (t2 > t64 * (1 + 1e-4))
    assert well.sum() > 1000
    assert (idb == id64)[well].all()
    rel = np.abs(tb[well].astype(np.float64) - t64[well]) / t64[well]
    assert rel.max() < 1e-5, rel.max()
    assert ((idb == -1) == (id64 == -1)).mean() > 0.999


def _random_rays_like(rays, seed):
    d = np.random.default_rng(seed).normal(size=(len(rays), 3)).astype(np.float32)
    return np.concatenate([rays[:, :3], d], 1).astype(np.float32)


def test_gb300_vs_ref_same_paths(oracle):
    """The GB300 arithmetic and the reference arithmetic trace the same paths:
    at the same seeds > 99% of samples agree within 1e-3, and the
    image RMSE is far below the seed-to-seed noise.  (subframe 0: the
    reference lerps subframe k > 0 with the previous buffer.)"""
    sp = oracle.scene_rtiow(0)
    W, H = 32, 18
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    a = oracle.render(sp, cam, W, H, 16, subframe=0, max_depth=4, mode=pyoracle.MODE_GB300, want_samples=True)
    b = oracle.render(sp, cam, W, H, 16, subframe=0, max_depth=4, mode=pyoracle.MODE_REF, want_samples=True)
    err = np.abs(a["samples"] - b["samples"]).max(axis=2)
    assert (err <= 1e-3).mean() > 0.99, (err <= 1e-3).mean()
    rmse = np.sqrt(((a["image_f"][:, :3] - b["accum"][:, :3]) ** 2).mean())
    c = oracle.render(sp, cam, W, H, 16, subframe=0, max_depth=4, mode=pyoracle.MODE_REF)
    d = oracle.render(sp, cam, W, H, 16, subframe=5, max_depth=4, mode=pyoracle.MODE_GB300)
    noise = np.sqrt(((d["image_f"][:, :3] - c["accum"][:, :3]) ** 2).mean())
    assert rmse < 0.25 * noise, (rmse, noise)


def test_scene_generators_match_product(oracle, venu):
    a = venu.generate_rtiow(0)
    assert a.tobytes() == oracle.scene_rtiow(0).tobytes()
    assert len(a) == 485
    b = venu.generate_random(5000, 9)
    assert b.tobytes() == oracle.scene_random(5000, 9).tobytes()
    assert b["radius"][1:].min() >= 0.01 and b["radius"][1:].max() <= 0.5
    frac = np.bincount(b["material"][1:], minlength=3) / (len(b) - 1)
    assert abs(frac[0] - 0.8) < 0.03 and abs(frac[1] - 0.15) < 0.03


def test_camera_matches_product(oracle, venu):
    for args in (((13, 2, 3), (0, 0, 0), 20.0, 16 / 9, 0.1, 10.0), ((60, 15, 60), (0, 0, 0), 20.0, 1.0, 0.1, 10.0)):
        assert venu.Camera.look_at(*args).tobytes() == oracle.camera(*args).tobytes()


def _moved(spheres, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    out = spheres.copy()
    for a in range(3):
        out["center"][1:, a] += (rng.normal(size=len(out) - 1) * scale).astype(np.float32)
    out["radius"][1:] *= rng.uniform(0.5, 1.5, size=len(out) - 1).astype(np.float32)
    return out


def test_refit_identity_and_moved(oracle):
    """Refit to the same spheres reproduces the build; after moving the
    spheres the refit tree still bounds every sphere, and rendering through
    it gives the same image as a fresh build (closest hit does not depend on
    the tree, ties aside)."""
    sp = oracle.scene_random(3000, 21)
    built = oracle.lbvh(sp)
    assert np.array_equal(oracle.lbvh_refit(sp, sp).view(np.uint32), built["nodes"].view(np.uint32))
    mv = _moved(sp, 5, scale=3.0)
    nodes = oracle.lbvh_refit(sp, mv)
    ids = built["ids"]
    # every leaf box inside its parent's box, children boxes inside parents
    lo, hi = nodes["lo"], nodes["hi"]
    for i, nd in enumerate(nodes):
        for c in (int(nd["left"]), int(nd["right"])):
            if c & 0x80000000:
                k = c & 0x3FFFFFFF
                s = mv[ids[k]]
                r = abs(float(s["radius"]))
                assert np.all(lo[i] <= s["center"] - r) and np.all(hi[i] >= s["center"] + r)
            else:
                assert np.all(lo[i] <= lo[c]) and np.all(hi[i] >= hi[c])
    cam = oracle.camera((60, 15, 60), (0, 0, 0), 20.0, 1.5, 0.1, 10.0)
    a = oracle.render(mv, cam, 36, 24, 2, subframe=3, max_depth=8, built_from=sp)
    b = oracle.render(mv, cam, 36, 24, 2, subframe=3, max_depth=8)
    assert np.array_equal(a["accum"].view(np.uint32), b["accum"].view(np.uint32))
    assert a["segments"] == b["segments"]


def test_invariant_division_magic():
    """The kernels divide path and pixel indices (< 2^31) by per-wave
    constants (1..2^30) as a multiply and a shift (Granlund & Montgomery,
    N = 31): l = ceil(log2 d), m = floor(2^(31+l)/d) + 1 < 2^32,
    x / d = (x m) >> (31 + l).  Exact for every divisor tried at its
    boundary dividends."""
    rng = np.random.default_rng(2)
    ds = list(range(1, 3000)) + [1 << k for k in range(31)] + [(1 << k) + j for k in range(2, 31) for j in (-1, 1)]
    ds += [int(x) for x in rng.integers(1, (1 << 30) + 1, 3000)] + [1920, 2073600, 147456, 1 << 30]
    for d in ds:
        if not 1 <= d <= 1 << 30:
            continue
        l = (d - 1).bit_length()
        m = (1 << (31 + l)) // d + 1
        assert m < 1 << 32
        top = (1 << 31) - 1
        for x in [0, 1, d - 1, d, d + 1, top, top - 1, top // d * d, top // d * d - 1] + \
                 [int(v) for v in rng.integers(0, 1 << 31, 8)]:
            if 0 <= x <= top:
                assert (x * m) >> (31 + l) == x // d, (x, d)


def srgb_pow_inputs(stride=1):
    """Every float in [0.0031308, 1] (the sRGB power's inputs), every
    `stride`-th one."""
    lo = int(np.float32(0.0031308).view(np.uint32))
    hi = int(np.float32(1.0).view(np.uint32))
    return np.arange(lo, hi + 1, stride, dtype=np.uint32).view(np.float32)


def test_srgb_pow_accuracy(oracle):
    """The GB300 arithmetic's x^(1/2.4) (oracle restatement of the kernels'
    routine) against double-precision pow on every input of the sRGB branch:
    within 1.2 ulp of the exact value."""
    x = srgb_pow_inputs()
    y = np.float64(np.float32(1.0) / np.float32(2.4))
    worst = 0.0
    for k in range(0, len(x), 1 << 23):
        xs = x[k:k + (1 << 23)]
        got = oracle.srgb_pow(xs).astype(np.float64)
        ref = np.power(xs.astype(np.float64), y)
        worst = max(worst, float((np.abs(got - ref) / np.spacing(ref.astype(np.float32))).max()))
    assert worst <= 1.2, worst
    assert oracle.srgb_pow(np.array([1.0], np.float32))[0] == 1.0


def test_srgb_bytes_gb300_vs_pow(oracle):
    """The GB300 encode differs from the pow() encode only where the value
    sits on a byte boundary: at most 1 apart, and rarely."""
    rgb = np.random.default_rng(3).random((200_000, 3)).astype(np.float32)
    a = oracle.make_color(rgb).astype(int)
    b = oracle.make_color_gb300(rgb).astype(int)
    assert np.abs(a - b).max() <= 1 and (a != b).mean() < 1e-3
