"""The device arithmetic that results depend on bit for bit, word for word
against the host: the TEA-4 / LCG stream against the golden vectors made from
the reference's own Core/random.cuh, and the sRGB power routine against the
oracle's restatement on every input of the sRGB branch (with CUDA's powf
measured beside it)."""
import ctypes as C
import os

import numpy as np
import pytest

from test_oracle import srgb_pow_inputs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden.npz")


@pytest.mark.gpu
def test_device_rng_matches_reference_golden(venu, cuda):
    import torch

    from venusaur_gb300._lib import check, lib, ptr

    g = np.load(GOLDEN)
    pairs = g["rng_pairs"].astype(np.uint32)
    a = torch.from_numpy(np.ascontiguousarray(pairs[:, 0]).view(np.int32)).cuda()
    b = torch.from_numpy(np.ascontiguousarray(pairs[:, 1]).view(np.int32)).cuda()
    tea = torch.zeros(len(pairs), dtype=torch.int32, device="cuda")
    n = len(g["rng_states"])
    vals = torch.zeros(n, dtype=torch.float32, device="cuda")
    states = torch.zeros(n, dtype=torch.int32, device="cuda")
    # the golden stream starts from tea<4>(0, 1), itself computed on the device
    tmp = torch.zeros(1, dtype=torch.int32, device="cuda")
    z = torch.zeros(1, dtype=torch.int32, device="cuda")
    one = torch.ones(1, dtype=torch.int32, device="cuda")
    check(lib().venu_selftest_rng(ptr(z), ptr(one), 1, ptr(tmp), 0, 0, None, None, None))
    torch.cuda.synchronize()
    seed = int(tmp.cpu().numpy().view(np.uint32)[0])
    check(lib().venu_selftest_rng(ptr(a), ptr(b), len(pairs), ptr(tea), seed, n, ptr(vals), ptr(states), None))
    torch.cuda.synchronize()
    assert np.array_equal(tea.cpu().numpy().view(np.uint32), g["rng_tea4"])
    assert np.array_equal(vals.cpu().numpy().view(np.uint32), g["rng_rnd"].view(np.uint32))
    assert np.array_equal(states.cpu().numpy().view(np.uint32), g["rng_states"])


@pytest.mark.gpu
def test_device_srgb_pow_matches_host_everywhere(venu, oracle, cuda):
    import torch

    from venusaur_gb300._lib import check, lib, ptr

    x = srgb_pow_inputs()
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    check(lib().venu_selftest_srgb_pow(ptr(xd), C.c_uint64(len(x)), 0, ptr(out), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    want = oracle.srgb_pow(x)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # CUDA's powf on the same inputs, for the record: the routine is at
    # least as accurate
    check(lib().venu_selftest_srgb_pow(ptr(xd), C.c_uint64(len(x)), 1, ptr(out), None))
    torch.cuda.synchronize()
    pw = out.cpu().numpy().astype(np.float64)
    ref = np.power(x.astype(np.float64), np.float64(np.float32(1.0) / np.float32(2.4)))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    mine = float((np.abs(got.astype(np.float64) - ref) / ulp).max())
    theirs = float((np.abs(pw - ref) / ulp).max())
    print(f"max error over [0.0031308, 1]: srgb_pow {mine:.3f} ulp, powf {theirs:.3f} ulp")
    assert mine <= 1.2
