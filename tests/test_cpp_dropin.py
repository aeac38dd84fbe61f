"""The C++17 drop-in (include/venu_core.hpp): a headless version of the
reference's main loop (tests/cpp/render_main.cpp) builds against the header
and the library (CPU), and on a GPU renders the same bytes as the oracle."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "render_main.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_exe(tmp_path, venu):
    from venusaur_gb300._lib import LIB_PATH

    exe = str(tmp_path / "render_main")
    libdir = os.path.dirname(LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           SRC, "-o", exe, "-L", libdir, "-lvenusaur_gb300", f"-Wl,-rpath,{libdir}",
           "-L", os.path.join(CUDA, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_dropin_builds(tmp_path, venu):
    assert os.path.exists(build_exe(tmp_path, venu))


@pytest.mark.gpu
def test_cpp_dropin_renders(tmp_path, venu, oracle, cuda):
    from oracle import pyoracle

    exe = build_exe(tmp_path, venu)
    # the reference's Renderer: 16 samples per pixel per Draw, depth 4
    W, H, spp, depth = 48, 30, 16, 4
    ppm, raw, pfm = str(tmp_path / "o.ppm"), str(tmp_path / "o.rgba"), str(tmp_path / "o.pfm")
    r = subprocess.run([exe, str(W), str(H), "2", ppm, raw, pfm], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(raw, np.uint8).reshape(-1, 4)
    sp = oracle.scene_rtiow(0)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    a = oracle.render(sp, cam, W, H, spp, subframe=1, max_depth=depth, mode=pyoracle.MODE_GB300)
    b = oracle.render(sp, cam, W, H, spp, subframe=2, max_depth=depth, mode=pyoracle.MODE_GB300, accum=a["accum"])
    assert np.array_equal(got, b["image8"])
    assert open(ppm, "rb").read(2) == b"P6"
    head = f"PF\n{W} {H}\n-1.0\n".encode()
    data = open(pfm, "rb").read()
    assert data[: len(head)] == head and len(data) == len(head) + W * H * 12


def test_cpp_gl_buffer_types_rejected(tmp_path, venu):
    """CUDAOutputBuffer<uchar4>(GL_INTEROP, ...) throws venu_core::Exception
    (VENU_ERR_INVALID) before touching the GPU: there is no GL display."""
    exe = build_exe(tmp_path, venu)
    r = subprocess.run([exe, "gl"], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)


@pytest.mark.gpu
def test_cpp_dropin_zero_copy(tmp_path, venu, oracle, cuda):
    """The ZERO_COPY buffer type: the kernels write the pixels into mapped
    host memory; the bytes equal the CUDA_DEVICE path's (the oracle's)."""
    from oracle import pyoracle

    exe = build_exe(tmp_path, venu)
    W, H = 40, 24
    ppm, raw, pfm = str(tmp_path / "z.ppm"), str(tmp_path / "z.rgba"), str(tmp_path / "z.pfm")
    r = subprocess.run([exe, str(W), str(H), "2", ppm, raw, pfm, "zero_copy"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(raw, np.uint8).reshape(-1, 4)
    sp = oracle.scene_rtiow(0)
    cam = oracle.camera((13, 2, 3), (0, 0, 0), 20.0, W / H, 0.1, 10.0)
    a = oracle.render(sp, cam, W, H, 16, subframe=1, max_depth=4, mode=pyoracle.MODE_GB300)
    b = oracle.render(sp, cam, W, H, 16, subframe=2, max_depth=4, mode=pyoracle.MODE_GB300, accum=a["accum"])
    assert np.array_equal(got, b["image8"])
