"""CPU tests of the C-ABI library: it builds, loads, exports every symbol that
include/*.h declares, and its GPU entry points fail loudly without a device
(there is no CPU fallback)."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names |= set(re.findall(r"VENU_API\s+[\w\s\*]*?\b(venu_\w+)\s*\(", src))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("venu_scene_create", "venu_render", "venu_trace", "venu_renderer_create"):
        assert must in names


def test_library_exports_every_declared_symbol(venu):
    from venusaur_gb300._lib import LIB_PATH

    out = subprocess.run(["nm", "-D", "--defined-only", LIB_PATH], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT\s+(venu_\w+)", out))
    missing = [n for n in declared_symbols() if n not in exported]
    assert not missing, missing
    L = C.CDLL(LIB_PATH)
    for n in declared_symbols():
        assert getattr(L, n) is not None


def test_header_compiles_as_c():
    src = '#include "venu.h"\nint main(void){ venu_sphere s; (void)s; return (int)sizeof(venu_camera) - 52; }\n'
    r = subprocess.run(["gcc", "-x", "c", "-std=c99", "-I", os.path.join(ROOT, "include"), "-fsyntax-only", "-"],
                       input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_struct_layouts(venu):
    assert venu.SPHERE_DTYPE.itemsize == 48
    assert venu.CAMERA_DTYPE.itemsize == 52
    assert venu.NODE_DTYPE.itemsize == 32


def test_no_device_fails_loudly(venu):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(venu.VenuError) as e:
        venu.DeviceScene(venu.generate_rtiow(0))
    assert e.value.status == 4  # VENU_ERR_NO_DEVICE
    with pytest.raises(venu.VenuError):
        venu.Wavefront()


def test_invalid_arguments(venu):
    from venusaur_gb300._lib import check, lib

    with pytest.raises(venu.VenuError) as e:
        check(lib().venu_scene_generate_random(10, 0, None, None, 0.0, 1.0, None))
    assert e.value.status == 1


def test_host_generators(venu):
    s = venu.Scene()
    assert len(s) == 485
    assert s.m_aabbs.shape == (485, 6)
    sp = s.m_spheres
    assert sp[0].GetRadius() == 1000.0 and sp[0].GetMaterial().GetType() == venu.Material.Lambertian
    assert sp[-1].GetMaterial().GetType() == venu.Material.Metal
    r = venu.Scene.random(1000, seed=3)
    assert len(r) == 1000
    back = venu.Scene(spheres=r.m_spheres)
    assert back.spheres.tobytes() == r.spheres.tobytes()
    cam = venu.Camera((13, 2, 3), 20.0, 1.5, 0.1, 10.0)
    cam.SetForward(np.float32([-13, -2, -3]))
    u, v, w = cam.UVWFrame()
    assert abs(float(np.dot(w, w)) - 100.0) < 1e-3


def test_ctypes_mirrors_match_the_header(venu, tmp_path):
    """Every ctypes structure of the Python binding has the size and field
    offsets of its C declaration (compiled here with gcc)."""
    from venusaur_gb300 import _lib

    pairs = {"venu_render_opts": _lib.RenderOpts, "venu_scene_info": _lib.SceneInfo,
             "venu_render_stats": _lib.RenderStats, "venu_tuning": _lib.Tuning, "venu_camera": _lib.CameraC,
             "venu_job_desc": _lib.JobDesc, "venu_batch_stats": _lib.BatchStats, "venu_request": _lib.Request,
             "venu_result": _lib.Result, "venu_server_stats": _lib.ServerStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "venu.h"', "int main(void) {"]
    for cname, cls in pairs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    want = []
    for cname, cls in pairs.items():
        want.append(f"{cname} size {C.sizeof(cls)}")
        for f in cls._fields_:
            want.append(f"{cname} {f[0]} {getattr(cls, f[0]).offset}")
    assert [g for g in got if g] == want
