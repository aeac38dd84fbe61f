"""The benchmark's JSON contract, on CPU: the reference arm (the host
restatement of the reference's arithmetic, no GPU involved) prints one line
with the keys the harness reads, and loads nothing of the product library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


RUN_AND_LIST_MAPS = (
    "import runpy, sys\n"
    "sys.argv = ['bench.py', '--impl', 'reference', '--config', 'c1', '--steps', '1', '--warmup', '0']\n"
    "runpy.run_path('bench.py', run_name='__main__')\n"
    "maps = open('/proc/self/maps').read()\n"
    "print('LOADED', int('libvenusaur_gb300' in maps), int('venusaur_gb300' in sys.modules))\n"
)


def test_reference_arm_line(venu):
    r = subprocess.run([sys.executable, "-c", RUN_AND_LIST_MAPS], cwd=ROOT, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    loaded = [ln for ln in r.stdout.splitlines() if ln.startswith("LOADED")]
    assert loaded == ["LOADED 0 0"], loaded  # neither the library nor the package
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True and d["unit"] == "segments/s"
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["arithmetic"] == "reference"
    assert d["cpu_baseline"]["sample"] == d["config"]["cpu_sample"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
