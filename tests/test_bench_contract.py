"""CPU: bench.py's reference arm prints one JSON line with the keys the
benchmark contract names (it times the oracle's restatements of pwm's
parallel CPU paths on the host cores, so it runs without a GPU) and never
loads the GPU library."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    n = 1 << 24  # the default is the full 2^30 text; a smaller one keeps the CPU suite short
    script = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1', "
              f"'--n', '{n}']\n"
              "try:\n    runpy.run_path('bench.py', run_name='__main__')\n"
              "except SystemExit as e:\n    assert not e.code, e.code\n"
              "assert not any(m.startswith('pwm_gb300') for m in sys.modules), 'GPU library loaded'\n"
              "assert 'torch' not in sys.modules\n")
    r = subprocess.run([sys.executable, "-c", script], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "WM/WT build text GB/s" and d["unit"] == "GB/s"
    assert d["higher_is_better"] is True and d["value"] > 0 and d["warmup"] >= 3 and d["steps"] == 1
    assert d["config"]["workload"] and d["config"]["n"] == n and d["config"]["levels"] == 8
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert set(cb["legs"]) == {"ppc", "dd_ps"} and cb["leg"] in cb["legs"]
    assert d["e2e"] == {"value": d["value"], "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
