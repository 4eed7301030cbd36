"""The bench's output contract, checked on the host: the reference arm (the
reference's CPU minimum variance, no GPU involved) prints one JSON line with
the keys the contract names, and the bench accepts every workload the
documentation lists."""

from __future__ import annotations

import json
import os
import re
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    # The arm runs in a process that then reports whether this engine's
    # modules were imported: the reference arm must not load the product.
    code = ("import runpy, sys\n"
            "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0', '--lines', '4']\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit as e:\n"
            "    assert not e.code, e.code\n"
            "print('LOADED', sorted(m for m in sys.modules if m == 'usx' or m.startswith(('usx.', '_usx'))))\n")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, cwd=ROOT,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["value"] > 0 and d["unit"] == "frames/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == "learned_75pw_512x1024"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] == 2 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "LOADED []" in out.stdout
    # One step is the sample of lines; value = lines per second / 512.
    assert abs(d["value"] - 4 / 512 / (d["ms_per_step"] / 1e3)) < 1e-6 * d["value"]


def test_reference_arm_geometry_equals_the_engines():
    """The CPU arm builds the headline transmits and grid with numpy alone;
    they equal this engine's host objects bit for bit."""
    sys.path.insert(0, str(ROOT))
    import bench
    angles, delays, apod, pts = bench.reference_workload()
    usx, probe, medium, acq, sim, txs, ph, grid = bench.workload_setup(n_scat=10)
    assert np.array_equal(angles, np.asarray([t.angle for t in txs], np.float32))
    assert np.array_equal(delays, np.asarray([t.delays for t in txs], np.float32))
    assert np.array_equal(apod, np.asarray([t.apodization for t in txs], np.float32))
    assert np.array_equal(pts, np.asarray(grid.points, np.float32).reshape(-1, 3))


def test_bench_accepts_every_documented_workload():
    readme = (ROOT / "README.md").read_text()
    listed = re.search(r"--workload ([a-z_|]+)", readme).group(1).split("|")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                         cwd=ROOT, timeout=120)
    assert out.returncode == 0
    choices = re.search(r"--workload \{([^}]*)\}", out.stdout).group(1).split(",")
    assert set(listed) <= set(choices), set(listed) - set(choices)
    assert "learned" in choices
