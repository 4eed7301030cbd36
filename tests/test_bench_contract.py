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

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)
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


def test_bench_accepts_every_documented_workload():
    readme = (ROOT / "README.md").read_text()
    listed = re.search(r"--workload ([a-z_|]+)", readme).group(1).split("|")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                         cwd=ROOT, timeout=120)
    assert out.returncode == 0
    choices = re.search(r"--workload \{([^}]*)\}", out.stdout).group(1).split(",")
    assert set(listed) <= set(choices), set(listed) - set(choices)
    assert "learned" in choices
