"""The benchmark's JSON contract on the CPU: the reference arm (the oracle timed on
the host cores) prints one well-formed line, and the issue roofline helper."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "C384 cell-steps/s" and d["unit"] == "cell-steps/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["ms_per_step"] > 0 and d["scaling"] in ("weak", "strong")
    assert d["config"]["workload"].startswith("C384") and d["config"]["N"] == 384
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_issue_roofline():
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.issue_roofline(0.05, 3.0e7, 152, {"sm_mhz": 2000.0, "sm_max_mhz": 2070.0})
    assert r["peak"] == pytest.approx(4 * 152 * 2000e6)
    assert r["achieved"] == pytest.approx(3.0e7 / 0.05e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert bench.issue_roofline(0.05, None, 152, {"sm_mhz": 2000.0}) is None
    assert bench.issue_roofline(0.05, 3.0e7, 152, {"sm_mhz": None, "sm_max_mhz": None}) is None


def test_fp64_roofline():
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.fp64_roofline(3.5, 1.9e9, 152, {"sm_mhz": 2070.0})
    assert r["peak"] == pytest.approx(2 * 152 * 2070e6)
    assert r["frac"] == pytest.approx(1.9e9 / 3.5e-3 / (2 * 152 * 2070e6))
    assert bench.fp64_roofline(3.5, None, 152, {"sm_mhz": 2070.0}) is None
