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


def test_reference_arm_maps_no_cuda_library():
    """The reference arm makes its inputs with the CPU-only set-up library: the
    process that times the oracle never maps libccs_gpu.so."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '1']; "
            "runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); "
            "print('MAPPED', int('libccs_gpu' in maps), int('libccs_setup' in maps), int('libccs_oracle' in maps))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    tail = [ln for ln in r.stdout.splitlines() if ln.startswith("MAPPED")]
    assert tail == ["MAPPED 0 1 1"], r.stdout[-2000:]


def test_kernel_counters_are_tied_to_the_sources():
    """bench.py uses the committed ncu counters only for the kernel sources they were
    taken on."""
    sys.path.insert(0, str(ROOT))
    import bench
    h = bench.kernel_sources_hash()
    assert len(h) == 16
    d = json.loads((ROOT / "profiles" / "roofline_traffic.json").read_text())
    assert bench.profiled_counters() == (d if d.get("sources_sha16") == h else {})


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


def test_counters_cover_both_32_wide_mixed_tiles():
    """The autotuner picks either 32-wide mixed tile at C384 (they run within a few
    tenths of a percent of each other), so the committed counters hold both."""
    d = json.loads((ROOT / "profiles" / "roofline_traffic.json").read_text())
    for v in ("0", "1"):
        c = d["mixed_C384"][v]
        assert c["dram_bytes"] > 0 and c["warp_inst"] > 0
        assert len(c["dram_bytes_per_launch"]) == len(c["warp_inst_per_launch"]) == 4
    assert d["f64_stage_C384_fp64_thread_inst"] > 0


def test_variant_names():
    sys.path.insert(0, str(ROOT))
    import bench
    from conformal_cubed_sphere_gb300 import _lib as L
    assert [bench.variant_name("mixed", v) for v in range(len(L.MIXED_VARIANTS))] == \
        ["32x32 loads", "32x16 loads", "32x32 async", "32x16 async"]
    assert [bench.variant_name("fp64", v) for v in range(3)] == ["32x8", "16x16", "64x4"]
