"""The bounds-checked build (-DCCS_BOUNDS): its kernels check the indices of their
array accesses and record, instead of performing, any access outside an array.
Small cases on both lanes must record none."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

from conformal_cubed_sphere_gb300 import _lib as L

ROOT = Path(__file__).resolve().parents[1]


def test_normal_build_reports_no_checks():
    import ctypes as C
    site, idx = C.c_int(0), C.c_int64(0)
    assert L.lib().ccs_debug_bounds(C.byref(site), C.byref(idx)) == L.CCS_OK
    assert site.value == -1
    assert L.lib().ccs_debug_bounds_selftest() == L.CCS_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_bounds_checked_build_records_no_out_of_range_index():
    from conformal_cubed_sphere_gb300 import build as B
    lib = B.build_bounds()
    env = dict(os.environ, CCS_GPU_LIB=str(lib))
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "bounds_cases.py")], env=env, capture_output=True,
                       text=True, timeout=1200, cwd=ROOT)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "bounds-checked cases clean" in r.stdout
