"""The reference arm of bench.py makes its inputs with oracle/case_setup.py (the
package's host set-up code built for the CPU alone, libccs_setup.so), so that the
process timing the oracle maps no file of the CUDA library.  Its mesh, seeded
state and CFL time step must be the GPU arm's, bit for bit."""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import case_setup as CS

MESH_FIELDS = ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis")


@pytest.mark.parametrize("N,halo,seed,oro", [(12, 3, 1, 8), (24, 3, 3, 8), (20, 4, 7, 0)])
def test_reference_arm_inputs_equal_the_gpu_arms(N, halo, seed, oro):
    ref_mesh, ref_state, ref_dt = CS.seeded_case(N, halo, seed=seed, lmax_oro=oro)
    mesh = M.Mesh(N, halo)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=seed, lmax_oro=oro)
    dt = M.cfl_dt(mesh, s, 0.5)
    for k in MESH_FIELDS:
        assert np.array_equal(getattr(ref_mesh, k).view(np.int64), getattr(mesh, k).view(np.int64)), k
    for k in M.STATE_FIELDS:
        assert np.array_equal(ref_state[k].view(np.int64), s[k].view(np.int64)), k
    assert (ref_mesh.dx, ref_mesh.dy, ref_dt) == (mesh.dx, mesh.dy, dt)


def test_setup_library_is_cpu_only():
    """libccs_setup.so links no CUDA library (it is what the reference arm maps)."""
    import subprocess
    CS.lib()
    out = subprocess.run(["ldd", str(CS.LIB_PATH)], capture_output=True, text=True).stdout
    assert "cuda" not in out.lower() and "libccs_gpu" not in out
