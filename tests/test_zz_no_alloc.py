"""ccs_diag_noalloc: the diagnostics for callers that cannot allocate device memory.

A model driver that runs inside another framework's memory pool, or under a device
arena sized once at start-up, must not call cudaMalloc; it holds the state in device
memory already.  This test gives the entry point device buffers it did not allocate
(the test allocates them through torch), calls it twice in a row through the C ABI,
and checks both results against ccs_diag of the same state through a normal handle;
a further call after those must leave the device's free memory unchanged.  It sits
in its own file, collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M

pytestmark = pytest.mark.gpu


def test_diag_noalloc_matches_diag_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    mesh = M.Mesh(24, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=9, lmax_oro=8)
    dt = M.cfl_dt(mesh, s, 0.5)
    ref = M.Stepper(mesh, dt, precision="fp64")
    ref.set_state(s)
    ref.step(2)
    st = ref.get_state()
    mass, energy = ref.diag()

    dev = torch.device("cuda", 0)
    arrays = [st["phiG"], st["phi"], st["u"], st["v"], st["uC"], st["vC"], mesh.sqrtG, mesh.phis]
    d = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]
    out = torch.full((2,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    lib = L.lib()
    for _ in range(2):
        rc = lib.ccs_diag_noalloc(mesh.N, mesh.halo, *[t.data_ptr() for t in d], out.data_ptr(), stream)
        assert rc == L.CCS_OK
        torch.cuda.synchronize(dev)
        m2, e2 = out.cpu().tolist()
        assert m2 == pytest.approx(mass, rel=1e-13)
        assert e2 == pytest.approx(energy, rel=1e-13)
        out.fill_(float("nan"))

    # a call after the first ones allocates nothing: the device's free memory stays
    torch.cuda.synchronize(dev)
    free0, _ = torch.cuda.mem_get_info(dev)
    rc = lib.ccs_diag_noalloc(mesh.N, mesh.halo, *[t.data_ptr() for t in d], out.data_ptr(), stream)
    assert rc == L.CCS_OK
    torch.cuda.synchronize(dev)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
    m3, e3 = out.cpu().tolist()
    assert m3 == pytest.approx(mass, rel=1e-13) and e3 == pytest.approx(energy, rel=1e-13)

    # above the fixed scratch capacity the call is rejected before any launch
    big = L.CCS_NOALLOC_MAX_N + 1
    rc = lib.ccs_diag_noalloc(big, 3, *[t.data_ptr() for t in d], out.data_ptr(), stream)
    assert rc == L.CCS_ERR_TOO_LARGE
