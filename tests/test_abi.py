"""The C ABI library loads and exports every declared entry point; the host-only
entry points work without a GPU; invalid configurations are rejected before any
device call."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M

HEADER = Path(__file__).resolve().parents[1] / "include" / "ccs_gpu.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(ccs_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("ccs_init", "ccs_set_state", "ccs_step", "ccs_get_state", "ccs_diag", "ccs_destroy",
                     "ccs_strerror", "ccs_batch_create", "ccs_batch_step", "ccs_spatial_operator"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(L.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(declared_functions()) <= set(L.SIGNATURES)


def test_abi_version_and_strerror():
    lib = L.lib()
    assert lib.ccs_abi_version() == 1
    assert lib.ccs_strerror(0) == b"ok"
    assert lib.ccs_strerror(L.CCS_ERR_ARG) == b"invalid argument"


def _cfg(**kw):
    base = dict(N=8, halo=3, scheme=0, precision=0, e_dissipation=0, device=0, dx=0.1, dy=0.1, dt=10.0,
                radius=6.371e6, gravity=9.80616, omega=7.292e-5, phi_mean=0.0)
    base.update(kw)
    return L.Config(**base)


@pytest.mark.parametrize("bad", [dict(N=0), dict(halo=2), dict(scheme=7), dict(precision=3), dict(dt=-1.0),
                                 dict(dx=float("nan")), dict(e_dissipation=5), dict(radius=0.0)])
def test_invalid_config_rejected_without_device(bad):
    mesh = M.Mesh(8, 3)
    mv = mesh.view()
    h = C.c_void_p()
    rc = L.lib().ccs_init(C.byref(_cfg(**bad)), C.byref(mv), C.byref(h))
    assert rc == L.CCS_ERR_ARG
    assert not h.value


def test_null_arguments_rejected():
    lib = L.lib()
    assert lib.ccs_init(None, None, None) == L.CCS_ERR_ARG
    assert lib.ccs_step(None, 1) == L.CCS_ERR_ARG
    assert lib.ccs_set_state(None, None) == L.CCS_ERR_ARG
    assert lib.ccs_get_state(None, None) == L.CCS_ERR_ARG
    assert lib.ccs_ghost_map(0, 3, None) == L.CCS_ERR_ARG
    lib.ccs_destroy(None)


def test_host_mesh_and_initial_state_on_cpu():
    mesh = M.Mesh(12, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=5, lmax_oro=8)
    im = mesh.interior_mask()
    h = s["phi"][im] / mesh.gravity
    assert abs(np.sqrt(np.mean((h - 8000.0) ** 2)) - 200.0) < 1e-6
    speed = np.hypot(s["zonal_wind"][im], s["meridional_wind"][im])
    assert abs(speed.max() - 40.0) < 1e-9
    hs = mesh.phis[im] / mesh.gravity
    assert hs.min() >= 0.0 and hs.max() <= 2000.0 and hs.max() > 0.0
    assert M.cfl_dt(mesh, s, 0.5) > 0
    # the same seed gives the same state; another seed does not
    s2 = M.initial_state(M.Mesh(12, 3), kind=L.CCS_IC_SEEDED, seed=5, lmax_oro=8)
    s3 = M.initial_state(M.Mesh(12, 3), kind=L.CCS_IC_SEEDED, seed=6, lmax_oro=8)
    assert np.array_equal(s["phi"], s2["phi"]) and not np.array_equal(s["phi"], s3["phi"])


def test_streamfunction_winds_are_nondivergent():
    # divergence of the seeded wind on the sphere, by finite differences of the
    # analytic winds along the mesh: small compared with the vorticity
    mesh = M.Mesh(32, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=2, lmax_oro=0)
    F = mesh.field
    h, N = 3, 32
    sg = F(mesh.sqrtG)
    uC = F(s["uC"])
    vC = F(s["vC"])
    div = ((sg * uC)[h + 1:h + N + 1, h:h + N] - (sg * uC)[h - 1:h + N - 1, h:h + N]) / (2 * mesh.dx) + \
          ((sg * vC)[h:h + N, h + 1:h + N + 1] - (sg * vC)[h:h + N, h - 1:h + N - 1]) / (2 * mesh.dy)
    u = F(s["u"])
    v = F(s["v"])
    vort = (v[h + 1:h + N + 1, h:h + N] - v[h - 1:h + N - 1, h:h + N]) / (2 * mesh.dx) - \
           (u[h:h + N, h + 1:h + N + 1] - u[h:h + N, h - 1:h + N - 1]) / (2 * mesh.dy)
    inner = (slice(4, N - 4), slice(4, N - 4))
    assert np.max(np.abs(div[inner])) < 0.05 * np.max(np.abs(vort[inner]))


def test_set_operator_rejects_null_handle_without_device():
    assert L.lib().ccs_set_operator(None, L.CCS_OP_CENTRAL4) == L.CCS_ERR_ARG


def test_autotune_entry_points_reject_null_handle_without_device():
    lib = L.lib()
    assert lib.ccs_autotune(None, 3, 0, None, None) == L.CCS_ERR_ARG
    assert lib.ccs_set_variant(None, 0) == L.CCS_ERR_ARG
    assert lib.ccs_get_variant(None, None, None, None) == L.CCS_ERR_ARG


def test_check_state_rejects_null_handle_without_device():
    assert L.lib().ccs_check_state(None, None) == L.CCS_ERR_ARG


def test_mixed_lane_needs_a_cube_symmetric_metric_without_device():
    """The mixed lane keeps one metric for all panels; a mesh whose panels differ is
    refused before any device call (the FP64 lane takes any mesh)."""
    mesh = M.Mesh(8, 3)
    mesh.sqrtG = mesh.sqrtG.copy()
    mesh.field(mesh.sqrtG)[5, 5, 2] *= 1.0 + 1e-9
    mv = mesh.view()
    h = C.c_void_p()
    rc = L.lib().ccs_init(C.byref(_cfg(precision=1)), C.byref(mv), C.byref(h))
    assert rc == L.CCS_ERR_UNSUPPORTED and not h.value


def test_generated_meshes_pass_the_panel_symmetry_check():
    """Every generated mesh (conformal, halos 3 and 5) passes the mixed lane's
    one-metric-for-all-panels check: ccs_init gets past it to the device set-up
    (no GPU here: CCS_ERR_NODEVICE or a CUDA error, not CCS_ERR_UNSUPPORTED)."""
    for N, h in ((6, 3), (12, 5), (32, 3)):
        mesh = M.Mesh(N, h)
        mv = mesh.view()
        hd = C.c_void_p()
        rc = L.lib().ccs_init(C.byref(_cfg(N=N, halo=h, precision=1)), C.byref(mv), C.byref(hd))
        assert rc != L.CCS_ERR_UNSUPPORTED and rc != L.CCS_ERR_ARG, rc
        if rc == 0:
            L.lib().ccs_destroy(hd)


def test_cfl_dt_is_the_largest_wave_speed_restated():
    """ccs_cfl_dt against a numpy restatement: cfl * min(dx, dy) over the largest
    max(|uC| + sqrt(IG11 phit), |vC| + sqrt(IG22 phit)) of the interior and edge-halo
    cells; a non-positive depth makes it undefined (-1)."""
    mesh = M.Mesh(10, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=4, lmax_oro=6)
    h, N = mesh.halo, mesh.N
    idx = np.arange(mesh.nh) - h + 1
    inb = (idx >= 0) & (idx <= N + 1)
    out_i = (idx < 1) | (idx > N)
    sel = (inb[:, None] & inb[None, :]) & ~(out_i[:, None] & out_i[None, :])
    sel = np.repeat(sel[:, :, None], 6, axis=2).reshape(-1, order="F")
    pt = s["phi"] + mesh.phis
    ig = mesh.matrixIG.reshape(-1, 4)
    lx = np.abs(s["uC"]) + np.sqrt(ig[:, 0] * pt)
    ly = np.abs(s["vC"]) + np.sqrt(ig[:, 3] * pt)
    lmax = np.max(np.maximum(lx, ly)[sel])
    assert M.cfl_dt(mesh, s, 0.5) == pytest.approx(0.5 * min(mesh.dx, mesh.dy) / lmax, rel=1e-15)
    bad = s.copy()
    bad["phi"][np.flatnonzero(mesh.interior_mask())[0]] = -1e6
    with pytest.raises(ValueError):
        M.cfl_dt(mesh, bad, 0.5)
