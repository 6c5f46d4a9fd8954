"""FP64 lane parity: the CUDA step through the C ABI against the CPU oracle on
the same seeded inputs.  The bar is bit-for-bit equality on every interior and
edge-halo cell (corner blocks are never written by either side)."""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O
from tests.helpers import CHECK_FIELDS, bitwise_equal, max_rel, seeded_case, valid_mask

pytestmark = pytest.mark.gpu


def _pair(N, halo=3, seed=7, oro=True, scheme="RK4", ediss=0, kind=L.CCS_IC_SEEDED):
    mesh, s, dt = seeded_case(N, halo, seed, oro, kind)
    gpu = M.Stepper(mesh, dt, precision="fp64", scheme=scheme, e_dissipation=ediss)
    gpu.set_state(s)
    orc = O.Oracle.from_mesh(mesh, e_dissipation=ediss)
    orc.set_state(s.arrays)
    return mesh, s, dt, gpu, orc


@pytest.mark.parametrize("N,halo,oro", [(8, 3, True), (20, 4, False), (33, 3, True)])
def test_spatial_operator_bitwise(N, halo, oro):
    mesh, s, dt, gpu, orc = _pair(N, halo, oro=oro)
    tg = gpu.spatial_operator()
    to = orc.spatial_operator()
    im = mesh.interior_mask()
    for a, b in zip(tg, to):
        assert bitwise_equal(a, b, im), max_rel(a, b, im)


@pytest.mark.parametrize("scheme", ["RK4", "RK3_TVD"])
@pytest.mark.parametrize("ediss", [0, 1])
def test_one_step_bitwise(scheme, ediss):
    mesh, s, dt, gpu, orc = _pair(12, 3, scheme=scheme, ediss=ediss)
    gpu.step(1)
    orc.run(dt, 1, scheme)
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))


def test_c32_100_steps_within_1e12():
    """Plain-method configuration: C32, halo 3, FP64, RK4, 100 steps at CFL 0.5,
    flat bottom, seeded state.  Target <= 1e-12 relative; the lane is bitwise."""
    mesh, s, dt, gpu, orc = _pair(32, 3, seed=1, oro=False)
    gpu.step(100)
    orc.run(dt, 100)
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert max_rel(g[k], o[k], m) <= 1e-12, k
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))


def test_multi_call_equals_single_call():
    mesh, s, dt, gpu, orc = _pair(16, 3)
    gpu.step(3)
    gpu.step(2)
    other = M.Stepper(mesh, dt, precision="fp64")
    other.set_state(s)
    other.step(5)
    a, b = gpu.get_state(), other.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(a[k], b[k], m), k


def test_async_step_and_timing_path_match():
    mesh, s, dt, gpu, orc = _pair(16, 3)
    gpu.step_async(2)
    gpu.sync()
    t = M.Stepper(mesh, dt, precision="fp64")
    t.set_state(s)
    t.timing(enable=1, reset=1)
    t.step(2)
    ms, n = t.timing(enable=0)
    assert n == 8 and ms > 0
    a, b = gpu.get_state(), t.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(a[k], b[k], m), k


def test_halo_cells_equal_their_source_after_a_step():
    """Ghost indexing on the device: every halo cell's phiG is the bitwise copy of
    the interior cell CubedSphereFillHalo names."""
    mesh, s, dt, gpu, orc = _pair(16, 4)
    gpu.step(1)
    g = gpu.get_state()
    gm = M.ghost_map(16, 4)
    halo = (~mesh.interior_mask()) & (~mesh.corner_mask())
    assert np.array_equal(g["phiG"][halo], g["phiG"][gm[halo]])
    assert np.array_equal(g["zonal_wind"][halo], g["zonal_wind"][gm[halo]])


def test_set_get_round_trip():
    mesh, s, dt, gpu, orc = _pair(10, 3)
    g = gpu.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert np.array_equal(g[k][m], s[k][m]), k


def test_diagnostics_match_oracle():
    mesh, s, dt, gpu, orc = _pair(24, 3)
    gpu.step(3)
    orc.run(dt, 3)
    mg, eg = gpu.diag()
    assert mg == pytest.approx(orc.total_mass(), rel=1e-13)
    assert eg == pytest.approx(orc.total_energy(), rel=1e-13)


def test_shared_mesh_and_batch_bitwise():
    """Members on one grid share the device mesh; a batch of them advanced in one
    launch per stage equals each member advanced alone."""
    mesh = M.Mesh(16, 3)
    states = [M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=20 + k) for k in range(3)]
    dt = min(M.cfl_dt(mesh, st, 0.5) for st in states)
    owner = M.Stepper(mesh, dt, precision="fp64")
    members = [owner] + [M.Stepper(mesh, dt, precision="fp64", share_with=owner) for _ in range(2)]
    for st, m in zip(states, members):
        m.set_state(st)
    b = M.Batch(members)
    b.step(3)
    msk = valid_mask(mesh)
    for st, m in zip(states, members):
        alone = M.Stepper(mesh, dt, precision="fp64")
        alone.set_state(st)
        alone.step(3)
        a, c = m.get_state(), alone.get_state()
        for k in CHECK_FIELDS:
            assert bitwise_equal(a[k], c[k], msk), k


def test_reference_test_cases_run():
    for kind in (L.CCS_IC_CASE2, L.CCS_IC_CASE5, L.CCS_IC_CASE6):
        mesh, s, dt, gpu, orc = _pair(12, 3, kind=kind)
        gpu.step(2)
        orc.run(dt, 2)
        g, o = gpu.get_state(), orc.get_state()
        m = valid_mask(mesh)
        for k in CHECK_FIELDS:
            assert bitwise_equal(g[k], o[k], m), (kind, k)


@pytest.mark.parametrize("b", [3.0, 6.0, 12.0])
def test_constant_division_is_correctly_rounded(b):
    """The FP64 lane divides by the constants 3, 6 and 12 with a reciprocal and one
    FMA correction; every quotient must equal IEEE division bit for bit."""
    import ctypes as C
    rng = np.random.default_rng(int(b))
    n = 1 << 23
    sig = rng.integers(0, 1 << 52, size=n, dtype=np.uint64)
    exp = rng.integers(1023 - 200, 1023 + 200, size=n, dtype=np.uint64)
    sgn = rng.integers(0, 2, size=n, dtype=np.uint64)
    x = ((sgn << np.uint64(63)) | (exp << np.uint64(52)) | sig).view(np.float64).copy()
    # exact multiples, halfway-style significands, signed zeros and infinities, a NaN
    x[:11] = [0.0, -0.0, 3.0, -6.0, 1.0, 1.5, 2.0 ** -40, 7.0, np.inf, -np.inf, np.nan]
    x[16:4096] = np.arange(16, 4096) * b
    fast = np.empty(n)
    ieee = np.empty(n)
    dp = C.POINTER(C.c_double)
    rc = L.lib().ccs_selftest_div(x.ctypes.data_as(dp), n, b, fast.ctypes.data_as(dp), ieee.ctypes.data_as(dp))
    assert rc == 0
    ok = ~np.isnan(x)
    assert np.array_equal(fast[ok].view(np.int64), ieee[ok].view(np.int64))
    assert np.array_equal(ieee[ok], x[ok] / b)
    assert np.isnan(fast[10]) and np.isnan(ieee[10])


def test_shared_divisor_division_is_correctly_rounded():
    """The WENO-Z weights alpha_k / sum(alpha) share their divisor: the FP64 lane takes
    its IEEE reciprocal once and corrects each product with one FMA.  Every quotient
    must equal IEEE division bit for bit: random significands and exponents (normal
    quotients), divisors with all-ones and all-zeros significands, and the kernels'
    own range (0.1 <= a <= b)."""
    import ctypes as C
    rng = np.random.default_rng(77)
    n = 1 << 23

    def doubles(exp_lo, exp_hi, size):
        sig = rng.integers(0, 1 << 52, size=size, dtype=np.uint64)
        exp = rng.integers(exp_lo, exp_hi, size=size, dtype=np.uint64)
        return ((exp << np.uint64(52)) | sig).view(np.float64).copy()

    a = doubles(1023 - 400, 1023 + 400, n)
    b = doubles(1023 - 400, 1023 + 400, n)
    q = n // 4  # the kernels' range: a >= 0.1, b = a + (two more such terms)
    a[:q] = 0.1 + rng.random(q) * rng.choice([1.0, 1e3, 1e9], size=q)
    b[:q] = a[:q] + (0.7 + rng.random(q) * rng.choice([1.0, 1e3, 1e12], size=q))
    m = 1 << 16  # divisors whose significand is all ones or all zeros
    expb = rng.integers(1023 - 300, 1023 + 300, size=m, dtype=np.uint64) << np.uint64(52)
    b[q:q + m] = (expb | np.uint64((1 << 52) - 1)).view(np.float64)
    b[q + m:q + 2 * m] = expb.view(np.float64)
    fast = np.empty(n)
    ieee = np.empty(n)
    dp = C.POINTER(C.c_double)
    rc = L.lib().ccs_selftest_div_pairs(a.ctypes.data_as(dp), b.ctypes.data_as(dp), n, fast.ctypes.data_as(dp),
                                        ieee.ctypes.data_as(dp))
    assert rc == 0
    assert np.array_equal(ieee, a / b)
    assert np.array_equal(fast.view(np.int64), ieee.view(np.int64))


@pytest.mark.parametrize("op", [L.CCS_OP_CENTRAL2, L.CCS_OP_CENTRAL4, L.CCS_OP_CENTRAL6])
def test_central_difference_operator_bitwise(op):
    """spatial_operators_mod_{2nd,4th,6th}.F90: tendency and 5 RK4 steps bit for bit."""
    mesh, s, dt = seeded_case(20, 3, seed=5, oro=True)
    gpu = M.Stepper(mesh, 0.5 * dt, precision="fp64", operator=op)
    gpu.set_state(s)
    orc = O.Oracle.from_mesh(mesh, operator=op)
    orc.set_state(s.arrays)
    im = mesh.interior_mask()
    for a, b in zip(gpu.spatial_operator(), orc.spatial_operator()):
        assert bitwise_equal(a, b, im), max_rel(a, b, im)
    gpu.step(5)
    orc.run(0.5 * dt, 5)
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))


def test_operator_switch_and_batch_carry_the_operator():
    """Switching a handle's operator takes effect on its next step; a batch built
    afterwards steps each member with its own operator (RK3_TVD member included)."""
    mesh, s, dt = seeded_case(16, 3, seed=9, oro=False)
    a = M.Stepper(mesh, dt, precision="fp64")
    a.set_operator(L.CCS_OP_CENTRAL4)
    b = M.Stepper(mesh, dt, precision="fp64", scheme="RK3_TVD", operator=L.CCS_OP_CENTRAL2)
    c = M.Stepper(mesh, dt, precision="fp64")  # WENO
    for x in (a, b, c):
        x.set_state(s)
    M.Batch([a, b, c]).step(3)
    m = valid_mask(mesh)
    for stepper, op, scheme in ((a, 4, "RK4"), (b, 2, "RK3_TVD"), (c, 0, "RK4")):
        orc = O.Oracle.from_mesh(mesh, operator=op)
        orc.set_state(s.arrays)
        orc.run(dt, 3, scheme)
        g, o = stepper.get_state(), orc.get_state()
        for k in CHECK_FIELDS:
            assert bitwise_equal(g[k], o[k], m), (op, k, max_rel(g[k], o[k], m))


@pytest.mark.parametrize("op", [L.CCS_OP_CENTRAL2, L.CCS_OP_CENTRAL4, L.CCS_OP_CENTRAL6])
def test_mixed_lane_central_operators_close_to_fp64(op):
    """The central-difference operators on the mixed lane: tendency within FP32
    rounding of the FP64 lane's, and ten steps at FP32 rounding level in h."""
    mesh, s, dt = seeded_case(24, 3, seed=4, oro=True)
    mx = M.Stepper(mesh, 0.5 * dt, precision="mixed", phi_mean=8000.0 * mesh.gravity, operator=op)
    f64 = M.Stepper(mesh, 0.5 * dt, precision="fp64", operator=op)
    for g in (mx, f64):
        g.set_state(s)
    im = mesh.interior_mask()
    rel = lambda a, b: float(np.linalg.norm(a[im] - b[im]) / np.linalg.norm(b[im]))  # noqa: E731
    for a, b in zip(mx.spatial_operator(), f64.spatial_operator()):
        assert rel(a, b) < 2e-4
    mx.step(10)
    f64.step(10)
    a, b = mx.get_state(), f64.get_state()
    assert rel(a["phi"], b["phi"]) < 1e-6


def test_c192_1000_steps_with_orography_bitwise():
    """Long-run configuration: C192, halo 3, FP64, RK4, 1000 steps at CFL 0.5 over
    seeded orography (about 1.5 simulated days).  The oracle takes one to three
    minutes on the host cores; the lane must stay bit for bit on every checked field."""
    mesh, s, dt, gpu, orc = _pair(192, 3, seed=1, oro=True)
    gpu.step(1000)
    orc.run(dt, 1000)
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))


def test_rk3_reconstruct_halo5_60_steps_bitwise():
    """RK3-TVD with the E-reconstruction option at halo 5, 60 steps of C24."""
    mesh, s, dt, gpu, orc = _pair(24, 5, seed=13, oro=True, scheme="RK3_TVD", ediss=1)
    gpu.step(60)
    orc.run(dt, 60, "RK3_TVD")
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_health_check_counts_bad_cells(precision):
    """ccs_check_state: 0 on a healthy state; planted non-finite wind and a
    non-positive depth (host-side inputs) are counted."""
    mesh, s, dt = seeded_case(16, 3, seed=1, oro=False)
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    g = M.Stepper(mesh, dt, precision=precision, **kw)
    g.set_state(s)
    g.step(2)
    assert g.check_state() == 0
    bad = s.copy()
    F = mesh.field
    F(bad["u"])[3 + 2, 3 + 5, 1] = np.nan
    F(bad["phi"])[3 + 7, 3 + 7, 4] = -1.0
    F(bad["phiG"])[3 + 7, 3 + 7, 4] = -1.0
    F(bad["phi"])[0, 5, 0] = np.nan  # a halo cell: not counted
    g.set_state(bad)
    assert g.check_state() == 2


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_corner_blocks_are_never_read(precision):
    """NaN in every corner-block cell of the input changes nothing outside the corner
    blocks (both lanes): the step never reads a cell the reference never fills."""
    mesh, s, dt = seeded_case(16, 3, seed=17, oro=True)
    poisoned = s.copy()
    cm = mesh.corner_mask()
    for k in ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind"):
        poisoned[k][cm] = np.nan
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    out = []
    for st in (s, poisoned):
        g = M.Stepper(mesh, dt, precision=precision, **kw)
        g.set_state(st)
        g.step(4)
        assert g.check_state() == 0
        out.append(g.get_state())
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(out[0][k], out[1][k], m), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_odd_n_runs_with_the_pole_inverse_option(precision):
    """With CCS_MESH_POLE_INVERSE an odd-N grid (a cell centred on each pole) steps
    stably; the FP64 lane stays bit for bit with the oracle on the same arrays."""
    mesh = M.Mesh(33, 3, pole_inverse=True)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=4, lmax_oro=8)
    dt = M.cfl_dt(mesh, s, 0.5)
    assert dt > 100.0
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    g = M.Stepper(mesh, dt, precision=precision, **kw)
    g.set_state(s)
    g.step(5)
    assert g.check_state() == 0
    if precision == "fp64":
        orc = O.Oracle.from_mesh(mesh)
        orc.set_state(s.arrays)
        orc.run(dt, 5)
        a, b = g.get_state(), orc.get_state()
        m = valid_mask(mesh)
        for k in CHECK_FIELDS:
            assert bitwise_equal(a[k], b[k], m), k


@pytest.mark.parametrize("N,halo", [(4, 3), (4, 4), (6, 6)])
def test_smallest_grids(N, halo):
    """Grids smaller than one tile, up to a halo as wide as a panel (the ghost map
    then copies whole neighbour panels): the FP64 lane stays bitwise with the oracle
    over three RK4 steps, and the mixed lane stays close to it."""
    mesh, s, dt, gpu, orc = _pair(N, halo)
    gpu.step(3)
    orc.run(dt, 3)
    g, o = gpu.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(g[k], o[k], m), (k, max_rel(g[k], o[k], m))
    mx = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000.0 * mesh.gravity)
    mx.set_state(s)
    mx.step(3)
    assert mx.check_state() == 0
    x = mx.get_state()
    im = mesh.interior_mask()
    assert max_rel(x["phi"], o["phi"], im) < 1e-6


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_courant_number_matches_the_host_cfl(precision):
    """ccs_courant (device, current state) against the host's CFL step of the same
    state: dt / cfl_dt(cfl = 1); a state with a negative depth gives inf."""
    mesh, s, dt = seeded_case(20, 3, seed=9, oro=True)
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    g = M.Stepper(mesh, dt, precision=precision, **kw)
    g.set_state(s)
    ref = dt / M.cfl_dt(mesh, s, 1.0)
    assert ref == pytest.approx(0.5, rel=1e-12)  # dt itself came from CFL 0.5
    tol = 1e-12 if precision == "fp64" else 2e-6  # the mixed lane holds the state in FP32
    assert g.courant() == pytest.approx(ref, rel=tol)
    g.step(3)
    st = g.get_state()
    assert g.courant() == pytest.approx(dt / M.cfl_dt(mesh, st, 1.0), rel=tol)
    bad = s.copy()
    k = np.flatnonzero(mesh.interior_mask())[5]
    bad["phi"][k] = -(mesh.phis[k] + 1.0)  # phit = phi + phis = -1
    bad["phiG"][k] = bad["phi"][k] * mesh.sqrtG[k]
    g.set_state(bad)
    assert g.courant() == float("inf")
