"""Known-answer tests pinning the CPU oracle against the reference source.

The reference ships no tests or golden vectors and cannot be compiled here (no
Fortran compiler), so these checks restate behaviour the Fortran source implies:
WENO exactness on polynomials, the ghost-fill permutation, the metric
derivation, projection round trips, the steady interior of test case 2 and the
sphere-area check of io_mod.F90:306.
"""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O
from tests.helpers import seeded_case


# ---- WENO_limiter (spatial_operators_mod.F90:282-361) -------------------------

@pytest.mark.parametrize("c", [0.0, 1.0, -3.5, 1e18])
def test_weno_constant_is_reproduced(c):
    # the candidate stencils sum to one: constant data comes back to within rounding
    for d in (1, -1):
        assert O.weno_limiter([c] * 5, d) == pytest.approx(c, rel=4e-16, abs=0)


@pytest.mark.parametrize("a,b", [(1.0, 0.5), (-2.0, 3.0), (1e3, 1e-3)])
def test_weno_linear_reconstructs_face_value(a, b):
    # cell averages of a + b x on unit cells centred at -2..2; face at x = +1/2 ("+")
    # and x = -1/2 ("-" reconstructs the left face of the centre cell)
    Q = [a + b * x for x in (-2, -1, 0, 1, 2)]
    assert O.weno_limiter(Q, 1) == pytest.approx(a + 0.5 * b, rel=1e-13, abs=1e-12)
    assert O.weno_limiter(Q, -1) == pytest.approx(a - 0.5 * b, rel=1e-13, abs=1e-12)


def test_weno_mirror_symmetry():
    rng = np.random.default_rng(0)
    for _ in range(200):
        Q = rng.normal(size=5)
        assert O.weno_limiter(Q, -1) == pytest.approx(O.weno_limiter(Q[::-1], 1), rel=1e-12, abs=1e-14)


def test_weno_smooth_data_fifth_order():
    # WENO-Z on smooth data converges at 5th order to the point value at the face
    errs = []
    for n in (40, 80):
        h = 1.0 / n
        x = np.arange(-2, 3) * h
        cell_avg = (np.sin(x + h / 2) - np.sin(x - h / 2)) / h  # averages of cos
        errs.append(abs(O.weno_limiter(cell_avg, 1) - np.cos(h / 2)))
    assert errs[0] / errs[1] > 16  # at least 4th order; 5th asymptotically


def test_weno_branch_switches():
    # tau40 <= min(beta) and tau41 > min(beta): omega = [1/3, 2/3, 0]
    Q = np.array([0.0, 0.0, 0.0, 1.0, 1.0])
    b1 = 0.0
    st = [Q[0] / 3 - 7 / 6 * Q[1] + 11 / 6 * Q[2], -Q[1] / 6 + 5 / 6 * Q[2] + Q[3] / 3,
          Q[2] / 3 + 5 / 6 * Q[3] - Q[4] / 6]
    beta = [13 / 12 * (Q[0] - 2 * Q[1] + Q[2]) ** 2 + 0.25 * (Q[0] - 4 * Q[1] + 3 * Q[2]) ** 2,
            13 / 12 * (Q[1] - 2 * Q[2] + Q[3]) ** 2 + 0.25 * (Q[1] - Q[3]) ** 2,
            13 / 12 * (Q[2] - 2 * Q[3] + Q[4]) ** 2 + 0.25 * (3 * Q[2] - 4 * Q[3] + Q[4]) ** 2]
    assert beta[0] == b1
    t40, t41 = abs(beta[0] - beta[1]), abs(beta[1] - beta[2])
    assert not (t40 <= min(beta) and t41 > min(beta))  # this data takes the WENO-Z branch
    w = np.array([0.1, 0.6, 0.3]) * (1 + abs(beta[2] - beta[0]) / (1e-2 + np.array(beta)))
    expect = np.dot(st, w / w.sum())
    assert O.weno_limiter(Q, 1) == pytest.approx(expect, rel=1e-14)


# ---- ghost fill (ghost_mod.f90:18-82) ------------------------------------------

@pytest.mark.parametrize("N,h", [(4, 3), (8, 3), (12, 4), (16, 3)])
def test_ghost_map_equals_fill_halo(N, h):
    mesh = M.Mesh(N, h)
    idx = np.arange(mesh.ncell, dtype=np.float64)
    filled = O.fill_halo(N, h, np.where(mesh.interior_mask(), idx, -1.0))
    gm = M.ghost_map(N, h)
    cm = mesh.corner_mask()
    assert np.array_equal(gm[~cm], filled[~cm].astype(np.int64))
    assert np.all(gm[cm] == -1)
    # every halo edge cell is a copy of an interior cell; interior cells map to themselves
    assert np.array_equal(gm[mesh.interior_mask()], np.flatnonzero(mesh.interior_mask()))


def test_halo_cells_are_geometric_neighbours():
    N, h = 16, 3
    mesh = M.Mesh(N, h)
    x = O.fill_halo(N, h, _cart(mesh, 0))
    y = O.fill_halo(N, h, _cart(mesh, 1))
    z = O.fill_halo(N, h, _cart(mesh, 2))
    F = mesh.field
    X, Y, Z = F(x), F(y), F(z)

    def gap(i1, i2, p):
        a = np.stack([X[i1, h:h + N, p], Y[i1, h:h + N, p], Z[i1, h:h + N, p]])
        b = np.stack([X[i2, h:h + N, p], Y[i2, h:h + N, p], Z[i2, h:h + N, p]])
        return np.arccos(np.clip(np.sum(a * b, axis=0), -1, 1))

    away = slice(3, N - 3)  # rows away from the corner singularities
    for p in range(6):
        # on the conformal grid the halo cells continue the panel's grid lines: the
        # spacing across the edge matches the spacing just inside it
        inside = gap(h, h + 1, p)
        for k in range(h):
            across = gap(h - k, h - k - 1, p)
            r = across / inside
            assert np.all(np.abs(r[away] - 1) < 0.2 + 0.15 * k), (p, k)
            assert np.all((r > 0.2) & (r < 5))


def _cart(mesh, comp):
    N, h = mesh.N, mesh.halo
    out = np.zeros(mesh.ncell)
    F = mesh.field(out)
    f = mesh.file[("x", "y", "z")[comp]].reshape((N, N, 6), order="F")
    F[h:h + N, h:h + N, :] = f
    return out


# ---- metric derivation (io_mod.F90:119-220, 295-306) -----------------------------

@pytest.mark.parametrize("N,h", [(8, 3), (20, 4)])
def test_metric_derivation_matches_oracle_bitwise(N, h):
    mesh = M.Mesh(N, h)
    f = mesh.file
    d = O.derive_metrics(N, h, mesh.radius, mesh.omega, f["lon"], f["lat"], f["x"], f["y"], f["z"], f["jab"])
    for k in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "lon", "lat", "sinlat", "coslat"):
        assert np.array_equal(d[k], getattr(mesh, k)), k


def test_jab_fill_matches_halo_metric_continuity():
    # FillJab re-expresses the neighbour's Jacobian in this panel's axes: the halo
    # cell's sqrtG equals its source cell's sqrtG exactly (a signed permutation of
    # the columns leaves det(J^T J) unchanged)
    N, h = 12, 3
    mesh = M.Mesh(N, h)
    gm = M.ghost_map(N, h)
    halo = (~mesh.interior_mask()) & (~mesh.corner_mask())
    assert np.allclose(mesh.sqrtG[halo], mesh.sqrtG[gm[halo]], rtol=1e-14, atol=0)


def test_sphere_area():
    for N in (16, 48):
        mesh = M.Mesh(N, 3)
        area = np.sum(mesh.sqrtG[mesh.interior_mask()]) * mesh.dx * mesh.dy
        assert abs(area / (4 * np.pi * mesh.radius ** 2) - 1) < 2e-3 * (16 / N) ** 2


def test_projection_round_trip():
    # covProjSphere2Plane(covProjPlane2Sphere(u)) = u (projection_mod.F90:60-96)
    mesh = M.Mesh(10, 3)
    m = ~mesh.corner_mask()
    G = mesh.matrixG.reshape(-1, 2, 2).transpose(0, 2, 1)
    IG = mesh.matrixIG.reshape(-1, 2, 2).transpose(0, 2, 1)
    A = mesh.matrixA.reshape(-1, 2, 2).transpose(0, 2, 1)
    IA = mesh.matrixIA.reshape(-1, 2, 2).transpose(0, 2, 1)
    R = np.einsum("nij,njk,nkl,nlm->nim", G, IA, A, IG)[m]
    assert np.allclose(R, np.eye(2)[None], atol=1e-12)


# ---- the step ------------------------------------------------------------------

def test_case2_interior_tendency_converges():
    """Test case 2 is an exact steady state of the continuous equations
    (test_case_mod.F90:61-95): away from panel edges the discrete tendency is pure
    truncation error and falls at high order with resolution."""
    errs = []
    for N in (24, 48):
        h = 3
        mesh = M.Mesh(N, h)
        s = M.initial_state(mesh, kind=L.CCS_IC_CASE2)
        orc = O.Oracle.from_mesh(mesh)
        orc.set_state(s.arrays)
        tp, tu, tv = orc.spatial_operator()
        F = mesh.field
        q = N // 4  # the central half of each panel
        inner = (slice(h + q, h + N - q), slice(h + q, h + N - q), slice(None))
        errs.append(np.max(np.abs(F(tp)[inner] / F(s["phiG"])[inner])))
    # cell-centre point values fed to a cell-average reconstruction: third order
    assert errs[0] / errs[1] > 6
    assert errs[1] < 1e-9


@pytest.mark.parametrize("op,ratio", [(2, 3.3), (4, 13.0), (6, 40.0)])
def test_central_difference_operators_converge_at_their_order(op, ratio):
    """spatial_operators_mod_{2nd,4th,6th}.F90 on the steady state of test case 2:
    the tendency in the central half of each panel falls by about 2^op per halving
    of the cell size (measured 3.8, 15.7, 47 from C24 to C48)."""
    errs = []
    for N in (24, 48):
        h = 3
        mesh = M.Mesh(N, h)
        s = M.initial_state(mesh, kind=L.CCS_IC_CASE2)
        orc = O.Oracle.from_mesh(mesh, operator=op)
        orc.set_state(s.arrays)
        tp, tu, tv = orc.spatial_operator()
        F = mesh.field
        q = N // 4
        inner = (slice(h + q, h + N - q), slice(h + q, h + N - q), slice(None))
        errs.append(np.max(np.abs(F(tp)[inner] / F(s["phiG"])[inner])))
    assert errs[0] / errs[1] > ratio


@pytest.mark.parametrize("op", [2, 4, 6])
def test_central_difference_operator_matches_numpy_restatement(op):
    """A second, vectorised restatement of the central-difference tendencies
    (same operand order) agrees with the oracle bit for bit."""
    mesh, s, dt = seeded_case(10, 3, oro=True)
    orc = O.Oracle.from_mesh(mesh, operator=op)
    orc.set_state(s.arrays)
    tp, tu, tv = (mesh.field(t) for t in orc.spatial_operator())
    F = mesh.field
    h, N = 3, 10
    phit = F(s["phi"]) + F(mesh.phis)
    E = phit + 0.5 * (F(s["u"]) * F(s["uC"]) + F(s["v"]) * F(s["vC"]))
    fx, fy = F(s["phiG"]) * F(s["uC"]), F(s["phiG"]) * F(s["vC"])

    def d(f, axis, dd):
        def sh(k):
            sl = [slice(h, h + N), slice(h, h + N), slice(None)]
            sl[axis] = slice(h + k, h + N + k)
            return f[tuple(sl)]
        if op == 2:
            return (sh(1) - sh(-1)) / (2. * dd)
        if op == 4:
            return (sh(-2) - 8. * sh(-1) + 8. * sh(1) - sh(2)) / (12. * dd)
        return (-sh(-3) + 9. * sh(-2) - 45. * sh(-1) + 45. * sh(1) - 9. * sh(2) + sh(3)) / (60. * dd)

    I = (slice(h, h + N), slice(h, h + N), slice(None))
    vort = d(F(s["v"]), 0, mesh.dx) - d(F(s["u"]), 1, mesh.dy) + F(mesh.sqrtG)[I] * F(mesh.f)[I]
    ref_p = -(d(fx, 0, mesh.dx) + d(fy, 1, mesh.dy))
    ref_u = -d(E, 0, mesh.dx) + vort * F(s["vC"])[I]
    ref_v = -d(E, 1, mesh.dy) - vort * F(s["uC"])[I]
    for a, b in ((tp[I], ref_p), (tu[I], ref_u), (tv[I], ref_v)):
        assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_oracle_rejects_unknown_operator():
    mesh = M.Mesh(8, 3)
    with pytest.raises(ValueError):
        O.Oracle.from_mesh(mesh, operator=3)


def test_oracle_mass_conserved_and_deterministic():
    mesh, s, dt = seeded_case(12, oro=True)
    a = O.Oracle.from_mesh(mesh)
    a.set_state(s.arrays)
    m0 = a.total_mass()
    a.run(dt, 5)
    assert abs(a.total_mass() - m0) / abs(m0) < 1e-12
    b = O.Oracle.from_mesh(mesh)
    b.set_state(s.arrays)
    b.run(dt, 5)
    sa, sb = a.get_state(), b.get_state()
    for k in ("phiG", "u", "v"):
        assert np.array_equal(sa[k], sb[k])


def test_rk4_combination_matches_four_stage_formula():
    """phiG(new) = phiG(old) + dt (((k1 + 2k2) + 2k3) + k4) / 6 on the interior,
    bit for bit (time_scheme_mod.F90:13-44; the boundary correction leaves interior
    phiG untouched)."""
    mesh, s, dt = seeded_case(8, oro=False)
    o = O.Oracle.from_mesh(mesh)
    o.set_state(s.arrays)
    o.rk4_once(dt)
    new = o.get_state(slot=1)
    k = [o.get_tend(slot)[0] for slot in (-1, -2, -3, -4)]
    im = mesh.interior_mask()
    comb = (k[0] + 2.0 * k[1] + 2.0 * k[2] + k[3]) / 6.0
    assert np.array_equal(new["phiG"][im], (s["phiG"] + dt * comb)[im])


def test_pole_cell_inverse_follows_the_reference_formula():
    """Odd N puts a cell centre on each pole, where read_mesh replaces A^-1 by its
    'analytical approximation' (io_mod.F90:190-210): the lon rotation times the
    radius.  The metric derivation keeps that formula as written.  (A^-1 elsewhere
    scales as 1/radius, so the pole cell's covariant wind comes out a^2 times too
    large and an odd-N run of the reference step blows up in its first step; even N
    has no pole cell.)"""
    N, h = 5, 3
    mesh = M.Mesh(N, h)
    IA = mesh.matrixIA.reshape((2, 2, N + 2 * h, N + 2 * h, 6), order="F")
    lon = mesh.field(mesh.lon)
    c = h + N // 2
    for p, sign in ((4, 1.0), (5, -1.0)):  # panel 5 north pole, panel 6 south pole
        lo = lon[c, c, p]
        if sign > 0:
            want = np.array([[np.cos(lo), -np.sin(lo)], [np.sin(lo), np.cos(lo)]]) * mesh.radius
        else:
            want = np.array([[-np.cos(lo), np.sin(lo)], [np.sin(lo), np.cos(lo)]]) * mesh.radius
        assert np.allclose(IA[:, :, c, c, p], want, rtol=1e-15, atol=0)
    # an off-pole cell: A^-1 is the inverse of A, of order 1/radius
    assert np.max(np.abs(IA[:, :, c + 1, c, 4])) < 1e-5


def test_pole_inverse_option_inverts_a_at_the_poles():
    """CCS_MESH_POLE_INVERSE: the pole cells' A^-1 is the inverse of A (scale 1/radius),
    every other cell unchanged, and odd-N states come out with covariant winds of
    the usual size."""
    N, h = 5, 3
    ref, fix = M.Mesh(N, h), M.Mesh(N, h, pole_inverse=True)
    A = fix.matrixA.reshape((2, 2, -1), order="F")
    IA = fix.matrixIA.reshape((2, 2, -1), order="F")
    pole = np.abs(np.abs(fix.lat) - np.pi / 2) < 1e-12
    pole &= ~fix.corner_mask()
    assert pole.sum() >= 2  # the two pole cells and the halo copies of them
    for c in np.nonzero(pole)[0]:
        assert np.allclose(A[:, :, c] @ IA[:, :, c], np.eye(2), atol=1e-12)
    same = ~pole
    keep = np.repeat(same, 4)
    assert np.array_equal(ref.matrixIA[keep], fix.matrixIA[keep])
    s = M.initial_state(fix, kind=L.CCS_IC_SEEDED, seed=4, lmax_oro=8)
    assert np.max(np.abs(s["u"][~fix.corner_mask()])) < 1e12


# ---- initTestCase's conversion (test_case_mod.F90:38-48) ----------------------

@pytest.mark.parametrize("N,halo", [(8, 3), (20, 4), (33, 5)])
@pytest.mark.parametrize("kind", [L.CCS_IC_CASE2, L.CCS_IC_CASE5, L.CCS_IC_CASE6, L.CCS_IC_SEEDED])
def test_state_from_sphere_matches_oracle_bitwise(N, halo, kind):
    """phiG = phi sqrtG, (u, v) = G IA (zonal, meridional), (uC, vC) = IA (zonal,
    meridional) over the whole array.  The product's ccs_state_from_sphere, which
    makes the initial state of every parity test, equals the oracle's restatement
    bit for bit (corner blocks included)."""
    mesh = M.Mesh(N, halo)
    s = M.initial_state(mesh, kind=kind, seed=5, lmax_oro=8)
    orc = O.Oracle.from_mesh(mesh)
    given = {k: np.full(mesh.ncell, np.nan) for k in O.FIELDS}
    for k in ("phi", "zonal_wind", "meridional_wind"):
        given[k] = s[k]
    orc.set_state(given)
    orc.init_from_sphere(0)
    o = orc.get_state()
    for k in ("phiG", "u", "v", "uC", "vC"):
        assert np.array_equal(s[k].view(np.int64), o[k].view(np.int64)), k
