"""Tile variants of the stage kernels and the autotuner: every variant gives the
same bits (FP64 lane: the oracle's), the autotuner leaves the state unchanged and
caches its choice, and batches run one variant per lane group."""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O
from tests.helpers import CHECK_FIELDS, bitwise_equal, max_rel, seeded_case, valid_mask

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("var", [0, 1, 2])
@pytest.mark.parametrize("N", [20, 34])  # partial tiles for every shape; even N (no cell on a pole)
def test_fp64_variants_bitwise_against_oracle(var, N):
    mesh, s, dt = seeded_case(N, 3, seed=4, oro=True)
    g = M.Stepper(mesh, dt, precision="fp64")
    g.set_variant(var)
    assert g.variant[0] == var
    g.set_state(s)
    g.step(2)
    orc = O.Oracle.from_mesh(mesh)
    orc.set_state(s.arrays)
    orc.run(dt, 2)
    a, b = g.get_state(), orc.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(a[k], b[k], m), (var, k, max_rel(a[k], b[k], m))


@pytest.mark.parametrize("N", [40, 64])
def test_mixed_variants_agree_bitwise(N):
    """Both tile shapes with both halo-staging schedules give the same bits."""
    mesh, s, dt = seeded_case(N, 3, seed=6, oro=True)
    out = []
    for var, (tx, ty, _) in enumerate(L.MIXED_VARIANTS):
        g = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000.0 * mesh.gravity)
        g.set_variant(var)
        assert g.variant == (var, tx, ty)
        g.set_state(s)
        g.step(5)
        out.append(g.get_state())
    m = valid_mask(mesh)
    for var in range(1, len(out)):
        for k in CHECK_FIELDS:
            assert bitwise_equal(out[0][k], out[var][k], m), (var, k)


@pytest.mark.parametrize("scheme,ediss,op", [("RK3_TVD", L.CCS_EDISS_RECONSTRUCT, L.CCS_OP_WENO),
                                              ("RK4", L.CCS_EDISS_RECONSTRUCT, L.CCS_OP_WENO),
                                              ("RK3_TVD", L.CCS_EDISS_ZERO, L.CCS_OP_CENTRAL6)])
def test_mixed_variants_agree_bitwise_other_kernels(scheme, ediss, op):
    """Every stage-kind instance of the update phase and the E-flux and central
    operator kernels give the same bits with both tile shapes and both halo-staging
    schedules, on a grid with partial tiles (N = 40)."""
    mesh, s, dt = seeded_case(40, 3, seed=16, oro=True)
    out = []
    for var in range(len(L.MIXED_VARIANTS)):
        g = M.Stepper(mesh, dt, precision="mixed", scheme=scheme, e_dissipation=ediss, operator=op,
                      phi_mean=8000.0 * mesh.gravity)
        g.set_variant(var)
        g.set_state(s)
        g.step(3)
        out.append((g.get_state(), g.spatial_operator()))
    m = valid_mask(mesh)
    for var in range(1, len(out)):
        for k in CHECK_FIELDS:
            assert bitwise_equal(out[0][0][k], out[var][0][k], m), (var, k)
        for a, b in zip(out[0][1], out[var][1]):
            assert np.array_equal(a.view(np.int64), b.view(np.int64)), var


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_autotune_keeps_state_and_caches(precision):
    mesh, s, dt = seeded_case(24, 3, seed=2, oro=False)
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    g = M.Stepper(mesh, dt, precision=precision, **kw)
    g.set_state(s)
    g.step(1)
    before = g.get_state()
    var, times = g.autotune(reps=3, force=True)
    nvar = 3 if precision == "fp64" else len(L.MIXED_VARIANTS)
    assert 0 <= var < nvar and all(t > 0 for t in times[:nvar]) and times[var] == min(times[:nvar])
    assert g.variant[0] == var
    after = g.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(before[k], after[k], m), k
    # a second handle of the same grid reuses the cached choice without timing
    h = M.Stepper(mesh, dt, precision=precision, **kw)
    h.set_state(s)
    var2, times2 = h.autotune(reps=3)
    assert var2 == var and not any(times2)
    # stepping after the switch still matches a default-variant handle
    ref = M.Stepper(mesh, dt, precision=precision, **kw)
    ref.set_state(s)
    h.step(3)
    ref.step(3)
    a, b = h.get_state(), ref.get_state()
    for k in CHECK_FIELDS:
        assert bitwise_equal(a[k], b[k], m), k


def test_batch_runs_one_launch_per_lane_whatever_the_members_variants():
    """Members tuned to different tile variants share one launch per lane and RK
    stage (the group runs one variant for all); ccs_batch_autotune re-picks each
    group's variant by timing its work list; every member equals its single run bit
    for bit before and after."""
    mesh, s, dt = seeded_case(20, 3, seed=8, oro=True)
    kw = dict(phi_mean=8000.0 * mesh.gravity)
    members, lanes = [], []
    for var in (0, 1, 2):
        x = M.Stepper(mesh, dt, precision="fp64")
        x.set_variant(var)
        x.set_state(s)
        members.append(x)
        lanes.append("fp64")
    for var in (1, 0, 3, 2):
        y = M.Stepper(mesh, dt, precision="mixed", **kw)
        y.set_variant(var)
        y.set_state(s)
        members.append(y)
        lanes.append("mixed")
    b = M.Batch(members)
    launches, groups = b.info()
    assert launches == 2
    assert sorted((lane, n) for lane, _, n in groups) == [(L.CCS_FP64, 3), (L.CCS_MIXED, 4)]
    b.step(1)
    b.autotune(reps=2)
    assert b.info()[0] == 2
    b.step(1)
    m = valid_mask(mesh)
    for x, lane in zip(members, lanes):
        r = M.Stepper(mesh, dt, precision=lane, **(kw if lane == "mixed" else {}))
        r.set_state(s)
        r.step(2)
        a, c = x.get_state(), r.get_state()
        for k in CHECK_FIELDS:
            assert bitwise_equal(a[k], c[k], m), (lane, k)


def test_batch_groups_mixed_members_by_operator():
    """Mixed members with the WENO and a central operator run in separate launches
    of one batch and equal their single runs bit for bit."""
    mesh, s, dt = seeded_case(24, 3, seed=21, oro=True)
    kw = dict(phi_mean=8000.0 * mesh.gravity)
    members = []
    for op in (L.CCS_OP_WENO, L.CCS_OP_CENTRAL4, L.CCS_OP_CENTRAL6):
        x = M.Stepper(mesh, 0.5 * dt, precision="mixed", operator=op, **kw)
        x.set_state(s)
        members.append((op, x))
    M.Batch([x for _, x in members]).step(3)
    m = valid_mask(mesh)
    for op, x in members:
        r = M.Stepper(mesh, 0.5 * dt, precision="mixed", operator=op, **kw)
        r.set_state(s)
        r.step(3)
        a, b = x.get_state(), r.get_state()
        for k in CHECK_FIELDS:
            assert bitwise_equal(a[k], b[k], m), (op, k)


def test_batch_members_with_different_halos():
    """One launch per group over members whose arrays have different halo widths
    (3, 4, 5; FP64 and mixed): each member's layout travels in its own stage
    descriptor, and every member equals its single run bit for bit."""
    members, refs = [], []
    for k, (N, halo, lane) in enumerate([(16, 3, "fp64"), (16, 5, "fp64"), (20, 4, "fp64"),
                                         (16, 3, "mixed"), (20, 4, "mixed"), (24, 5, "mixed")]):
        mesh, s, dt = seeded_case(N, halo, seed=60 + k, oro=True)
        kw = dict(phi_mean=8000.0 * mesh.gravity) if lane == "mixed" else {}
        x = M.Stepper(mesh, dt, precision=lane, **kw)
        x.set_state(s)
        r = M.Stepper(mesh, dt, precision=lane, **kw)
        r.set_state(s)
        members.append(x)
        refs.append(r)
    M.Batch(members).step(3)
    for x, r in zip(members, refs):
        r.step(3)
        a, b = x.get_state(), r.get_state()
        m = valid_mask(x.mesh)
        for k in CHECK_FIELDS:
            assert bitwise_equal(a[k], b[k], m), (x.mesh.N, x.mesh.halo, k)
