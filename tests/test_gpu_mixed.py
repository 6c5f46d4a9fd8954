"""Mixed-precision lane: errors against the FP64 oracle on the same inputs,
conservation, and batching (ensembles and uneven grids) against single runs."""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O
from tests.helpers import CHECK_FIELDS, bitwise_equal, seeded_case, valid_mask

pytestmark = pytest.mark.gpu


def rel_l2(a, b, m):
    return float(np.linalg.norm(a[m] - b[m]) / np.linalg.norm(b[m]))


@pytest.mark.parametrize("oro", [False, True])
def test_tendency_close_to_fp64(oro):
    mesh, s, dt = seeded_case(32, 3, seed=3, oro=oro)
    g = M.Stepper(mesh, dt, precision="mixed")
    g.set_state(s)
    o = O.Oracle.from_mesh(mesh)
    o.set_state(s.arrays)
    tg, to = g.spatial_operator(), o.spatial_operator()
    im = mesh.interior_mask()
    # tolerance: FP32 differences of O(1e4) geopotentials give ~1e-7 relative
    # errors per face value; the tendency is a difference of faces
    for a, b, tol in zip(tg, to, (2e-4, 2e-4, 2e-4)):
        assert rel_l2(a, b, im) < tol


@pytest.mark.parametrize("oro", [False, True])
def test_short_horizon_error_vs_fp64(oro):
    """Ten steps of C32: the h error stays at FP32 rounding level, well inside the
    1e-6 relative L2 bound."""
    from conformal_cubed_sphere_gb300 import accuracy as A
    res = A.run(N=32, days=1.0, checkpoints=1, seed=1, oro=oro, max_steps=10)
    err = res["checkpoints"][-1]["mixed_vs_fp64"]
    assert err["h"]["L2"] < 1e-6, err
    assert err["zonal_wind"]["L2"] < 1e-4 and err["meridional_wind"]["L2"] < 1e-4, err


def test_error_within_the_fp64_divergence_floor():
    """Over 200 steps the WENO branch switches make any non-bitwise run diverge;
    the mixed lane's h error stays within 2x the divergence of the FP64 lane perturbed
    by one FP32 ulp (6e-8) in phiG (measured ratios 0.9-1.35 at steps 100 and 200 on
    seeds 2 and 3)."""
    from conformal_cubed_sphere_gb300 import accuracy as A
    res = A.run(N=32, days=10.0, checkpoints=2, seed=2, oro=True, floor=True, floor_eps=6e-8, max_steps=200)
    for row in res["checkpoints"]:
        mixed = row["mixed_vs_fp64"]["h"]["L2"]
        floor = row["fp64_perturbed_vs_fp64"]["h"]["L2"]
        assert mixed < 2 * floor, row


def test_mass_drift_small():
    mesh, s, dt = seeded_case(32, 3, seed=4, oro=True)
    g = M.Stepper(mesh, dt, precision="mixed")
    g.set_state(s)
    m0, e0 = g.diag()
    g.step(50)
    m1, e1 = g.diag()
    assert abs(m1 - m0) / abs(m0) < 1e-8


def test_ensemble_batch_equals_members_alone():
    mesh = M.Mesh(24, 3)
    states = [M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=100 + k, h_rms=150 + 25 * k,
                              wind_max=30 + 5 * k) for k in range(4)]
    dt = min(M.cfl_dt(mesh, st, 0.5) for st in states)
    owner = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000 * 9.80616)
    members = [owner] + [M.Stepper(mesh, dt, precision="mixed", share_with=owner, phi_mean=8000 * 9.80616)
                         for _ in range(3)]
    for st, m in zip(states, members):
        m.set_state(st)
    b = M.Batch(members)
    b.step(4)
    msk = valid_mask(mesh)
    for st, m in zip(states, members):
        alone = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000 * 9.80616)
        alone.set_state(st)
        alone.step(4)
        x, y = m.get_state(), alone.get_state()
        for k in ("phiG", "u", "v", "phi"):
            assert bitwise_equal(x[k], y[k], msk), k


def test_uneven_batch_mixed_lanes():
    """Different resolutions, time steps and lanes in one batch: each member's
    result equals its single run bit for bit."""
    specs = [(16, "mixed"), (24, "fp64"), (12, "mixed"), (20, "fp64")]
    members, ref = [], []
    for k, (N, lane) in enumerate(specs):
        mesh = M.Mesh(N, 3)
        st = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=40 + k, lmax_oro=8)
        dt = M.cfl_dt(mesh, st, 0.5)
        a = M.Stepper(mesh, dt, precision=lane)
        a.set_state(st)
        members.append(a)
        b = M.Stepper(mesh, dt, precision=lane)
        b.set_state(st)
        ref.append(b)
    batch = M.Batch(members)
    assert batch.info()[0] == 2  # one launch per lane and RK stage
    batch.step(3)
    for a, b in zip(members, ref):
        b.step(3)
        x, y = a.get_state(), b.get_state()
        msk = valid_mask(a.mesh)
        for k in ("phiG", "u", "v"):
            assert bitwise_equal(x[k], y[k], msk), k


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_async_transfers_match_synchronous_calls(precision):
    """set_state_async / step_async / get_state_async in a loop (double-buffered
    staging, copy streams) give the same bits as the synchronous calls."""
    mesh, s, dt = seeded_case(24, 3, seed=3, oro=True)
    kw = dict(phi_mean=8000.0 * mesh.gravity) if precision == "mixed" else {}
    a = M.Stepper(mesh, dt, precision=precision, **kw)
    b = M.Stepper(mesh, dt, precision=precision, **kw)
    inputs = [s]
    for k in range(3):  # three different inputs: the results of 1, 2, 3 steps
        b.set_state(inputs[-1])
        b.step(1)
        inputs.append(b.get_state())
    outs = [M.State.zeros(mesh) for _ in range(3)]
    for k in range(3):
        a.set_state_async(inputs[k])
        a.step_async(2)
        a.get_state_async(outs[k])
    a.sync()
    m = valid_mask(mesh)
    for k in range(3):
        b.set_state(inputs[k])
        b.step(2)
        ref = b.get_state()
        for f in CHECK_FIELDS:
            assert bitwise_equal(outs[k][f], ref[f], m), (k, f)


def _block_state(mesh, order, fill=None):
    """A State whose fields are consecutive slices of one array, `order` first."""
    names = list(order) + [k for k in M.STATE_FIELDS if k not in order]
    block = np.zeros(len(names) * mesh.ncell)
    st = M.State({k: block[q * mesh.ncell:(q + 1) * mesh.ncell] for q, k in enumerate(names)})
    if fill is not None:
        for k in M.STATE_FIELDS:
            st[k][:] = fill[k]
    return st


@pytest.mark.parametrize("layout", ["one block", "gaps"])
def test_mixed_async_transfers_of_field_blocks(layout):
    """Host fields that are consecutive slices of one block move as merged copies;
    the result equals the per-field copies bit for bit (and a block with the fields
    out of the lane's order, which splits into several runs, too)."""
    mesh, s, dt = seeded_case(24, 3, seed=5, oro=True)
    kw = dict(phi_mean=8000.0 * mesh.gravity)
    a = M.Stepper(mesh, dt, precision="mixed", **kw)
    b = M.Stepper(mesh, dt, precision="mixed", **kw)
    if layout == "one block":
        order_in, order_out = ("phi", "u", "v"), M.STATE_FIELDS
    else:  # u before phi; phi and uC apart
        order_in, order_out = ("u", "v", "phi"), ("phiG", "u", "v", "uC", "phi", "vC", "zonal_wind")
    sin = _block_state(mesh, order_in, fill=s)
    outs = [_block_state(mesh, order_out) for _ in range(2)]
    for k in range(2):
        a.set_state_async(sin)
        a.step_async(1 + k)
        a.get_state_async(outs[k])
    a.sync()
    m = valid_mask(mesh)
    for k in range(2):
        b.set_state(s)
        b.step(1 + k)
        ref = b.get_state()
        for f in CHECK_FIELDS:
            assert bitwise_equal(outs[k][f], ref[f], m), (layout, k, f)


@pytest.mark.parametrize("scheme,halo", [("RK3_TVD", 3), ("RK4", 4), ("RK3_TVD", 5)])
def test_mixed_schemes_and_halos_short_horizon(scheme, halo):
    """Ten steps of C32 with orography for each RK scheme and wider halos: the mixed
    lane stays at FP32 rounding level against the FP64 lane (h relative L2 < 1e-6)."""
    mesh, s, dt = seeded_case(32, halo, seed=2, oro=True)
    mx = M.Stepper(mesh, dt, precision="mixed", scheme=scheme, phi_mean=8000.0 * mesh.gravity)
    f64 = M.Stepper(mesh, dt, precision="fp64", scheme=scheme)
    for g in (mx, f64):
        g.set_state(s)
        g.step(10)
    a, b = mx.get_state(), f64.get_state()
    m = mesh.interior_mask()
    h = lambda st: st["phi"] / mesh.gravity  # noqa: E731
    assert rel_l2(h(a), h(b), m) < 1e-6
    for k in ("zonal_wind", "meridional_wind"):
        assert rel_l2(a[k], b[k], m) < 1e-4, k


def test_mixed_e_reconstruction_close_to_fp64():
    """CCS_EDISS_RECONSTRUCT on the mixed lane against the FP64 lane's: tendency within
    FP32 rounding, ten steps at FP32 rounding level in h."""
    mesh, s, dt = seeded_case(32, 3, seed=8, oro=True)
    mx = M.Stepper(mesh, dt, precision="mixed", e_dissipation=L.CCS_EDISS_RECONSTRUCT,
                   phi_mean=8000.0 * mesh.gravity)
    f64 = M.Stepper(mesh, dt, precision="fp64", e_dissipation=L.CCS_EDISS_RECONSTRUCT)
    for g in (mx, f64):
        g.set_state(s)
    im = mesh.interior_mask()
    for a, b in zip(mx.spatial_operator(), f64.spatial_operator()):
        assert rel_l2(a, b, im) < 2e-4
    # the option changes the answer: the E dissipation is not zero
    z = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000.0 * mesh.gravity)
    z.set_state(s)
    assert rel_l2(z.spatial_operator()[1], mx.spatial_operator()[1], im) > 1e-6
    mx.step(10)
    f64.step(10)
    a, b = mx.get_state(), f64.get_state()
    assert rel_l2(a["phi"], b["phi"], im) < 1e-6


def test_long_run_stays_healthy_and_conserves_mass():
    """Ten thousand steps of C48 (about five simulated days): every cell healthy and
    the mass drift within 1e-9 (FP32 state with compensated updates)."""
    mesh, s, dt = seeded_case(48, 3, seed=12, oro=True)
    g = M.Stepper(mesh, dt, precision="mixed", phi_mean=8000.0 * mesh.gravity)
    g.set_state(s)
    m0, _ = g.diag()
    g.step(10000)
    assert g.check_state() == 0
    m1, _ = g.diag()
    assert abs(m1 - m0) / abs(m0) < 1e-9


def test_member_async_transfers_around_an_async_batch_step():
    """Members' asynchronous uploads, an asynchronous batch step and the members'
    asynchronous downloads, in call order with no synchronisation between them: the
    batch waits for the uploads and the downloads wait for the batch (bit for bit
    the single runs)."""
    mesh = M.Mesh(48, 3)
    first = [M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=80 + k) for k in range(3)]
    inputs = [M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=90 + k, h_rms=220.0) for k in range(3)]
    dt = min(M.cfl_dt(mesh, st, 0.5) for st in first + inputs)
    kw = dict(phi_mean=8000.0 * mesh.gravity)
    lanes = ("mixed", "mixed", "fp64")
    members = [M.Stepper(mesh, dt, precision=lane, **(kw if lane == "mixed" else {})) for lane in lanes]
    for m, st in zip(members, first):
        m.set_state(st)
    batch = M.Batch(members)
    for m, st in zip(members, inputs):
        m.set_state_async(st)
    batch.step_async(2)
    outs = [M.State.zeros(mesh) for _ in members]
    for m, o in zip(members, outs):
        m.get_state_async(o)
    for m in members:
        m.sync()
    msk = valid_mask(mesh)
    for lane, st, o in zip(lanes, inputs, outs):
        r = M.Stepper(mesh, dt, precision=lane, **(kw if lane == "mixed" else {}))
        r.set_state(st)
        r.step(2)
        ref = r.get_state()
        for k in CHECK_FIELDS:
            assert bitwise_equal(o[k], ref[k], msk), (lane, k)
