"""Small cases run in a process that loaded the bounds-checked library (CCS_GPU_LIB):
both lanes, every tile variant, partial tiles, halos from 3 to the panel width, both
RK schemes, the E-flux options, the central operators, the tendency entry point,
transfers and a batch.  Exits non-zero at the first recorded out-of-range index or
at a state that the health check rejects (the checked build poisons each tile's
shared arrays with NaN, so a read of a never-written slot would show there).
The FP64 results are also checked bit for bit against the oracle on one case, so
the checked build is known to compute what the normal build computes."""
import ctypes as C
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

from conformal_cubed_sphere_gb300 import _lib as L  # noqa: E402
from conformal_cubed_sphere_gb300 import model as M  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import CHECK_FIELDS, bitwise_equal, seeded_case, valid_mask  # noqa: E402


def hits(tag):
    site, idx = C.c_int(0), C.c_int64(0)
    L.check(L.lib().ccs_debug_bounds(C.byref(site), C.byref(idx)), "ccs_debug_bounds")
    if site.value != 0:
        raise SystemExit(f"{tag}: out-of-range index {idx.value} at check site {site.value}")


def healthy(stepper, tag):
    """The checked build fills each tile's shared arrays with NaN before use, so a
    read of a slot the tile never wrote would reach the state as NaN."""
    nbad = stepper.check_state()
    if nbad:
        raise SystemExit(f"{tag}: {nbad} cells non-finite or of non-positive depth")


def main():
    lib = L.lib()
    if not str(L.LIB_PATH).endswith("bounds/libccs_gpu.so"):
        raise SystemExit(f"not the bounds-checked library: {L.LIB_PATH}")
    rc = lib.ccs_debug_bounds_selftest()
    if rc != L.CCS_OK:
        raise SystemExit(f"selftest of the recording path failed: {rc}")
    hits("start")
    cases = [(4, 3), (4, 4), (6, 6), (8, 3), (20, 4), (24, 5), (33, 3)]
    for N, halo in cases:
        pole = N % 2 == 1
        mesh = M.Mesh(N, halo, pole_inverse=pole)
        s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=N, lmax_oro=8)
        dt = M.cfl_dt(mesh, s, 0.5)
        kw = dict(phi_mean=8000.0 * mesh.gravity)
        for var in (0, 1, 2):
            for scheme, ediss in (("RK4", 0), ("RK3_TVD", 1)):
                g = M.Stepper(mesh, dt, precision="fp64", scheme=scheme, e_dissipation=ediss)
                g.set_variant(var)
                g.set_state(s)
                g.step(2)
                g.spatial_operator()
                g.get_state()
                hits(f"fp64 C{N} h{halo} tile {var} {scheme} ediss {ediss}")
                healthy(g, f"fp64 C{N} h{halo} tile {var} {scheme} ediss {ediss}")
        for var in range(len(L.MIXED_VARIANTS)):
            for scheme, ediss, op in (("RK4", 0, L.CCS_OP_WENO), ("RK3_TVD", 1, L.CCS_OP_WENO),
                                      ("RK4", 0, L.CCS_OP_CENTRAL4)):
                g = M.Stepper(mesh, dt, precision="mixed", scheme=scheme, e_dissipation=ediss, operator=op, **kw)
                g.set_variant(var)
                g.set_state(s)
                g.step(2)
                g.spatial_operator()
                g.get_state()
                g.diag()
                hits(f"mixed C{N} h{halo} tile {var} {scheme} ediss {ediss} op {op}")
                healthy(g, f"mixed C{N} h{halo} tile {var} {scheme} ediss {ediss} op {op}")
    # a batch over both lanes and several halo widths
    members = []
    for k, (N, halo, lane) in enumerate([(8, 3, "fp64"), (20, 4, "mixed"), (6, 6, "mixed"), (4, 4, "fp64")]):
        mesh, s, dt = seeded_case(N, halo, seed=70 + k)
        x = M.Stepper(mesh, dt, precision=lane, **(dict(phi_mean=8000.0 * mesh.gravity) if lane == "mixed" else {}))
        x.set_state(s)
        members.append(x)
    M.Batch(members).step(2)
    hits("batch")
    for x in members:
        healthy(x, "batch")
    # the checked build computes what the normal build does: FP64 bitwise with the oracle
    mesh, s, dt = seeded_case(20, 4, seed=3)
    g = M.Stepper(mesh, dt, precision="fp64")
    g.set_state(s)
    g.step(2)
    o = O.Oracle.from_mesh(mesh)
    o.set_state(s.arrays)
    o.run(dt, 2)
    a, b = g.get_state(), o.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        if not bitwise_equal(a[k], b[k], m):
            raise SystemExit(f"bounds-checked FP64 lane differs from the oracle in {k}")
    hits("parity")
    print("bounds-checked cases clean:", len(cases), "grids")


if __name__ == "__main__":
    main()
