"""Writes golden.json: SHA-256 digests (and a few values) of the oracle's results on
small seeded cases, plus digests of the host generator's mesh and initial state, and
golden_inputs.npz: every case's mesh and initial state as arrays.

The reference has no tests, fixtures or golden vectors and cannot be built here
(Fortran + NetCDF), so these fixtures are the oracle's own results: they pin the
oracle and the host set-up code against unintended change, and the GPU tests check
the CUDA path against the same digests.  Regenerate only when a change of the
numbers is intended:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from conformal_cubed_sphere_gb300 import _lib as L  # noqa: E402
from conformal_cubed_sphere_gb300 import model as M  # noqa: E402

FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind")
MESH_FIELDS = ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis")

# (name, N, halo, initial state, scheme, e_dissipation, operator, steps)
CASES = [
    ("seeded_rk4", 6, 3, dict(kind=L.CCS_IC_SEEDED, seed=11, lmax_oro=8), "RK4", 0, 0, 3),
    ("case6_rk3_reconstruct", 6, 4, dict(kind=L.CCS_IC_CASE6), "RK3_TVD", 1, 0, 2),
    ("seeded_central4", 8, 3, dict(kind=L.CCS_IC_SEEDED, seed=12, lmax_oro=0), "RK4", 0, 4, 2),
    ("case5_rk4", 10, 3, dict(kind=L.CCS_IC_CASE5), "RK4", 0, 0, 2),
]


def digest(a: np.ndarray, mask: np.ndarray | None = None) -> str:
    a = np.ascontiguousarray(a, dtype=np.float64)
    if mask is not None:
        a = a[mask]
    return hashlib.sha256(a.tobytes()).hexdigest()


def case_inputs(N, halo, ic):
    mesh = M.Mesh(N, halo)
    s = M.initial_state(mesh, **ic)
    dt = float(int(M.cfl_dt(mesh, s, 0.5)))  # whole seconds, as namelist settings are
    return mesh, s, dt


def valid_mask(mesh, width=1):
    m = ~mesh.corner_mask()
    return np.repeat(m, width) if width > 1 else m


def main():
    from oracle import oracle as O
    import platform
    out = {"note": "oracle results (not the Fortran reference, which cannot run here); see make_golden.py",
           "machine": platform.machine(), "cases": {}}
    for name, N, halo, ic, scheme, ediss, op, steps in CASES:
        mesh, s, dt = case_inputs(N, halo, ic)
        m = valid_mask(mesh)
        rec = {"N": N, "halo": halo, "ic": {k: int(v) for k, v in ic.items()}, "scheme": scheme,
               "e_dissipation": ediss, "operator": op, "steps": steps, "dt": dt,
               "mesh": {k: digest(getattr(mesh, k), valid_mask(mesh, 4) if k.startswith("matrix") else m)
                        for k in MESH_FIELDS},
               "input": {k: digest(s[k], m) for k in FIELDS}}
        orc = O.Oracle.from_mesh(mesh, e_dissipation=ediss, operator=op)
        orc.set_state(s.arrays)
        im = mesh.interior_mask()
        rec["tendency"] = {k: digest(t, im) for k, t in zip(("phiG", "u", "v"), orc.spatial_operator())}
        orc.run(dt, steps, scheme)
        g = orc.get_state()
        rec["output"] = {k: digest(g[k], m) for k in FIELDS}
        c = (halo + N // 2) + (N + 2 * halo) * (halo + N // 2)  # a cell near the centre of panel 1
        rec["sample"] = {k: float(g[k][c]) for k in ("phiG", "u", "v")}
        out["cases"][name] = rec
    (HERE / "golden.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "golden.json")
    # every case's inputs as arrays, so that a machine whose libm rounds the
    # generator's sin/cos/atan2 differently still steps exactly these inputs
    arrays = {}
    for name, N, halo, ic, scheme, ediss, op, steps in CASES:
        mesh, s, dt = case_inputs(N, halo, ic)
        arrays.update({f"{name}/mesh_{k}": getattr(mesh, k) for k in MESH_FIELDS})
        arrays.update({f"{name}/state_{k}": s[k] for k in FIELDS})
        arrays[f"{name}/scalars"] = np.array([N, halo, mesh.dx, mesh.dy, dt, mesh.radius, mesh.gravity,
                                              mesh.omega])
    np.savez_compressed(HERE / "golden_inputs.npz", **arrays)
    print("wrote", HERE / "golden_inputs.npz")

if __name__ == "__main__":
    main()
