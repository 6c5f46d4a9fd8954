"""Error of the mixed-precision lane against the FP64 lane.

Runs the same seeded state through the FP64 lane (bit-for-bit the reference
arithmetic) and the mixed lane and reports, at checkpoints, the L1, L2 and Linf
relative errors of h = phi / g and of the zonal and meridional wind over the
interior cells, and the relative mass and energy drift of each lane.

The reference's WENO limiter switches between weight sets discontinuously
(spatial_operators_mod.F90:348-351), so two runs whose states differ in the last
bits eventually take different branches at some faces; ``--floor`` also runs the
FP64 lane from the same state perturbed by ``--floor-eps`` (relative, in phiG)
and reports that divergence as the floor any non-bitwise lane is measured against.

  python -m conformal_cubed_sphere_gb300.accuracy --N 96 --days 1 --checkpoints 6 --floor
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import _lib as L
from . import model as M


def norms(a: np.ndarray, b: np.ndarray, m: np.ndarray) -> dict:
    d = a[m] - b[m]
    ref = b[m]
    return {"L1": float(np.sum(np.abs(d)) / np.sum(np.abs(ref))),
            "L2": float(np.linalg.norm(d) / np.linalg.norm(ref)),
            "Linf": float(np.max(np.abs(d)) / np.max(np.abs(ref)))}


def compare(mesh: M.Mesh, a: M.State, b: M.State) -> dict:
    m = mesh.interior_mask()
    g = mesh.gravity
    return {"h": norms(a["phi"] / g, b["phi"] / g, m),
            "zonal_wind": norms(a["zonal_wind"], b["zonal_wind"], m),
            "meridional_wind": norms(a["meridional_wind"], b["meridional_wind"], m)}


def run(N: int = 96, days: float = 1.0, checkpoints: int = 4, seed: int = 1, oro: bool = True, cfl: float = 0.5,
        floor: bool = False, floor_eps: float = 1e-9, device: int = 0, max_steps: int | None = None) -> dict:
    mesh = M.Mesh(N, 3)
    s = M.initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=seed, lmax_oro=8 if oro else 0)
    dt = M.cfl_dt(mesh, s, cfl)
    nsteps = int(round(days * 86400.0 / dt))
    if max_steps is not None:
        nsteps = min(nsteps, max_steps)
    f64 = M.Stepper(mesh, dt, precision="fp64", device=device)
    f64.set_state(s)
    mix = M.Stepper(mesh, dt, precision="mixed", device=device, phi_mean=8000.0 * mesh.gravity)
    mix.set_state(s)
    pert = None
    if floor:
        p = s.copy()
        rng = np.random.default_rng(seed + 1000)
        p["phiG"] = p["phiG"] * (1.0 + floor_eps * rng.standard_normal(p["phiG"].shape))
        safe = np.where(mesh.sqrtG > 0, mesh.sqrtG, 1.0)
        p["phi"] = p["phiG"] / safe
        pert = M.Stepper(mesh, dt, precision="fp64", device=device)
        pert.set_state(p)
    m64_0, e64_0 = f64.diag()
    mmx_0, emx_0 = mix.diag()
    marks = sorted(set(max(1, int(round(nsteps * (k + 1) / checkpoints))) for k in range(checkpoints)))
    out = {"N": N, "dt_s": dt, "steps": nsteps, "seed": seed, "orography": oro, "cfl": cfl, "checkpoints": []}
    done = 0
    t_f64 = t_mix = 0.0
    for mk in marks:
        n = mk - done
        t0 = time.perf_counter()
        f64.step(n)
        t1 = time.perf_counter()
        mix.step(n)
        t2 = time.perf_counter()
        if pert is not None:
            pert.step(n)
        t_f64 += t1 - t0
        t_mix += t2 - t1
        done = mk
        a, b = mix.get_state(), f64.get_state()
        row = {"step": done, "hours": done * dt / 3600.0, "mixed_vs_fp64": compare(mesh, a, b)}
        m64, e64 = f64.diag()
        mmx, emx = mix.diag()
        row["mass_drift"] = {"fp64": (m64 - m64_0) / m64_0, "mixed": (mmx - mmx_0) / mmx_0}
        row["energy_drift"] = {"fp64": (e64 - e64_0) / e64_0, "mixed": (emx - emx_0) / emx_0}
        if pert is not None:
            row["fp64_perturbed_vs_fp64"] = compare(mesh, pert.get_state(), b)
        out["checkpoints"].append(row)
    out["wall_s"] = {"fp64": t_f64, "mixed": t_mix}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--N", type=int, default=96)
    ap.add_argument("--days", type=float, default=1.0)
    ap.add_argument("--checkpoints", type=int, default=4)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--flat", action="store_true")
    ap.add_argument("--floor", action="store_true")
    ap.add_argument("--floor-eps", type=float, default=1e-9)
    ap.add_argument("--max-steps", type=int, default=None)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    res = run(a.N, a.days, a.checkpoints, a.seed, not a.flat, floor=a.floor, floor_eps=a.floor_eps,
              max_steps=a.max_steps)
    txt = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)
    print(txt)


if __name__ == "__main__":
    sys.exit(main())
