"""Shared helpers of the test suite (cases, comparisons)."""
from __future__ import annotations

import numpy as np

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O

CHECK_FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind")


def seeded_case(N, halo=3, seed=7, oro=True, kind=L.CCS_IC_SEEDED):
    mesh = M.Mesh(N, halo)
    s = M.initial_state(mesh, kind=kind, seed=seed, lmax_oro=8 if oro else 0)
    dt = M.cfl_dt(mesh, s, 0.5)
    return mesh, s, dt


def valid_mask(mesh):
    """Interior and edge-halo cells (the corner blocks are never written)."""
    return ~mesh.corner_mask()


def max_rel(a, b, mask):
    a, b = a[mask], b[mask]
    scale = np.max(np.abs(b)) or 1.0
    return float(np.max(np.abs(a - b)) / scale)


def bitwise_equal(a, b, mask):
    return np.array_equal(a[mask].view(np.int64), b[mask].view(np.int64))


def oracle_for(mesh, **kw):
    return O.Oracle.from_mesh(mesh, **kw)
