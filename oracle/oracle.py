"""ctypes driver of the CPU FP64 oracle (oracle/ccs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, never by the library.  Parity is unpinned against the
Fortran binary (no Fortran compiler exists here); see the header of ccs_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libccs_oracle.so"
FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind", "phit")

_dp = C.POINTER(C.c_double)
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        sig = {
            "orc_create": (C.c_void_p, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 7),
            "orc_destroy": (None, [C.c_void_p]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
            "orc_set_e_dissipation": (None, [C.c_void_p, C.c_int]),
            "orc_set_operator": (C.c_int, [C.c_void_p, C.c_int]),
            "orc_set_field": (None, [C.c_void_p, C.c_int, C.c_int, _dp]),
            "orc_get_field": (None, [C.c_void_p, C.c_int, C.c_int, _dp]),
            "orc_get_tend": (None, [C.c_void_p, C.c_int, C.c_int, _dp]),
            "orc_spatial_operator": (None, [C.c_void_p, C.c_int, C.c_int]),
            "orc_rk4": (None, [C.c_void_p, C.c_double]),
            "orc_rk3_tvd": (None, [C.c_void_p, C.c_double]),
            "orc_copy_new_to_old": (None, [C.c_void_p]),
            "orc_run": (None, [C.c_void_p, C.c_int, C.c_double, C.c_int]),
            "orc_init_from_sphere": (None, [C.c_void_p, C.c_int]),
            "orc_p2sp": (None, [C.c_void_p, C.c_int]),
            "orc_total_mass": (C.c_double, [C.c_void_p, C.c_int]),
            "orc_total_energy": (C.c_double, [C.c_void_p, C.c_int]),
            "orc_weno_limiter": (C.c_double, [_dp, C.c_int]),
            "orc_fill_halo": (None, [C.c_int, C.c_int, _dp]),
            "orc_fill_jab": (None, [C.c_int, C.c_int, _dp]),
            "orc_derive_metrics": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 16),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def weno_limiter(Q, direction: int) -> float:
    q = np.ascontiguousarray(Q, dtype=np.float64)
    return lib().orc_weno_limiter(_p(q), int(direction))


def fill_halo(N: int, h: int, field: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(field, dtype=np.float64).copy()
    lib().orc_fill_halo(N, h, _p(out))
    return out


def fill_jab(N: int, h: int, jab: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(jab, dtype=np.float64).copy()
    lib().orc_fill_jab(N, h, _p(out))
    return out


def derive_metrics(N, h, radius, omega, lon_deg, lat_deg, x, y, z, jab):
    nc = (N + 2 * h) ** 2 * 6
    out = {k: np.zeros(nc) for k in ("sqrtG", "f", "lon", "lat", "sinlat", "coslat")}
    for k in ("matrixG", "matrixIG", "matrixA", "matrixIA"):
        out[k] = np.zeros(4 * nc)
    rc = lib().orc_derive_metrics(N, h, radius, omega, _p(lon_deg), _p(lat_deg), _p(x), _p(y), _p(z), _p(jab),
                                  _p(out["sqrtG"]), _p(out["matrixG"]), _p(out["matrixIG"]), _p(out["matrixA"]),
                                  _p(out["matrixIA"]), _p(out["f"]), _p(out["lon"]), _p(out["lat"]),
                                  _p(out["sinlat"]), _p(out["coslat"]))
    if rc != 0:
        raise RuntimeError("oracle metric derivation failed")
    return out


class Oracle:
    """The reference step on the CPU: stat(0) -> stat(1) by RK4 / RK3_TVD."""

    def __init__(self, N, halo, dx, dy, sqrtG, matrixG, matrixIG, matrixA, matrixIA, f, phis,
                 e_dissipation: int = 0, threads: int = 0, operator: int = 0):
        L = lib()
        if threads:
            L.orc_set_threads(int(threads))
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (sqrtG, matrixG, matrixIG, matrixA,
                                                                    matrixIA, f, phis)]
        self.ctx = L.orc_create(N, halo, dx, dy, *[_p(a) for a in arrs])
        if not self.ctx:
            raise ValueError("oracle: bad sizes")
        L.orc_set_e_dissipation(self.ctx, int(e_dissipation))
        if L.orc_set_operator(self.ctx, int(operator)) != 0:
            raise ValueError(f"oracle: unknown spatial operator {operator}")
        self.N, self.halo = N, halo
        self.ncell = (N + 2 * halo) ** 2 * 6

    @classmethod
    def from_mesh(cls, mesh, **kw):
        return cls(mesh.N, mesh.halo, mesh.dx, mesh.dy, mesh.sqrtG, mesh.matrixG, mesh.matrixIG, mesh.matrixA,
                   mesh.matrixIA, mesh.f, mesh.phis, **kw)

    def close(self):
        if getattr(self, "ctx", None):
            lib().orc_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, state, slot: int = 0):
        for k, name in enumerate(FIELDS):
            a = np.ascontiguousarray(state[name], dtype=np.float64)
            lib().orc_set_field(self.ctx, slot, k, _p(a))

    def get_state(self, slot: int = 0) -> dict:
        out = {}
        for k, name in enumerate(FIELDS):
            a = np.zeros(self.ncell)
            lib().orc_get_field(self.ctx, slot, k, _p(a))
            out[name] = a
        return out

    def run(self, dt: float, nsteps: int, scheme: str = "RK4"):
        lib().orc_run(self.ctx, 0 if scheme == "RK4" else 1, float(dt), int(nsteps))

    def rk4_once(self, dt: float):
        """RK4(stat(1), stat(0)) without the copy back (stage tendencies stay readable)."""
        lib().orc_rk4(self.ctx, float(dt))

    def get_tend(self, slot: int):
        out = []
        for k in range(3):
            a = np.zeros(self.ncell)
            lib().orc_get_tend(self.ctx, slot, k, _p(a))
            out.append(a)
        return tuple(out)

    def spatial_operator(self, slot: int = 0):
        lib().orc_spatial_operator(self.ctx, slot, -1)
        out = []
        for k in range(3):
            a = np.zeros(self.ncell)
            lib().orc_get_tend(self.ctx, -1, k, _p(a))
            out.append(a)
        return tuple(out)

    def init_from_sphere(self, slot: int = 0):
        lib().orc_init_from_sphere(self.ctx, slot)

    def total_mass(self, slot: int = 0) -> float:
        return lib().orc_total_mass(self.ctx, slot)

    def total_energy(self, slot: int = 0) -> float:
        return lib().orc_total_energy(self.ctx, slot)
