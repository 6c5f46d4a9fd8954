"""Seeded benchmark inputs for the CPU oracle, made without the GPU library.

TEST INFRASTRUCTURE ONLY: used by the reference arm of bench.py (and checked by
tests/), never by the library.  libccs_setup.so is the host set-up code of the
package (conformal cubic mesh, read_mesh's metric derivation io_mod.F90:119-306,
the seeded initial state and initTestCase's conversion test_case_mod.F90:38-48,
the CFL step) compiled for the CPU alone by oracle/Makefile, so that a process
timing the oracle maps no file of the CUDA library.  The arrays equal the ones
conformal_cubed_sphere_gb300.model makes through libccs_gpu.so, bit for bit (the
same source and flags; tests/test_reference_inputs.py).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libccs_setup.so"

CCS_MAP_CONFORMAL = 1
CCS_IC_SEEDED = 100
RADIUS, GRAVITY, OMEGA = 6.371e6, 9.80616, 7.292e-5

_dp = C.POINTER(C.c_double)
_lib = None


class _MeshView(C.Structure):
    _fields_ = [(n, _dp) for n in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis")]


STATE_FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind", "phit")


class _StateView(C.Structure):
    _fields_ = [(n, _dp) for n in STATE_FIELDS]


class _ICParams(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("lmax_h", C.c_int), ("lmax_psi", C.c_int), ("lmax_oro", C.c_int),
        ("seed", C.c_uint64),
        ("h0", C.c_double), ("h_rms", C.c_double), ("wind_max", C.c_double),
        ("oro_rms", C.c_double), ("oro_max", C.c_double),
    ]


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE), str(Path("_build") / "libccs_setup.so")], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"set-up library build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        sig = {
            "ccs_mesh_generate": (C.c_int, [C.c_int, C.c_int] + [_dp] * 6),
            "ccs_mesh_derive": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double] + [_dp] * 16),
            "ccs_initial_condition": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                                C.POINTER(_ICParams)] + [_dp] * 8),
            "ccs_state_from_sphere": (C.c_int, [C.c_int, C.c_int, C.POINTER(_MeshView), C.POINTER(_StateView)]),
            "ccs_cfl_dt": (C.c_double, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                        C.POINTER(_MeshView), C.POINTER(_StateView)]),
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


class SetupMesh:
    """The metric arrays of an N x N x 6 conformal cubed sphere (the attributes the
    oracle reads: N, halo, dx, dy, sqrtG, matrixG, matrixIG, matrixA, matrixIA, f,
    phis)."""

    def __init__(self, N: int, halo: int = 3, radius: float = RADIUS, omega: float = OMEGA,
                 gravity: float = GRAVITY):
        lib()
        self.N, self.halo = int(N), int(halo)
        self.radius, self.omega, self.gravity = float(radius), float(omega), float(gravity)
        self.nh = self.N + 2 * self.halo
        self.ncell = self.nh * self.nh * 6
        n = self.N * self.N * 6
        f = {k: np.zeros(n) for k in ("lon", "lat", "x", "y", "z")}
        f["jab"] = np.zeros(6 * n)
        if _lib.ccs_mesh_generate(self.N, CCS_MAP_CONFORMAL, _p(f["lon"]), _p(f["lat"]), _p(f["x"]),
                                  _p(f["y"]), _p(f["z"]), _p(f["jab"])) != 0:
            raise RuntimeError("ccs_mesh_generate failed")
        nc = self.ncell
        self.sqrtG = np.zeros(nc)
        self.matrixG, self.matrixIG = np.zeros(4 * nc), np.zeros(4 * nc)
        self.matrixA, self.matrixIA = np.zeros(4 * nc), np.zeros(4 * nc)
        self.f = np.zeros(nc)
        self.lon, self.lat, self.sinlat, self.coslat = (np.zeros(nc) for _ in range(4))
        if _lib.ccs_mesh_derive(self.N, self.halo, self.radius, self.omega, _p(f["lon"]), _p(f["lat"]),
                                _p(f["x"]), _p(f["y"]), _p(f["z"]), _p(f["jab"]), _p(self.sqrtG),
                                _p(self.matrixG), _p(self.matrixIG), _p(self.matrixA), _p(self.matrixIA),
                                _p(self.f), _p(self.lon), _p(self.lat), _p(self.sinlat), _p(self.coslat)) != 0:
            raise RuntimeError("ccs_mesh_derive failed")
        # dx = dy = (90/N) degrees in radians (io_mod.F90:54-55)
        self.dx = (90.0 / self.N) * (np.pi / 180.0)
        self.dy = self.dx
        self.phis = np.zeros(nc)

    def view(self) -> _MeshView:
        mv = _MeshView()
        for name in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis"):
            setattr(mv, name, _p(getattr(self, name)))
        return mv


def seeded_state(mesh: SetupMesh, seed: int = 1, h0: float = 8000.0, h_rms: float = 200.0,
                 wind_max: float = 40.0, lmax_h: int = 12, lmax_psi: int = 12, lmax_oro: int = 0,
                 oro_rms: float = 1000.0, oro_max: float = 2000.0) -> dict:
    """The seeded state (sets mesh.phis), as the package's initial_state makes it."""
    p = _ICParams(kind=CCS_IC_SEEDED, lmax_h=lmax_h, lmax_psi=lmax_psi, lmax_oro=lmax_oro, seed=seed, h0=h0,
                  h_rms=h_rms, wind_max=wind_max, oro_rms=oro_rms, oro_max=oro_max)
    s = {k: np.zeros(mesh.ncell) for k in STATE_FIELDS}
    if lib().ccs_initial_condition(mesh.N, mesh.halo, mesh.radius, mesh.gravity, mesh.omega, C.byref(p),
                                   _p(mesh.lon), _p(mesh.lat), _p(mesh.sinlat), _p(mesh.coslat), _p(s["phi"]),
                                   _p(s["zonal_wind"]), _p(s["meridional_wind"]), _p(mesh.phis)) != 0:
        raise RuntimeError("ccs_initial_condition failed")
    sv = _StateView()
    for k in STATE_FIELDS:
        setattr(sv, k, _p(s[k]))
    mv = mesh.view()
    if lib().ccs_state_from_sphere(mesh.N, mesh.halo, C.byref(mv), C.byref(sv)) != 0:
        raise RuntimeError("ccs_state_from_sphere failed")
    return s


def cfl_dt(mesh: SetupMesh, state: dict, cfl: float = 0.5) -> float:
    sv = _StateView()
    for k in STATE_FIELDS:
        setattr(sv, k, _p(state[k]))
    mv = mesh.view()
    dt = lib().ccs_cfl_dt(mesh.N, mesh.halo, cfl, mesh.dx, mesh.dy, C.byref(mv), C.byref(sv))
    if not dt > 0:
        raise ValueError("CFL time step undefined")
    return dt


def seeded_case(N: int, halo: int = 3, seed: int = 1, lmax_oro: int = 8, cfl: float = 0.5):
    """(mesh, state, dt) of the benchmark's seeded case with orography."""
    mesh = SetupMesh(N, halo)
    s = seeded_state(mesh, seed=seed, lmax_oro=lmax_oro)
    return mesh, s, cfl_dt(mesh, s, cfl)
