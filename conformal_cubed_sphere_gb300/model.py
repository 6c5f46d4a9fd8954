"""Host-side API over the C ABI: mesh, initial state and the GPU step.

Mirrors the reference driver (dynamic_core/src/ccsm.F90): ``Mesh`` stands for
read_mesh (io_mod.F90:15-307) on the arrays of the host mesh generator, ``State``
for stat_field (stat_mod.F90:7-17), ``initial_state`` for initTestCase
(test_case_mod.F90:13-58) and ``Stepper`` for the time loop body
(RK4 / RK3_TVD + copyStat, ccsm.F90:50-67).  All arrays are numpy float64 in the
reference's Fortran order, flattened: cell fields are (N+2h, N+2h, 6).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L

PI = np.pi
D2R = PI / 180.0

# planet constants of the benchmark cases: a = 6.371e6 m (the reference's
# constants_mod.F90:9 has 6371229 m; Mesh(radius=...) takes either), g and Omega as
# constants_mod.F90:6,12
RADIUS = 6.371e6
GRAVITY = 9.80616
OMEGA = 7.292e-5

STATE_FIELDS = L.STATE_FIELDS


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Mesh:
    """Metric arrays of an N x N x 6 cubed sphere with `halo` ghost cells."""

    def __init__(self, N: int, halo: int = 3, radius: float = RADIUS, omega: float = OMEGA,
                 gravity: float = GRAVITY, phis: np.ndarray | None = None, cube_map: str = "conformal",
                 mesh_file: str | None = None, pole_inverse: bool = False):
        lib = L.lib()
        if mesh_file is not None:
            fn, fmap = C.c_int(), C.c_int()
            L.check(lib.ccs_mesh_file_info(str(mesh_file).encode(), C.byref(fn), C.byref(fmap)),
                    "ccs_mesh_file_info")
            N = fn.value
            cube_map = {L.CCS_MAP_CONFORMAL: "conformal", L.CCS_MAP_GNOMONIC_EQUIANGULAR: "gnomonic"}.get(
                fmap.value, "file")
        self.N, self.halo = int(N), int(halo)
        self.cube_map = cube_map
        self.radius, self.omega, self.gravity = float(radius), float(omega), float(gravity)
        self.nh = self.N + 2 * self.halo
        self.ncell = self.nh * self.nh * 6
        n = self.N * self.N * 6
        self.file = {k: np.zeros(n) for k in ("lon", "lat", "x", "y", "z")}
        self.file["jab"] = np.zeros(6 * n)
        f = self.file
        if mesh_file is not None:
            L.check(lib.ccs_mesh_load(str(mesh_file).encode(), self.N, _ptr(f["lon"]), _ptr(f["lat"]),
                                      _ptr(f["x"]), _ptr(f["y"]), _ptr(f["z"]), _ptr(f["jab"])), "ccs_mesh_load")
        else:
            kind = {"conformal": L.CCS_MAP_CONFORMAL, "gnomonic": L.CCS_MAP_GNOMONIC_EQUIANGULAR}[cube_map]
            L.check(lib.ccs_mesh_generate(self.N, kind, _ptr(f["lon"]), _ptr(f["lat"]),
                                          _ptr(f["x"]), _ptr(f["y"]), _ptr(f["z"]), _ptr(f["jab"])),
                    "ccs_mesh_generate")
        nc = self.ncell
        self.sqrtG = np.zeros(nc)
        self.matrixG = np.zeros(4 * nc)
        self.matrixIG = np.zeros(4 * nc)
        self.matrixA = np.zeros(4 * nc)
        self.matrixIA = np.zeros(4 * nc)
        self.f = np.zeros(nc)
        self.lon = np.zeros(nc)
        self.lat = np.zeros(nc)
        self.sinlat = np.zeros(nc)
        self.coslat = np.zeros(nc)
        # pole_inverse: A^-1 of a cell centred on a pole (odd N) by inversion instead of
        # the reference's analytic formula (ccs_mesh_derive_ex, CCS_MESH_POLE_INVERSE)
        flags = L.CCS_MESH_POLE_INVERSE if pole_inverse else 0
        L.check(lib.ccs_mesh_derive_ex(self.N, self.halo, self.radius, self.omega, flags, _ptr(f["lon"]),
                                       _ptr(f["lat"]), _ptr(f["x"]), _ptr(f["y"]), _ptr(f["z"]), _ptr(f["jab"]),
                                       _ptr(self.sqrtG), _ptr(self.matrixG), _ptr(self.matrixIG),
                                       _ptr(self.matrixA), _ptr(self.matrixIA), _ptr(self.f), _ptr(self.lon),
                                       _ptr(self.lat), _ptr(self.sinlat), _ptr(self.coslat)), "ccs_mesh_derive")
        # dx = dy = (90/N) degrees in radians, as io_mod.F90:54-55 converts them
        self.dx = (90.0 / self.N) * D2R
        self.dy = self.dx
        self.phis = np.zeros(nc) if phis is None else np.ascontiguousarray(phis, dtype=np.float64)

    @classmethod
    def from_file(cls, path, halo: int = 3, **kw) -> "Mesh":
        """The mesh of a raw-binary mesh file (ccs_mesh_load), metric derived as
        read_mesh does (io_mod.F90:119-306)."""
        return cls(0, halo, mesh_file=path, **kw)

    def save(self, path) -> None:
        """Writes the generator samples as a raw-binary mesh file (ccs_mesh_save);
        Mesh(mesh_file=path, halo=...) reads it back."""
        f = self.file
        kind = {"conformal": L.CCS_MAP_CONFORMAL, "gnomonic": L.CCS_MAP_GNOMONIC_EQUIANGULAR}.get(self.cube_map, -1)
        L.check(L.lib().ccs_mesh_save(str(path).encode(), self.N, kind, _ptr(f["lon"]), _ptr(f["lat"]),
                                      _ptr(f["x"]), _ptr(f["y"]), _ptr(f["z"]), _ptr(f["jab"])), "ccs_mesh_save")

    def view(self) -> L.MeshView:
        mv = L.MeshView()
        for name in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis"):
            setattr(mv, name, _ptr(getattr(self, name)))
        return mv

    def field(self, a: np.ndarray) -> np.ndarray:
        """(i, j, panel) view of a flattened cell field."""
        return a.reshape((self.nh, self.nh, 6), order="F")

    def interior_mask(self) -> np.ndarray:
        m = np.zeros((self.nh, self.nh, 6), dtype=bool, order="F")
        h, N = self.halo, self.N
        m[h:h + N, h:h + N, :] = True
        return m.reshape(-1, order="F")

    def corner_mask(self) -> np.ndarray:
        """True on the never-filled h x h corner blocks."""
        idx = np.arange(self.nh) - self.halo + 1
        out_i = (idx < 1) | (idx > self.N)
        c = out_i[:, None] & out_i[None, :]
        return np.repeat(c[:, :, None], 6, axis=2).reshape(-1, order="F")


@dataclass
class State:
    """stat_field: nine (N+2h)^2 x 6 arrays."""
    arrays: dict = field(default_factory=dict)

    @classmethod
    def zeros(cls, mesh: Mesh) -> "State":
        return cls({k: np.zeros(mesh.ncell) for k in STATE_FIELDS})

    def __getitem__(self, k):
        return self.arrays[k]

    def __setitem__(self, k, v):
        self.arrays[k] = v

    def save(self, path, mesh: "Mesh") -> None:
        """Checkpoint file of this state (ccs_state_write)."""
        sv = self.view()
        L.check(L.lib().ccs_state_write(str(path).encode(), mesh.N, mesh.halo, C.byref(sv)), "ccs_state_write")

    @classmethod
    def load(cls, path, mesh: "Mesh") -> "State":
        """A state from a checkpoint file of this mesh's size (ccs_state_read)."""
        st = cls.zeros(mesh)
        sv = st.view()
        L.check(L.lib().ccs_state_read(str(path).encode(), mesh.N, mesh.halo, C.byref(sv)), "ccs_state_read")
        return st

    def copy(self) -> "State":
        return State({k: v.copy() for k, v in self.arrays.items()})

    def view(self, fields=STATE_FIELDS) -> L.StateView:
        sv = L.StateView()
        for k in fields:
            setattr(sv, k, _ptr(self.arrays[k]))
        return sv


def initial_state(mesh: Mesh, kind: int = L.CCS_IC_SEEDED, seed: int = 1, h0: float = 8000.0,
                  h_rms: float = 200.0, wind_max: float = 40.0, lmax_h: int = 12, lmax_psi: int = 12,
                  lmax_oro: int = 0, oro_rms: float = 1000.0, oro_max: float = 2000.0) -> State:
    """initTestCase equivalent: sets mesh.phis and returns stat(old)."""
    lib = L.lib()
    p = L.ICParams(kind=kind, lmax_h=lmax_h, lmax_psi=lmax_psi, lmax_oro=lmax_oro, seed=seed, h0=h0,
                   h_rms=h_rms, wind_max=wind_max, oro_rms=oro_rms, oro_max=oro_max)
    s = State.zeros(mesh)
    L.check(lib.ccs_initial_condition(mesh.N, mesh.halo, mesh.radius, mesh.gravity, mesh.omega, C.byref(p),
                                      _ptr(mesh.lon), _ptr(mesh.lat), _ptr(mesh.sinlat), _ptr(mesh.coslat),
                                      _ptr(s["phi"]), _ptr(s["zonal_wind"]), _ptr(s["meridional_wind"]),
                                      _ptr(mesh.phis)), "ccs_initial_condition")
    mv, sv = mesh.view(), s.view()
    L.check(lib.ccs_state_from_sphere(mesh.N, mesh.halo, C.byref(mv), C.byref(sv)), "ccs_state_from_sphere")
    return s


def cfl_dt(mesh: Mesh, state: State, cfl: float = 0.5) -> float:
    mv, sv = mesh.view(), state.view()
    dt = L.lib().ccs_cfl_dt(mesh.N, mesh.halo, cfl, mesh.dx, mesh.dy, C.byref(mv), C.byref(sv))
    if not dt > 0:
        raise ValueError("CFL time step undefined (non-positive depth?)")
    return dt


def ghost_map(N: int, halo: int) -> np.ndarray:
    nh = N + 2 * halo
    out = np.zeros(nh * nh * 6, dtype=np.int64)
    L.check(L.lib().ccs_ghost_map(N, halo, out.ctypes.data_as(C.POINTER(C.c_int64))), "ccs_ghost_map")
    return out


def ensemble_member_state(mesh: Mesh, k: int, seed: int = 1, lmax_oro: int = 0) -> State:
    """Member k of a seeded ensemble: seed + k, perturbation RMS drawn uniformly in
    150-250 m and maximum wind in 30-50 m/s from the member's own generator."""
    rng = np.random.default_rng(seed + k)
    h_rms = float(rng.uniform(150.0, 250.0))
    wind = float(rng.uniform(30.0, 50.0))
    return initial_state(mesh, kind=L.CCS_IC_SEEDED, seed=seed + k, h_rms=h_rms, wind_max=wind,
                         lmax_oro=lmax_oro)


class Stepper:
    """One instance of the GPU step (a ccs_handle)."""

    def __init__(self, mesh: Mesh, dt: float, precision: str = "fp64", scheme: str = "RK4",
                 e_dissipation: int = L.CCS_EDISS_ZERO, device: int = 0, phi_mean: float = 0.0,
                 share_with: "Stepper | None" = None, operator: int = L.CCS_OP_WENO):
        self.mesh = mesh
        self.dt = float(dt)
        self.precision = "fp64" if precision == "fp64" else "mixed"
        cfg = L.Config(N=mesh.N, halo=mesh.halo, scheme=L.CCS_RK4 if scheme == "RK4" else L.CCS_RK3_TVD,
                       precision=L.CCS_FP64 if precision == "fp64" else L.CCS_MIXED,
                       e_dissipation=e_dissipation, device=device, dx=mesh.dx, dy=mesh.dy, dt=self.dt,
                       radius=mesh.radius, gravity=mesh.gravity, omega=mesh.omega, phi_mean=phi_mean)
        self._cfg = cfg
        self._pending = []  # host arrays of async transfers, held until sync()
        h = C.c_void_p()
        lib = L.lib()
        if share_with is None:
            mv = mesh.view()
            L.check(lib.ccs_init(C.byref(cfg), C.byref(mv), C.byref(h)), "ccs_init")
        else:
            L.check(lib.ccs_init_shared(C.byref(cfg), share_with.handle, C.byref(h)), "ccs_init_shared")
        self.handle = h
        if operator != L.CCS_OP_WENO:
            self.set_operator(operator)

    def set_operator(self, op: int):
        """The spatial operator (CCS_OP_WENO or CCS_OP_CENTRAL2/4/6), either lane."""
        L.check(L.lib().ccs_set_operator(self.handle, int(op)), "ccs_set_operator", self.handle)

    def autotune(self, reps: int = 5, force: bool = False):
        """Picks the fastest tile variant of this lane for this grid (ccs_autotune);
        returns (variant, per-variant mean launch times in us, 0 where not timed)."""
        v = C.c_int()
        t = (C.c_double * L.CCS_MAX_VARIANTS)()
        L.check(L.lib().ccs_autotune(self.handle, int(reps), int(bool(force)), C.byref(v), t), "ccs_autotune",
                self.handle)
        return v.value, list(t)

    def set_variant(self, var: int):
        L.check(L.lib().ccs_set_variant(self.handle, int(var)), "ccs_set_variant", self.handle)

    @property
    def variant(self):
        """(variant, tile_x, tile_y) of this handle's stage kernel."""
        v, tx, ty = C.c_int(), C.c_int(), C.c_int()
        L.check(L.lib().ccs_get_variant(self.handle, C.byref(v), C.byref(tx), C.byref(ty)), "ccs_get_variant")
        return v.value, tx.value, ty.value

    def close(self):
        if self.handle:
            L.lib().ccs_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, s: State):
        sv = s.view()
        L.check(L.lib().ccs_set_state(self.handle, C.byref(sv)), "ccs_set_state", self.handle)

    def get_state(self, out: State | None = None) -> State:
        out = out if out is not None else State.zeros(self.mesh)
        sv = out.view()
        L.check(L.lib().ccs_get_state(self.handle, C.byref(sv)), "ccs_get_state", self.handle)
        return out

    def set_state_async(self, s: State):
        """ccs_set_state_async: the arrays of `s` are held until sync()."""
        sv = s.view()
        L.check(L.lib().ccs_set_state_async(self.handle, C.byref(sv)), "ccs_set_state_async", self.handle)
        self._pending.append(s)

    def get_state_async(self, out: State) -> State:
        """ccs_get_state_async into `out` (valid after sync())."""
        sv = out.view()
        L.check(L.lib().ccs_get_state_async(self.handle, C.byref(sv)), "ccs_get_state_async", self.handle)
        self._pending.append(out)
        return out

    def step(self, nsteps: int = 1):
        L.check(L.lib().ccs_step(self.handle, int(nsteps)), "ccs_step", self.handle)

    def step_async(self, nsteps: int = 1):
        L.check(L.lib().ccs_step_async(self.handle, int(nsteps)), "ccs_step_async", self.handle)

    def sync(self):
        L.check(L.lib().ccs_sync(self.handle), "ccs_sync", self.handle)
        self._pending.clear()

    def spatial_operator(self):
        n = self.mesh.ncell
        t = [np.zeros(n) for _ in range(3)]
        L.check(L.lib().ccs_spatial_operator(self.handle, _ptr(t[0]), _ptr(t[1]), _ptr(t[2])),
                "ccs_spatial_operator", self.handle)
        return tuple(t)

    def check_state(self) -> int:
        """Interior cells with non-positive depth or non-finite wind (ccs_check_state)."""
        n = C.c_int64()
        rc = L.lib().ccs_check_state(self.handle, C.byref(n))
        if rc not in (L.CCS_OK, L.CCS_ERR_NAN):
            L.check(rc, "ccs_check_state", self.handle)
        return n.value

    def courant(self) -> float:
        """Courant number of the current state (ccs_courant); inf when a cell has
        non-positive depth or a non-finite value."""
        c = C.c_double()
        rc = L.lib().ccs_courant(self.handle, C.byref(c))
        if rc == L.CCS_ERR_NAN:
            return float("inf")
        L.check(rc, "ccs_courant", self.handle)
        return c.value

    def diag(self):
        m, e = C.c_double(), C.c_double()
        L.check(L.lib().ccs_diag(self.handle, C.byref(m), C.byref(e)), "ccs_diag", self.handle)
        return m.value, e.value

    @property
    def stream_ptr(self) -> int:
        """The cudaStream_t of this handle (for torch.cuda.ExternalStream)."""
        return L.lib().ccs_stream(self.handle) or 0

    def timing(self, enable: int = -1, reset: int = 0):
        ms, n = C.c_double(), C.c_int64()
        L.check(L.lib().ccs_timing(self.handle, enable, reset, C.byref(ms), C.byref(n)), "ccs_timing")
        return ms.value, n.value


class Batch:
    """Members advanced together: one launch per group (lane, RK scheme, operator
    family, E-flux option) and RK stage."""

    def __init__(self, members: list[Stepper]):
        self.members = members
        arr = (C.c_void_p * len(members))(*[m.handle for m in members])
        b = C.c_void_p()
        L.check(L.lib().ccs_batch_create(arr, len(members), C.byref(b)), "ccs_batch_create")
        self.handle = b

    def _check(self, status: int, where: str):
        if status != L.CCS_OK:
            raise L.CCSError(status, where, (L.lib().ccs_batch_last_error(self.handle) or b"").decode())

    def step(self, nsteps: int = 1):
        self._check(L.lib().ccs_batch_step(self.handle, int(nsteps)), "ccs_batch_step")

    def step_async(self, nsteps: int = 1):
        self._check(L.lib().ccs_batch_step_async(self.handle, int(nsteps)), "ccs_batch_step_async")

    def autotune(self, reps: int = 3):
        """Times each group's tile variants on its own work list and keeps the fastest
        (ccs_batch_autotune)."""
        self._check(L.lib().ccs_batch_autotune(self.handle, int(reps)), "ccs_batch_autotune")

    def info(self):
        """(launches per RK stage, [(lane, tile variant, members) per group])."""
        n = C.c_int()
        L.check(L.lib().ccs_batch_info(self.handle, C.byref(n), 0, None, None, None), "ccs_batch_info")
        lane, var, mem = (C.c_int * n.value)(), (C.c_int * n.value)(), (C.c_int * n.value)()
        L.check(L.lib().ccs_batch_info(self.handle, C.byref(n), n.value, lane, var, mem), "ccs_batch_info")
        return n.value, [(lane[q], var[q], mem[q]) for q in range(n.value)]

    @property
    def stream_ptr(self) -> int:
        return L.lib().ccs_batch_stream(self.handle) or 0

    def close(self):
        if self.handle:
            L.lib().ccs_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
