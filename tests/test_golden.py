"""Golden fixtures (tests/golden): digests of the oracle's results on small cases.

The reference has no golden vectors and cannot run here, so the fixtures are the
oracle's own results (tests/golden/make_golden.py).  They pin the oracle and the
host set-up code against unintended change, and the FP64 lane must reproduce them
bit for bit.  Every case also stores its inputs as arrays (golden_inputs.npz), so that
the checks run on any machine, whatever its libm makes of the mesh generator's and
the initial states' sin, cos and atan2."""
import hashlib
import json
import platform
from pathlib import Path

import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"
G = json.loads((GOLDEN / "golden.json").read_text())
FIELDS = ("phiG", "u", "v", "phi", "uC", "vC", "zonal_wind", "meridional_wind")
MESH_FIELDS = ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f", "phis")


def digest(a, mask=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return hashlib.sha256((a[mask] if mask is not None else a).tobytes()).hexdigest()


def regenerate(rec):
    mesh = M.Mesh(rec["N"], rec["halo"])
    s = M.initial_state(mesh, **rec["ic"])
    return mesh, s


class StoredMesh:
    """The stored inputs' mesh, with the attributes Stepper and the oracle read."""

    def __init__(self, z):
        N, halo, dx, dy, dt, radius, gravity, omega = z["scalars"]
        self.N, self.halo = int(N), int(halo)
        self.dx, self.dy, self.dt = float(dx), float(dy), float(dt)
        self.radius, self.gravity, self.omega = float(radius), float(gravity), float(omega)
        self.nh = self.N + 2 * self.halo
        self.ncell = self.nh * self.nh * 6
        for k in MESH_FIELDS:
            setattr(self, k, np.ascontiguousarray(z[f"mesh_{k}"]))

    def view(self):
        mv = L.MeshView()
        for k in MESH_FIELDS:
            setattr(mv, k, getattr(self, k).ctypes.data_as(L._dp))
        return mv

    def corner_mask(self):
        return M.Mesh.corner_mask(self)

    def interior_mask(self):
        return M.Mesh.interior_mask(self)

    def field(self, a):
        return M.Mesh.field(self, a)


def stored_case(name):
    z = np.load(GOLDEN / "golden_inputs.npz")
    mesh = StoredMesh({k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")})
    s = M.State({k: np.ascontiguousarray(z[f"{name}/state_{k}"]) if k in FIELDS else np.zeros(mesh.ncell)
                 for k in M.STATE_FIELDS})
    return mesh, s, G["cases"][name]


@pytest.mark.parametrize("name", sorted(G["cases"]))
def test_stored_inputs_match_their_digests(name):
    mesh, s, rec = stored_case(name)
    m = ~mesh.corner_mask()
    m4 = np.repeat(m, 4)
    for k in MESH_FIELDS:
        assert digest(getattr(mesh, k), m4 if k.startswith("matrix") else m) == rec["mesh"][k], k
    for k in FIELDS:
        assert digest(s[k], m) == rec["input"][k], k
    assert mesh.dt == rec["dt"]


@pytest.mark.parametrize("name", sorted(G["cases"]))
def test_oracle_reproduces_the_stored_case(name):
    mesh, s, rec = stored_case(name)
    orc = O.Oracle(mesh.N, mesh.halo, mesh.dx, mesh.dy, *[getattr(mesh, k) for k in MESH_FIELDS],
                   e_dissipation=rec["e_dissipation"], operator=rec["operator"])
    orc.set_state(s.arrays)
    im = mesh.interior_mask()
    for k, t in zip(("phiG", "u", "v"), orc.spatial_operator()):
        assert digest(t, im) == rec["tendency"][k], k
    orc.run(mesh.dt, rec["steps"], rec["scheme"])
    g = orc.get_state()
    m = ~mesh.corner_mask()
    for k in FIELDS:
        assert digest(g[k], m) == rec["output"][k], k


@pytest.mark.skipif(platform.machine() != G["machine"], reason="digests of the host generator recorded on "
                    + G["machine"] + "; another libm may round its sin/cos/atan2 differently")
@pytest.mark.parametrize("name", sorted(G["cases"]))
def test_host_setup_and_oracle_reproduce_golden(name):
    rec = G["cases"][name]
    mesh, s = regenerate(rec)
    m = ~mesh.corner_mask()
    m4 = np.repeat(m, 4)
    for k in MESH_FIELDS:
        assert digest(getattr(mesh, k), m4 if k.startswith("matrix") else m) == rec["mesh"][k], k
    for k in FIELDS:
        assert digest(s[k], m) == rec["input"][k], k
    orc = O.Oracle.from_mesh(mesh, e_dissipation=rec["e_dissipation"], operator=rec["operator"])
    orc.set_state(s.arrays)
    orc.run(rec["dt"], rec["steps"], rec["scheme"])
    g = orc.get_state()
    for k in FIELDS:
        assert digest(g[k], m) == rec["output"][k], (name, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(G["cases"]))
def test_fp64_lane_reproduces_golden(name):
    """The FP64 lane steps each case's stored inputs to the golden digests: the
    spatial operator's tendencies and the state after the case's steps."""
    mesh, s, rec = stored_case(name)
    gpu = M.Stepper(mesh, mesh.dt, precision="fp64", scheme=rec["scheme"], e_dissipation=rec["e_dissipation"],
                    operator=rec["operator"])
    gpu.set_state(s)
    im = mesh.interior_mask()
    for k, t in zip(("phiG", "u", "v"), gpu.spatial_operator()):
        assert digest(t, im) == rec["tendency"][k], (name, k)
    gpu.step(rec["steps"])
    g = gpu.get_state()
    m = ~mesh.corner_mask()
    for k in FIELDS:
        assert digest(g[k], m) == rec["output"][k], (name, k)
