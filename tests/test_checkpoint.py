"""Checkpoint files: round trip of a state, rejection of mismatched or damaged files,
and a bitwise resume of the FP64 lane."""
import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M
from tests.helpers import CHECK_FIELDS, bitwise_equal, seeded_case, valid_mask


def test_round_trip_is_bitwise(tmp_path):
    mesh, s, dt = seeded_case(10, 3, seed=2, oro=True)
    path = tmp_path / "c10.ccsstate"
    s.save(path, mesh)
    assert path.stat().st_size == 24 + 8 * 8 * mesh.ncell
    back = M.State.load(path, mesh)
    for k in CHECK_FIELDS:
        assert np.array_equal(s[k].view(np.int64), back[k].view(np.int64)), k


def test_mismatch_and_damage_rejected(tmp_path):
    mesh, s, dt = seeded_case(10, 3, seed=2, oro=False)
    path = tmp_path / "c10.ccsstate"
    s.save(path, mesh)
    with pytest.raises(L.CCSError, match="invalid argument"):
        M.State.load(path, M.Mesh(12, 3))
    with pytest.raises(L.CCSError):
        M.State.load(path, M.Mesh(10, 4))
    raw = path.read_bytes()
    (tmp_path / "short").write_bytes(raw[:-8])
    (tmp_path / "magic").write_bytes(b"X" + raw[1:])
    for bad in ("short", "magic", "absent"):
        with pytest.raises(L.CCSError):
            M.State.load(tmp_path / bad, mesh)


@pytest.mark.gpu
def test_fp64_resume_is_bitwise(tmp_path):
    """Six steps, checkpoint, a fresh handle from the file, six more steps: the same
    bits as twelve steps in one go."""
    mesh, s, dt = seeded_case(24, 3, seed=6, oro=True)
    a = M.Stepper(mesh, dt, precision="fp64")
    a.set_state(s)
    a.step(6)
    path = tmp_path / "mid.ccsstate"
    a.get_state().save(path, mesh)
    b = M.Stepper(mesh, dt, precision="fp64")
    b.set_state(M.State.load(path, mesh))
    b.step(6)
    a.step(6)
    x, y = a.get_state(), b.get_state()
    m = valid_mask(mesh)
    for k in CHECK_FIELDS:
        assert bitwise_equal(x[k], y[k], m), k
