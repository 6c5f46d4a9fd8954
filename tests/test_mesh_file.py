"""Raw-binary mesh file (the NetCDF mesh file's attributes and cell-centre
variables, for machines without libnetcdf): round trip, metric derived from a
loaded file, and rejection of foreign, truncated or mismatched files."""
import ctypes as C

import numpy as np
import pytest

from conformal_cubed_sphere_gb300 import _lib as L
from conformal_cubed_sphere_gb300 import model as M


def test_round_trip_is_bitwise(tmp_path):
    a = M.Mesh(12, 3)
    path = tmp_path / "c12.ccsmesh"
    a.save(path)
    assert path.stat().st_size == 64 + 8 * (5 + 6) * 12 * 12 * 6
    b = M.Mesh.from_file(path, halo=4)
    assert b.N == 12 and b.cube_map == "conformal"
    for k in a.file:
        assert np.array_equal(a.file[k].view(np.int64), b.file[k].view(np.int64)), k
    # the derived metric of the loaded samples equals the generated mesh's (halo 4 vs 3
    # changes only the array frame)
    c = M.Mesh(12, 4)
    for name in ("sqrtG", "matrixG", "matrixIG", "matrixA", "matrixIA", "f"):
        assert np.array_equal(getattr(b, name), getattr(c, name)), name


def test_header_attributes(tmp_path):
    path = tmp_path / "g8.ccsmesh"
    M.Mesh(8, 3, cube_map="gnomonic").save(path)
    raw = path.read_bytes()
    assert raw[:8] == b"CCSMESH\x01"
    iv = np.frombuffer(raw[8:48], dtype="<i4")
    assert list(iv) == [1, 8, L.CCS_MAP_GNOMONIC_EQUIANGULAR, 1, 17, 1, 17, 1, 6, 0]
    dv = np.frombuffer(raw[48:64], dtype="<f8")
    assert list(dv) == [90.0 / 8, 90.0 / 8]
    n, m = C.c_int(), C.c_int()
    assert L.lib().ccs_mesh_file_info(str(path).encode(), C.byref(n), C.byref(m)) == 0
    assert (n.value, m.value) == (8, L.CCS_MAP_GNOMONIC_EQUIANGULAR)


def _load(path, N):
    n = N * N * 6
    bufs = [np.zeros(n) for _ in range(5)] + [np.zeros(6 * n)]
    ptrs = [b.ctypes.data_as(C.POINTER(C.c_double)) for b in bufs]
    return L.lib().ccs_mesh_load(str(path).encode(), N, *ptrs)


@pytest.mark.parametrize("damage", ["magic", "truncate", "extra", "version", "index"])
def test_bad_files_rejected(tmp_path, damage):
    path = tmp_path / "m.ccsmesh"
    M.Mesh(6, 3).save(path)
    raw = bytearray(path.read_bytes())
    if damage == "magic":
        raw[0:1] = b"X"
    elif damage == "truncate":
        raw = raw[:-8]
    elif damage == "extra":
        raw += b"\0"
    elif damage == "version":
        raw[8:12] = np.array([2], dtype="<i4").tobytes()
    else:
        raw[24:28] = np.array([99], dtype="<i4").tobytes()  # ide
    path.write_bytes(bytes(raw))
    assert _load(path, 6) == L.CCS_ERR_IO


def test_missing_file_and_size_mismatch(tmp_path):
    assert _load(tmp_path / "absent", 6) == L.CCS_ERR_IO
    path = tmp_path / "m.ccsmesh"
    M.Mesh(6, 3).save(path)
    assert _load(path, 7) == L.CCS_ERR_ARG
    with pytest.raises(L.CCSError):
        M.Mesh.from_file(tmp_path / "absent")
