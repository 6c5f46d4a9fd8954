"""The Fortran binding (include/ccs_gpu_mod.F90) against the C ABI it binds.

No Fortran compiler exists on the build or GPU machines, so the binding cannot be
compiled here; these checks read its source.  Every bind(C) entry point must be
declared in include/ccs_gpu.h with the same number of arguments and exported by
libccs_gpu.so; every bind(C) type must list the C struct's fields in order with the
interoperable kinds; every CCS_* constant must have the header's value."""
import re
from pathlib import Path

import pytest

from conformal_cubed_sphere_gb300 import _lib as L

ROOT = Path(__file__).resolve().parents[1]
F90 = (ROOT / "include" / "ccs_gpu_mod.F90").read_text()
HDR = (ROOT / "include" / "ccs_gpu.h").read_text()


def _strip_f90_comments(text):
    return "\n".join(line.split("!", 1)[0] for line in text.splitlines())


def _strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


SRC = _strip_f90_comments(F90)
CHDR = _strip_c_comments(HDR)


def fortran_procedures():
    """{bind name: number of dummy arguments}"""
    out = {}
    pat = re.compile(r"(?:function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*C\s*,\s*name\s*=\s*'(\w+)'\s*\)",
                     re.I)
    for m in pat.finditer(SRC):
        args = [a for a in m.group(2).replace("&", " ").split(",") if a.strip()]
        out[m.group(3)] = len(args)
    return out


def c_prototypes():
    """{function name: number of parameters} of the header's prototypes"""
    out = {}
    for m in re.finditer(r"^[\w\s\*]*?\b(ccs_\w+)\s*\(([^;{]*?)\)\s*;", CHDR, flags=re.M | re.S):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_every_bound_procedure_is_declared_and_exported():
    procs = fortran_procedures()
    assert len(procs) >= 20
    protos = c_prototypes()
    lib = L.lib()
    for name, nargs in procs.items():
        assert name in protos, f"{name} is not declared in ccs_gpu.h"
        assert protos[name] == nargs, (name, protos[name], nargs)
        assert hasattr(lib, name), f"{name} is not exported by libccs_gpu.so"


def test_the_drop_in_calls_are_bound():
    """The calls the driver change at ccsm.F90:50-67 needs."""
    procs = fortran_procedures()
    for name in ("ccs_init", "ccs_set_state", "ccs_get_state", "ccs_step", "ccs_diag", "ccs_destroy",
                 "ccs_strerror"):
        assert name in procs, name


_KIND = {"int": "integer(c_int)", "double": "real(c_double)", "uint64_t": "integer(c_int64_t)"}


def c_struct_fields(name):
    m = re.search(r"typedef\s+struct\s+" + name + r"\s*\{(.*?)\}\s*" + name + r"\s*;", CHDR, flags=re.S)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        decl = decl.replace("const ", "")
        base, rest = decl.split(" ", 1)
        for item in rest.split(","):
            item = item.strip()
            kind = "type(c_ptr)" if item.startswith("*") else _KIND[base]
            fields.append((kind, item.lstrip("*").strip()))
    return fields


def fortran_type_fields(name):
    m = re.search(r"type\s*,\s*bind\s*\(\s*C\s*\)\s*::\s*" + name + r"\s*\n(.*?)end\s+type", SRC, flags=re.S | re.I)
    assert m, name
    fields = []
    for line in m.group(1).splitlines():
        line = line.strip()
        if not line:
            continue
        kind, names = line.split("::")
        for n in names.split(","):
            fields.append((kind.strip().lower().replace(" ", ""), n.strip()))
    return fields


@pytest.mark.parametrize("name", ["ccs_config", "ccs_mesh_view", "ccs_state_view"])
def test_bound_types_follow_the_c_structs(name):
    assert fortran_type_fields(name) == c_struct_fields(name)


def test_constants_match_the_header():
    f = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(CCS_\w+)\s*=\s*(-?\d+)", SRC)}
    c = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(CCS_\w+)\s*=\s*(-?\d+)", CHDR)}
    assert len(f) >= 20
    for k, v in f.items():
        assert c.get(k) == v, k
