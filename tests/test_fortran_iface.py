"""The Fortran binding (include/nhw_gpu_iface.F90) against the C header.

A Fortran driver talks to the library through the bind(C) types and
interfaces of that module, so each must match include/nhwave_gb300.h: the
members of every struct in the same order with interoperable kinds, every
enum value, and one interface per entry point with the same number of
arguments.  The struct images built from the Fortran members must also have
the sizes the library reports (nhw_abi_sizes).  No Fortran compiler is
needed: both files are parsed as text.
"""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "nhwave_gb300.h")
F90 = os.path.join(REPO, "include", "nhw_gpu_iface.F90")

C_TO_F = {"int32_t": "c_int32_t", "int64_t": "c_int64_t", "double": "c_double", "float": "c_float"}
CTYPES = {"c_int32_t": ctypes.c_int32, "c_int64_t": ctypes.c_int64, "c_double": ctypes.c_double,
          "c_float": ctypes.c_float}
STRUCTS = ["nhw_params", "nhw_scalars", "nhw_stats", "nhw_ensemble_opts", "nhw_ensemble_info"]


def _header_text():
    s = open(HEADER).read()
    return re.sub(r"/\*.*?\*/", " ", s, flags=re.S)


def _f90_lines():
    out = []
    for ln in open(F90):
        ln = ln.split("!")[0].rstrip()
        if out and out[-1].endswith("&"):
            out[-1] = out[-1][:-1] + " " + ln.strip().lstrip("&")
        else:
            out.append(ln)
    return [ln for ln in out if ln.strip()]


def c_structs():
    """{struct: [(member, kind or struct name, array length)]} from the header."""
    text = _header_text()
    out = {}
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        members = []
        for stmt in m.group(2).split(";"):
            stmt = " ".join(stmt.split())
            if not stmt:
                continue
            typ, rest = stmt.split(" ", 1)
            for d in rest.split(","):
                d = d.strip()
                arr = re.match(r"(\w+)\[(\d+)\]", d)
                name, n = (arr.group(1), int(arr.group(2))) if arr else (d, 1)
                members.append((name.lower(), C_TO_F.get(typ, typ), n))
        out[m.group(3)] = members
    return out


def f90_types():
    out, cur = {}, None
    for ln in _f90_lines():
        s = ln.strip()
        m = re.match(r"type\s*,\s*bind\(C\)\s*::\s*(\w+)", s, flags=re.I)
        if m:
            cur = m.group(1)
            out[cur] = []
            continue
        if cur and re.match(r"end\s+type", s, flags=re.I):
            cur = None
            continue
        if cur:
            decl, names = s.split("::")
            km = re.match(r"(?:integer|real)\((\w+)\)|type\((\w+)\)", decl.strip(), flags=re.I)
            kind = (km.group(1) or km.group(2)).lower()
            for d in names.split(","):
                d = d.strip()
                arr = re.match(r"(\w+)\((\d+)\)", d)
                name, n = (arr.group(1), int(arr.group(2))) if arr else (d, 1)
                out[cur].append((name.lower(), kind, n))
    return out


def c_enums():
    out = {}
    for body in re.findall(r"enum\s+\w+\s*\{(.*?)\}", _header_text(), flags=re.S):
        val = -1
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            if "=" in item:
                name, v = (x.strip() for x in item.split("="))
                val = int(v)
            else:
                name, val = item, val + 1
            out[name] = val
    return out


def f90_parameters():
    out = {}
    for ln in _f90_lines():
        m = re.match(r"\s*integer\(c_int\),\s*parameter\s*::\s*(\w+)\s*=\s*(-?\d+)", ln, flags=re.I)
        if m:
            out[m.group(1)] = int(m.group(2))
    return out


def c_functions():
    """{entry point: number of arguments} of the header's declarations."""
    out = {}
    for m in re.finditer(r"(?:int|const\s+char\s*\*)\s+(nhw_\w+)\s*\(([^)]*)\)\s*;", _header_text()):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def f90_functions():
    out = {}
    for ln in _f90_lines():
        m = re.search(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", ln, flags=re.I)
        if m:
            assert m.group(1).lower() == m.group(3).lower(), ln
            args = m.group(2).strip()
            out[m.group(3)] = 0 if not args else len(args.split(","))
    return out


@pytest.mark.parametrize("struct", STRUCTS)
def test_struct_members_order_and_kinds(struct):
    c, f = c_structs(), f90_types()
    assert struct in c and struct in f
    assert f[struct] == c[struct], "\n".join(
        f"{i}: C {a} / Fortran {b}" for i, (a, b) in enumerate(zip(c[struct], f[struct])) if a != b)


def test_enum_values():
    c, f = c_enums(), f90_parameters()
    missing = sorted(set(c) - set(f))
    assert not missing, f"enum values without a Fortran parameter: {missing}"
    wrong = {k: (c[k], f[k]) for k in c if f[k] != c[k]}
    assert not wrong, wrong


def test_every_entry_point_has_an_interface():
    c, f = c_functions(), f90_functions()
    assert set(c) == set(f), (sorted(set(c) - set(f)), sorted(set(f) - set(c)))
    wrong = {k: (c[k], f[k]) for k in c if c[k] != f[k]}
    assert not wrong, f"argument counts (C, Fortran): {wrong}"
    from nhwave_gb300 import lib
    assert set(c) == set(lib.EXPORTS)


def _ctypes_image(name, types, cache):
    if name in cache:
        return cache[name]
    fields = []
    for member, kind, n in types[name]:
        t = CTYPES.get(kind) or _ctypes_image(kind, types, cache)
        fields.append((member, t * n if n > 1 else t))
    cls = type(name, (ctypes.Structure,), {"_fields_": fields})
    cache[name] = cls
    return cls


def test_fortran_images_have_the_library_sizes(gpu_lib):
    """bind(C) types follow the C layout rules; built from the Fortran
    members they must have the sizes compiled into the library."""
    types, cache = f90_types(), {}
    pb, sb = ctypes.c_int32(0), ctypes.c_int32(0)
    assert gpu_lib.nhw_abi_sizes(ctypes.byref(pb), ctypes.byref(sb)) == 0
    assert ctypes.sizeof(_ctypes_image("nhw_params", types, cache)) == pb.value
    assert ctypes.sizeof(_ctypes_image("nhw_scalars", types, cache)) == sb.value
    from nhwave_gb300 import lib, params
    assert ctypes.sizeof(_ctypes_image("nhw_ensemble_info", types, cache)) == ctypes.sizeof(lib.EnsembleInfo)
    assert ctypes.sizeof(_ctypes_image("nhw_stats", types, cache)) == ctypes.sizeof(lib.NhwStats)
    # and the Python image of nhw_params has the same members in the same order
    assert [n.lower() for n, _ in params.NhwParams._fields_] == [m for m, _, _ in types["nhw_params"]]
