"""The reference-side bindings of the boundary struct agree with the C header.

INTEGRATION.md gives the Fortran `bind(C)` type a maintainer would add to the reference
(it cannot be compiled here: no Fortran compiler), and camb_gb300/_lib.py the ctypes
mirror the Python side uses.  Both must list CambGpuTables' fields in the header's order
with the same kinds (double, int, pointer, fixed-size double array), or the library reads
the wrong words.  This test parses all three and compares them field by field.
"""
import os
import re

from camb_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_fields(struct):
    text = open(os.path.join(ROOT, "include", "cambgpu.h")).read()
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (struct, struct), text, re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(const\s+)?(double|int|CambGpuModeSpec)\s*(\*?)\s*(.*)", decl, re.S)
        base, ptr, names = m.group(2), m.group(3), m.group(4)
        for name in names.split(","):
            name = name.strip()
            star = ptr or name.startswith("*")
            name = name.lstrip("*").strip()
            arr = re.match(r"(\w+)\[(\d+)\]", name)
            if star:
                out.append((name, "ptr", 1))
            elif arr:
                out.append((arr.group(1), "f8" if base == "double" else "i4", int(arr.group(2))))
            else:
                out.append((name, "f8" if base == "double" else "i4", 1))
    return out


def fortran_fields():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    body = re.search(r"type, bind\(C\) :: CambGpuTables\n(.*?)\n\s*end type", text, re.S).group(1)
    kinds = {"real(c_double)": "f8", "integer(c_int)": "i4", "type(c_ptr)": "ptr"}
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [x.strip() for x in line.split("::")]
        for name in names.split(","):
            name = name.strip()
            arr = re.match(r"(\w+)\((\d+)\)", name)
            out.append((arr.group(1), kinds[kind], int(arr.group(2))) if arr else (name, kinds[kind], 1))
    return out


def ctypes_fields():
    out = []
    for name, t in _lib.CambGpuTables._fields_:
        if hasattr(t, "_length_"):
            out.append((name, "f8", t._length_))
        elif t is _lib.C.c_double:
            out.append((name, "f8", 1))
        elif t is _lib.C.c_int:
            out.append((name, "i4", 1))
        else:
            out.append((name, "ptr", 1))
    return out


def test_fortran_bind_c_type_matches_header():
    h = header_fields("CambGpuTables")
    f = fortran_fields()
    assert len(h) >= 80
    assert [x[0].lower() for x in f] == [x[0].lower() for x in h]
    assert [x[1:] for x in f] == [x[1:] for x in h]


def test_ctypes_mirror_matches_header():
    assert ctypes_fields() == header_fields("CambGpuTables")
