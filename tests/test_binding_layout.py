"""The documented Julia binding against the C ABI's structs.

A Julia `struct` of isbits fields has the C layout of the same fields, so a
`ccall` passing `Ref{Desc}` is right only if the Julia struct lists the
header's fields in the same order with the same widths. This test parses the
Julia structs `Desc`, `TransferDesc` and `Particle` out of INTEGRATION.md, lays
them out by C's rules, and holds every field's name and offset and the
struct's size to (a) the header itself, through a small C program compiled
here that prints `offsetof` and `sizeof` for include/twoldg.h, and (b) the
ctypes structures the Python binding and the tests use. No GPU is needed.
"""
import ctypes
import os
import re
import subprocess

import pytest

from twoldg import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Julia field type -> (size, alignment) under the C layout rules
SCALARS = {"Int32": (4, 4), "Int64": (8, 8), "Float64": (8, 8), "UInt8": (1, 1), "Float32": (4, 4)}

PAIRS = [("Desc", "twoldg_desc", _lib.Desc), ("TransferDesc", "twoldg_transfer_desc", _lib.TransferDesc),
         ("Particle", "twoldg_particle", _lib.Particle)]


def julia_type(t):
    t = t.strip()
    if t.startswith("Ptr{"):
        return 8, 8
    m = re.fullmatch(r"NTuple\{(\d+),(\w+)\}", t.replace(" ", ""))
    if m:
        size, align = SCALARS[m.group(2)]
        return int(m.group(1)) * size, align
    return SCALARS[t]


def julia_structs():
    """{name: [(field, size, align), ...]} of every `struct` in the Julia code blocks."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    code = "\n".join(re.findall(r"```julia\n(.*?)```", text, flags=re.S))
    out = {}
    for m in re.finditer(r"^struct (\w+)(.*?)\bend\b", code, flags=re.S | re.M):
        body = re.sub(r"#[^\n]*", "", m.group(2))
        fields = []
        for part in re.split(r"[;\n]", body):
            part = part.strip()
            if not part:
                continue
            name, typ = part.split("::", 1)
            size, align = julia_type(typ)
            fields.append((name.strip(), size, align))
        out[m.group(1)] = fields
    return out


def c_layout(fields):
    """[(field, offset)], sizeof under C's rules."""
    off, maxal, rows = 0, 1, []
    for name, size, align in fields:
        off = (off + align - 1) // align * align
        rows.append((name, off))
        off += size
        maxal = max(maxal, align)
    return rows, (off + maxal - 1) // maxal * maxal


def header_fields(cname):
    """The field names of `typedef struct cname {...} cname;` in include/twoldg.h, in order."""
    src = open(os.path.join(ROOT, "include", "twoldg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), src, flags=re.S).group(1)
    names = []
    for decl in body.split(";"):
        decl = decl.strip()
        for part in decl.split(",") if decl else []:   # "int32_t nsinh, nmid, ninner"
            names.append(re.search(r"(\w+)\s*(\[\s*\d+\s*\])?$", part.strip()).group(1))
    return names


@pytest.fixture(scope="module")
def header_layout(tmp_path_factory):
    """{c struct: ([(field, offset)], sizeof)} printed by a C program over include/twoldg.h."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "twoldg.h"', "int main(void) {"]
    for _, cname, cty in PAIRS:
        for name in header_fields(cname):
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, name, cname, name))
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
    lines += ["  return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = {}
    for row in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n"):
        if row:
            cname, field, val = row.split()
            rows, size = out.setdefault(cname, ([], [0]))
            if field == "sizeof":
                size[0] = int(val)
            else:
                rows.append((field, int(val)))
    return {k: (rows, size[0]) for k, (rows, size) in out.items()}


@pytest.mark.parametrize("jname,cname,cty", PAIRS, ids=[p[0] for p in PAIRS])
def test_julia_binding_matches_the_header(header_layout, jname, cname, cty):
    structs = julia_structs()
    assert jname in structs, "INTEGRATION.md declares no Julia struct %s" % jname
    rows, size = c_layout(structs[jname])
    hrows, hsize = header_layout[cname]
    assert [r[0] for r in rows] == [r[0] for r in hrows], "field names or order differ from %s" % cname
    assert rows == hrows, "field offsets differ from %s" % cname
    assert size == hsize


@pytest.mark.parametrize("jname,cname,cty", PAIRS, ids=[p[0] for p in PAIRS])
def test_ctypes_binding_matches_the_header(header_layout, jname, cname, cty):
    hrows, hsize = header_layout[cname]
    assert [(n, getattr(cty, n).offset) for n, _ in cty._fields_] == hrows
    assert ctypes.sizeof(cty) == hsize
