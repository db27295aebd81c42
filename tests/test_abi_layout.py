"""Layout of the C ABI's structs as the three sides see them: the C header (offsetof and sizeof
from a small program compiled with gcc against include/heatflow_gb300.h), the ctypes mirror
(heatflow_gb300/abi.py), and the Fortran iso_c_binding types that INTEGRATION.md gives for the
reference's host program (the module that replaces the simulate call at src/heatflow.f90:83).

No Fortran compiler exists on either machine, so the Fortran side is checked by laying out the
bind(C) field lists parsed from INTEGRATION.md with the C rules that interoperable derived types
follow (each component at the next multiple of its alignment, the type padded to the largest
alignment).  No GPU."""
import ctypes as C
import json
import os
import re
import shutil
import subprocess

import pytest

from heatflow_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (size, alignment) of the iso_c_binding kinds the binding uses
KINDS = {"integer(c_int64_t)": (8, 8), "real(c_double)": (8, 8), "type(c_ptr)": (8, 8),
         "integer(c_int32_t)": (4, 4), "integer(c_int)": (4, 4)}
TYPES = ("hf_problem", "hf_solver_opts", "hf_stats")


def fortran_types():
    """{type: [(field, element kind, count)]} of the bind(C) types in INTEGRATION.md."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", text, re.S):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, names = [p.strip() for p in line.split("::")]
            kind = re.sub(r"\s+", "", kind)
            assert kind in KINDS, (m.group(1), kind)
            for nm in re.findall(r"(\w+)(?:\((\d+)\))?", names):
                fields.append((nm[0].lower(), kind, int(nm[1]) if nm[1] else 1))
        out[m.group(1).lower()] = fields
    return out


def c_layout(fields):
    """(offsets {field: offset}, size) under the C rules for interoperable derived types."""
    off, align_max, offsets = 0, 1, {}
    for name, kind, count in fields:
        size, align = KINDS[kind]
        off = (off + align - 1) // align * align
        offsets[name] = off
        off += size * count
        align_max = max(align_max, align)
    return offsets, (off + align_max - 1) // align_max * align_max


@pytest.fixture(scope="module")
def header_layout(tmp_path_factory):
    """offsetof / sizeof of every field the Fortran types name, from the real header."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    ft = fortran_types()
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "heatflow_gb300.h"',
             "int main(void) {", '  printf("{");']
    first = True
    for t in TYPES:
        lines.append(f'  printf("{"" if first else ","}\\"{t}\\": {{\\"sizeof\\": %zu", sizeof({t}));')
        first = False
        for name, _, _ in ft[t]:
            lines.append(f'  printf(", \\"{name}\\": %zu", offsetof({t}, {name}));')
        lines.append('  printf("}");')
    lines += ['  printf("}\\n");', "  return 0;", "}"]
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return json.loads(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)


def test_fortran_types_present():
    ft = fortran_types()
    assert set(TYPES) <= set(ft)
    # every field of the C structs is named by the Fortran type, in the same order
    for t, cls in (("hf_problem", abi.HfProblem), ("hf_solver_opts", abi.HfSolverOpts),
                   ("hf_stats", abi.HfStats)):
        assert [f[0] for f in ft[t]] == [f[0] for f in cls._fields_], t


@pytest.mark.parametrize("t", TYPES)
def test_fortran_layout_matches_header(header_layout, t):
    offsets, size = c_layout(fortran_types()[t])
    got = dict(header_layout[t])
    assert got.pop("sizeof") == size, t
    assert got == offsets, t


@pytest.mark.parametrize("t,cls", [("hf_problem", abi.HfProblem),
                                   ("hf_solver_opts", abi.HfSolverOpts),
                                   ("hf_stats", abi.HfStats)])
def test_ctypes_layout_matches_header(header_layout, t, cls):
    got = dict(header_layout[t])
    assert C.sizeof(cls) == got.pop("sizeof"), t
    assert {name: getattr(cls, name).offset for name, _ in cls._fields_} == got, t
