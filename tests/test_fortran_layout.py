"""The Fortran BIND(C) declarations of include/sflow_types.f90 lay out
SflowBC, SflowParams and SflowStepStats exactly as the C header does.

No Fortran compiler exists on the machines this project runs on, so the
offsets a Fortran compiler gives an interoperable derived type are
computed here from the declaration by the C layout rules the standard
prescribes for BIND(C) types (each component at the next multiple of its
alignment, the type padded to its largest alignment), and compared with
offsetof() / sizeof() from a C program compiled against include/sflow.h.
"""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "sflow_types.f90")

SIZES = {"INTEGER(C_INT32_T)": 4, "INTEGER(C_INT64_T)": 8, "REAL(C_DOUBLE)": 8}


def _parameters(text):
    params = {}
    for m in re.finditer(r"PARAMETER\s*::\s*(\w+)\s*=\s*([^\n!]+)", text):
        params[m.group(1)] = eval(m.group(2), {}, dict(params))
    return params


def _types(text):
    """{type name: [(member, kind, element count)]} in declaration order."""
    params = _parameters(text)
    types = {}
    for m in re.finditer(r"TYPE, BIND\(C\) :: (\w+)\n(.*?)END TYPE", text, re.S):
        members = []
        for line in m.group(2).splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            kind, name = [x.strip() for x in line.split("::")]
            count = 1
            dims = re.match(r"(\w+)\((.*)\)$", name)
            if dims:
                name = dims.group(1)
                for d in dims.group(2).split(","):
                    count *= int(eval(d, {}, dict(params)))
            members.append((name, kind, count))
        types[m.group(1)] = members
    return types


def _layout(types, name):
    """Offsets, size and alignment of an interoperable type."""
    off, align, out = 0, 1, {}
    for member, kind, count in types[name]:
        if kind.startswith("TYPE("):
            sub = kind[5:-1]
            _, size, al = _layout(types, sub)
        else:
            size = al = SIZES[kind]
        off = (off + al - 1) // al * al
        out[member] = off
        off += size * count
        align = max(align, al)
    return out, (off + align - 1) // align * align, align


C_NAMES = {"sflow_bc": "SflowBC", "sflow_params": "SflowParams", "sflow_step_stats": "SflowStepStats"}


def _c_offsets(types, tmp_path):
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "sflow.h"', "int main(void) {"]
    for ft, ct in C_NAMES.items():
        lines.append(f'  printf("{ft} sizeof %zu\\n", sizeof({ct}));')
        for member, _, _ in types[ft]:
            lines.append(f'  printf("{ft} {member} %zu\\n", offsetof({ct}, {member}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = {}
    for line in subprocess.check_output([str(exe)]).decode().splitlines():
        t, m, v = line.split()
        out[(t, m)] = int(v)
    return out


def test_fortran_types_match_the_c_structs(tmp_path):
    with open(F90) as f:
        text = f.read()
    types = _types(text)
    assert set(types) == set(C_NAMES)
    c = _c_offsets(types, tmp_path)
    for ft in C_NAMES:
        offs, size, _ = _layout(types, ft)
        assert size == c[(ft, "sizeof")], ft
        for member, off in offs.items():
            assert off == c[(ft, member)], (ft, member, off, c[(ft, member)])


def test_fortran_constants_match_the_header():
    with open(F90) as f:
        params = _parameters(f.read())
    with open(os.path.join(ROOT, "include", "sflow.h")) as f:
        h = f.read()
    for name in ("SFLOW_ABI_VERSION", "SFLOW_MAX_SOLID", "SFLOW_MAX_LEVELS", "SFLOW_MAX_INTERVALS"):
        m = re.search(rf"#define {name} (\d+)", h)
        assert m and int(m.group(1)) == params[name], name
    assert params["SFLOW_MAX_VARS"] == 4 + params["SFLOW_MAX_SOLID"]
