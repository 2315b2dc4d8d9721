"""The ctypes mirror of the C ABI's structs has the header's layout (no device needed).

A probe compiled with gcc against include/molgpu.h prints sizeof and offsetof of every field of
every struct the ABI passes by pointer; the ctypes Structures that the Python binding (and the
tests) hand to the library must agree field for field.
"""
import ctypes as C
import json
import os
import shutil
import subprocess

import pytest

from molgpu import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = [L.mol_op1d, L.mol_term, L.mol_bc, L.mol_instr, L.mol_problem_desc, L.mol_stats]


def _probe_source():
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "molgpu.h"', "int main(void) {",
             '    printf("{");']
    first = True
    for S in STRUCTS:
        name = S.__name__
        sep = "" if first else ","
        first = False
        lines.append(f'    printf("{sep}\\"{name}\\": {{\\"size\\": %zu", sizeof({name}));')
        for fname, _ in S._fields_:
            lines.append(f'    printf(", \\"{fname}\\": %zu", offsetof({name}, {fname}));')
        lines.append('    printf("}");')
    lines += ['    printf("}\\n");', "    return 0;", "}"]
    return "\n".join(lines) + "\n"


def test_ctypes_structs_match_the_header(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not found")
    src = tmp_path / "probe.c"
    src.write_text(_probe_source())
    exe = tmp_path / "probe"
    subprocess.run([gcc, "-std=c11", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    got = json.loads(subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout)
    for S in STRUCTS:
        c = got[S.__name__]
        assert C.sizeof(S) == c["size"], (S.__name__, C.sizeof(S), c["size"])
        for fname, _ in S._fields_:
            assert getattr(S, fname).offset == c[fname], (S.__name__, fname, getattr(S, fname).offset, c[fname])


JULIA_TO_C = {"MolOp1d": L.mol_op1d, "MolTerm": L.mol_term, "MolBC": L.mol_bc, "MolInstr": L.mol_instr,
              "MolProblemDesc": L.mol_problem_desc, "MolStats": L.mol_stats}
_PRIM = {"Int32": (4, 4), "UInt16": (2, 2), "Int64": (8, 8), "Float64": (8, 8)}


def _julia_structs():
    """Field lists of the immutable structs of the Julia shim in INTEGRATION.md."""
    import re
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = text[text.index("```julia"):]
    block = block[:block.index("\n```\n")]
    block = "\n".join(line.split("#", 1)[0] for line in block.splitlines())
    out = {}
    for m in re.finditer(r"(?<!mutable )struct\s+(\w+)(.*?)\bend\b", block, re.S):
        fields = [f.strip() for f in re.split(r"[;\n]", m.group(2)) if "::" in f]
        out[m.group(1)] = [tuple(s.strip() for s in f.split("::", 1)) for f in fields]
    return out


def _julia_layout(structs, name, memo):
    """(size, alignment, field offsets) under C layout rules (isbits structs, natural alignment)."""
    if name in memo:
        return memo[name]
    import re

    def size_align(ty):
        if ty in _PRIM:
            return _PRIM[ty]
        if ty.startswith("Ptr{"):
            return 8, 8
        m = re.fullmatch(r"NTuple\{(\d+),\s*(.+)\}", ty)
        if m:
            s, a = size_align(m.group(2))
            return int(m.group(1)) * s, a
        s, a, _ = _julia_layout(structs, ty, memo)
        return s, a

    off, align, offs = 0, 1, []
    for _, ty in structs[name]:
        s, a = size_align(ty)
        off = (off + a - 1) // a * a
        offs.append(off)
        off += s
        align = max(align, a)
    memo[name] = ((off + align - 1) // align * align, align, offs)
    return memo[name]


def _julia_kind(ty):
    """int / uint / float / ptr / struct of a Julia field type (element type for NTuple)."""
    import re
    m = re.fullmatch(r"NTuple\{\d+,\s*(.+)\}", ty)
    if m:
        return _julia_kind(m.group(1))
    if ty.startswith("Ptr{"):
        return "ptr"
    return {"Int32": "int", "Int64": "int", "UInt16": "uint", "Float64": "float"}.get(ty, "struct")


def _ctypes_kind(t):
    while hasattr(t, "_length_"):      # arrays: their element type
        t = t._type_
    if isinstance(t, type) and issubclass(t, C.Structure):
        return "struct"
    if hasattr(t, "contents"):
        return "ptr"
    if t in (C.c_double, C.c_float):
        return "float"
    if t in (C.c_uint16, C.c_uint32, C.c_uint64):
        return "uint"
    return "int"


def test_julia_shim_structs_match_the_ctypes_layout():
    """The Julia shim's structs lay out like the header's (checked above through
    ctypes): same size, the same field offsets and the same kind of value (signed or unsigned
    integer, floating point, pointer, struct) field by field."""
    structs = _julia_structs()
    assert set(JULIA_TO_C) <= set(structs), sorted(structs)
    memo = {}
    for jname, S in JULIA_TO_C.items():
        size, _, offs = _julia_layout(structs, jname, memo)
        assert size == C.sizeof(S), (jname, size, C.sizeof(S))
        assert offs == [getattr(S, f).offset for f, _ in S._fields_], jname
        kinds = [_julia_kind(ty) for _, ty in structs[jname]]
        assert kinds == [_ctypes_kind(t) for _, t in S._fields_], (jname, kinds)


def _jl_class(ty):
    ty = ty.strip()
    if ty in ("Cint", "Int32"):
        return "i32"
    if ty == "Int64":
        return "i64"
    if ty == "Float64":
        return "f64"
    if ty == "Cstring" or ty.startswith(("Ptr{", "Ref{")):
        return "ptr"
    raise AssertionError(f"unmapped Julia type {ty}")


def _ct_class(t):
    if t in (C.c_int, C.c_int32):
        return "i32"
    if t == C.c_int64:
        return "i64"
    if t == C.c_double:
        return "f64"
    if t in (C.c_void_p, C.c_char_p) or hasattr(t, "contents"):
        return "ptr"
    raise AssertionError(f"unmapped ctypes type {t}")


def test_julia_shim_ccalls_match_the_prototypes():
    """Every ccall of the Julia shim names an exported entry point with the return type and the
    argument types (32/64-bit integer, double, pointer) of its prototype."""
    import re
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    block = text[text.index("```julia"):]
    block = block[:block.index("\n```\n")]
    calls = re.findall(r"ccall\(\(:(\w+),\s*lib\),\s*(\w+),\s*\((.*?)\),", block, re.S)
    assert len(calls) >= 10
    for name, ret, args in calls:
        assert name in L._PROTOS, name
        cret, cargs = L._PROTOS[name]
        types = [a for a in (s.strip() for s in args.split(",")) if a]
        assert _jl_class(ret) == _ct_class(cret), (name, ret)
        assert [_jl_class(a) for a in types] == [_ct_class(a) for a in cargs], (name, types)
