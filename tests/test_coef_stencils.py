"""Coefficient stencils in the generated code (no device needed): which problems get them,
the two forms' statements, and NVRTC compiles of both for sm_103a."""
import ctypes as C

import pytest

from molgpu import Descriptor, lower, problems
from molgpu import _lib as L


def _source(name, kw, flags=0):
    sys_, disc, _ = getattr(problems, name)(**kw)
    D = Descriptor(lower(sys_.to_spec(disc)))
    D.desc.flags = flags
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    return buf.value.decode(), D


def _cell(src):
    return src[src.index("void gen_cell("):src.index("void gen_coef(")]


def test_adr_difference_form():
    src, _ = _source("adr3d", dict(N=6, nz_pts=8))
    cell = _cell(src)
    assert "if (P.cw && " in cell
    assert "kCoefArrays = 6;" in src                    # the six face taps
    assert cell.count(" - u0)") == 6                     # applied to differences
    assert "const T u0 = fb[0];" in cell
    # the centre's constant parts (upwinding) cancel against the differenced taps: no centre tap
    assert "fb[0], acc" not in cell and "* fb[0];" not in cell


def test_adr_expanded_form():
    src, _ = _source("adr3d", dict(N=6, nz_pts=8), L.MOL_FLAG_EXPAND_STENCILS)
    cell = _cell(src)
    assert "kCoefArrays = 7;" in src                    # the face taps and the centre
    assert " - u0)" not in cell
    # -lambda u^2 joins the centre tap: (c_0 - lambda u) u
    assert "fma(fma(-U." in cell and "u0, acc)" in cell
    assert "out[0] = fg0;" in cell


def test_state_dependent_coefficient_is_not_a_coefficient_stencil():
    src, _ = _source("nonlinear_diffusion", dict(n=9, k=1.3, seed=1000))
    assert "kCoefArrays = 0;" in src and "P.cw &&" not in src


def test_constant_coefficients_keep_uniform_weights():
    src, _ = _source("brusselator", dict(N=8))
    assert "kCoefArrays = 0;" in src and "P.cw &&" not in src


def test_expanded_form_compiles_for_sm103a():
    """All four kernel groups of the expanded form (the difference form of the same problem is
    compiled by test_lowering.test_generated_code_compiles_for_sm103a)."""
    _, D = _source("adr3d", dict(N=6, nz_pts=8), L.MOL_FLAG_EXPAND_STENCILS)
    log = C.create_string_buffer(1 << 16)
    assert L.lib().mol_codegen_compile_check(C.byref(D.desc), log, 1 << 16) == 0, log.value.decode()


def _source_of(sys_disc, flags=0):
    sys_, disc, _ = sys_disc
    D = Descriptor(lower(sys_.to_spec(disc)))
    D.desc.flags = flags
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    return buf.value.decode()


def test_two_field_system_groups():
    """One group per output field; the parameter-scaled diffusivity (its face program reads a
    parameter) stays outside its field's group on its own statements."""
    diff = _source_of(problems.coefficient_system(12))
    exp = _source_of(problems.coefficient_system(12), L.MOL_FLAG_EXPAND_STENCILS)
    assert "kCoefArrays = 6;" in diff and "kCoefArrays = 8;" in exp
    for src in (diff, exp):
        cell = _cell(src)
        assert cell.count("if (P.cw && ") == 2
        assert "P.cw + (long long)0 * P.ncell" in cell and "P.cw + (long long)" in cell
        # the parameter-scaled term (term 1) is evaluated in the cell's main flow
        before_group = cell[:cell.index("if (P.cw && ")]
        assert "gt1<T>(" in before_group


def test_reaction_joins_the_centre_only_in_expanded_form():
    diff = _cell(_source("adr3d", dict(N=6, nz_pts=8))[0])
    exp = _cell(_source("adr3d", dict(N=6, nz_pts=8), L.MOL_FLAG_EXPAND_STENCILS)[0])
    assert "fma(fma(-U." not in diff and "v20" in diff.split("if (P.cw")[0]
    assert "fma(fma(-U." in exp


def test_coefficient_stencils_off(monkeypatch):
    """MOL_JIT_CFOLD=0 turns the stencil groups off: the terms' own statements (and the face
    pass) serve every cell."""
    monkeypatch.setenv("MOL_JIT_CFOLD", "0")
    src, _ = _source("adr3d", dict(N=6, nz_pts=8))
    assert "kCoefArrays = 0;" in src and "P.cw &&" not in src
