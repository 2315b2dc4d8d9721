"""ctypes binding of the molgpu C ABI (``include/molgpu.h``).

The shared library is the product: every compute call goes through it.  If it is
missing the import fails loudly; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmolgpu.so")

MOL_MAX_DIMS = 3
MOL_MAX_FIELDS = 8
MOL_MAX_REGS = 64
MOL_ABI_VERSION = 2
MOL_FLAG_EXPAND_STENCILS = 1   # mol_problem_desc.flags: coefficient stencils as one expanded sum

STATUS = {
    0: "MOL_OK", -1: "MOL_ERR_INVALID", -2: "MOL_ERR_OOM", -3: "MOL_ERR_NONFINITE",
    -4: "MOL_ERR_TIMEOUT", -5: "MOL_ERR_CUDA", -6: "MOL_ERR_UNSUPPORTED", -7: "MOL_ERR_MAXITERS",
    -8: "MOL_ERR_DTMIN",
}

# term kinds, bc kinds, opcodes (mirror of the header enums)
TERM_LINEAR, TERM_MIXED, TERM_WENO, TERM_NONLINLAP = 1, 2, 3, 4
BC_NONE, BC_PERIODIC, BC_ROBIN, BC_EDGE = 0, 1, 2, 3
(OP_CONST, OP_PARAM, OP_FIELD, OP_AUX, OP_COORD, OP_TIME, OP_TERM, OP_UPWIND, OP_ADD, OP_SUB, OP_MUL,
 OP_DIV, OP_NEG, OP_POWI, OP_POW, OP_FN, OP_CMP, OP_IFELSE, OP_OUT) = range(1, 20)
FN_IDS = {"sin": 0, "cos": 1, "tan": 2, "exp": 3, "log": 4, "sqrt": 5, "abs": 6, "tanh": 7, "sinh": 8,
          "cosh": 9, "atan": 10}
CMP_IDS = {"<=": 0, "<": 1, ">=": 2, ">": 3, "==": 4}
LOSS_MISFIT, LOSS_LAMBDA = 0, 1


class mol_op1d(C.Structure):
    _fields_ = [("L", C.c_int32), ("omin", C.c_int32), ("nlo", C.c_int32), ("bLlo", C.c_int32),
                ("nhi", C.c_int32), ("bLhi", C.c_int32), ("hi_base", C.c_int32), ("nrows", C.c_int32),
                ("w_int", C.c_int64), ("w_lo", C.c_int64), ("w_hi", C.c_int64)]


class mol_term(C.Structure):
    _fields_ = [("kind", C.c_int32), ("field", C.c_int32), ("dim", C.c_int32), ("dim2", C.c_int32),
                ("op", C.c_int32), ("op2", C.c_int32), ("op3", C.c_int32), ("prog", C.c_int32),
                ("aux0", C.c_int32), ("reserved0", C.c_int32), ("variant", C.c_int32),
                ("reserved2", C.c_int32), ("eps", C.c_double), ("dx", C.c_double)]


class mol_bc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("prog", C.c_int32), ("op", C.c_int32), ("extrap", C.c_int32),
                ("a", C.c_double), ("b", C.c_double), ("g", C.c_double), ("iop", C.c_int32), ("pad", C.c_int32)]


class mol_instr(C.Structure):
    _fields_ = [("op", C.c_uint16), ("dst", C.c_uint16), ("a", C.c_uint16), ("b", C.c_uint16),
                ("c", C.c_uint16), ("reserved", C.c_uint16), ("imm", C.c_int32)]


class mol_problem_desc(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("ndim", C.c_int32), ("nfields", C.c_int32), ("nparams", C.c_int32),
        ("npts", C.c_int64 * MOL_MAX_DIMS), ("lower", C.c_int32 * MOL_MAX_DIMS),
        ("upper", C.c_int32 * MOL_MAX_DIMS), ("dx", C.c_double * MOL_MAX_DIMS),
        ("coords", C.POINTER(C.c_double) * MOL_MAX_DIMS),
        ("bc", ((mol_bc * 2) * MOL_MAX_DIMS) * MOL_MAX_FIELDS),
        ("nops", C.c_int32), ("ops", C.POINTER(mol_op1d)),
        ("nweights", C.c_int64), ("weights", C.POINTER(C.c_double)),
        ("nterms", C.c_int32), ("terms", C.POINTER(mol_term)),
        ("ninstr", C.c_int32), ("code", C.POINTER(mol_instr)),
        ("nprogs", C.c_int32), ("prog_ranges", C.POINTER(C.c_int32)),
        ("cell_prog", C.c_int32),
        ("nconsts", C.c_int32), ("consts", C.POINTER(C.c_double)),
        ("naux", C.c_int32), ("aux", C.POINTER(C.POINTER(C.c_double))), ("aux_len", C.POINTER(C.c_int64)),
        ("params", C.POINTER(C.c_double)),
        ("flags", C.c_int32), ("reserved", C.c_int32),
    ]


class mol_stats(C.Structure):
    _fields_ = [("naccept", C.c_int64), ("nreject", C.c_int64), ("nf", C.c_int64), ("t", C.c_double),
                ("dt", C.c_double)]


_lib = None

# name -> (restype, argtypes)
_PROTOS = {
    "mol_version": (C.c_int, []),
    "mol_status_string": (C.c_char_p, [C.c_int]),
    "mol_plan_create": (C.c_int, [C.POINTER(mol_problem_desc), C.POINTER(C.c_void_p)]),
    "mol_plan_destroy": (C.c_int, [C.c_void_p]),
    "mol_generate_code": (C.c_int, [C.POINTER(mol_problem_desc), C.c_char_p, C.c_int64, C.POINTER(C.c_int64)]),
    "mol_codegen_compile_check": (C.c_int, [C.POINTER(mol_problem_desc), C.c_char_p, C.c_int64]),
    "mol_last_error": (C.c_char_p, [C.c_void_p]),
    "mol_plan_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mol_plan_n_unknowns": (C.c_int64, [C.c_void_p]),
    "mol_launch_count": (C.c_int64, []),
    "mol_plan_uses_codegen": (C.c_int, [C.c_void_p]),
    "mol_plan_coef_arrays": (C.c_int, [C.c_void_p]),
    "mol_plan_codegen_source": (C.c_char_p, [C.c_void_p]),
    "mol_plan_launch_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32)]),
    "mol_rhs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "mol_fill_grid": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p]),
    "mol_rhs_f32state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "mol_step_ssprk33": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]),
    "mol_step_ssprk33_f32state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                                            C.c_int64]),
    "mol_step_ssprk33_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64]),
    "mol_plan_check": (C.c_int, [C.c_void_p]),
    "mol_solve_tsit5": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_int64, C.POINTER(mol_stats)]),
    "mol_adjoint_ssprk33": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_int64,
                                      C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "mol_rhs_vjp": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_void_p,
                              C.c_void_p, C.c_void_p]),
    "mol_batch_create": (C.c_int, [C.POINTER(C.POINTER(mol_problem_desc)), C.c_int32, C.POINTER(C.c_void_p)]),
    "mol_batch_destroy": (C.c_int, [C.c_void_p]),
    "mol_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "mol_batch_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mol_batch_offsets": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "mol_batch_step_ssprk33": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int64]),
    "mol_batch_step_ssprk33_f32state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int64]),
    "mol_batch_tune": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int64]),
    "mol_batch_check": (C.c_int, [C.c_void_p]),
    "mol_batch_config": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
    "mol_diag_fp64_rate": (C.c_int, [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}

EXPORTED = sorted(_PROTOS)


def lib():
    """The loaded libmolgpu (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libmolgpu.so not found at {LIB_PATH}; build it with "
                "`python methodoflines.jl_gb300/build.py` (there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class MolError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


def check(status, plan=None, batch=None):
    if status != 0:
        msg = ""
        if plan is not None:
            msg = (lib().mol_last_error(plan) or b"").decode()
        elif batch is not None:
            msg = (lib().mol_batch_last_error(batch) or b"").decode()
        raise MolError(status, msg)
    return status
