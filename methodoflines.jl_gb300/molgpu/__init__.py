"""molgpu: GB300-native method-of-lines hot path (f! and explicit steppers) behind a C ABI.

The symbolic layer (``symbolic``) and the lowering (``lowering``) play the role
of MethodOfLines.jl's discretisation front end; every numerical evaluation runs
in ``libmolgpu.so`` on the GPU.
"""
from . import _lib
from .api import (Batch, MOLFiniteDifference, ODEFunction, ODEProblem, Plan, Solution, SSPRK33, Tsit5, UpwindScheme,
                  WENOScheme, center_align, chebyspace, discretize, edge_align, solve)
from .lowering import Descriptor, Lowered, lower
from .symbolic import (Differential, Eq, Equation, Field, Interval, IV, Param, PDESystem, abs_, atan, cos, cosh,
                       exp, ifelse, log, register, sin, sinh, sqrt, tan, tanh)

__all__ = [
    "Batch", "MOLFiniteDifference", "ODEFunction", "ODEProblem", "Plan", "Solution", "SSPRK33", "Tsit5", "UpwindScheme",
    "WENOScheme", "center_align", "chebyspace", "discretize", "edge_align", "solve", "Descriptor", "Lowered", "lower", "Differential", "Eq", "Equation",
    "Field", "Interval", "IV", "Param", "PDESystem", "abs_", "atan", "cos", "cosh", "exp", "ifelse", "log",
    "register", "sin", "sinh", "sqrt", "tan", "tanh",
]
