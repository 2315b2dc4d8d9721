"""ctypes binding of ``oracle/c/bruss_oracle.c``: the C/OpenMP restatement of the
Brusselator semi-discretisation and its fixed-step SSPRK33 solve.

Test infrastructure, like the rest of ``oracle/``: it is the multi-core CPU baseline of the
headline workload in ``bench.py`` and is checked against the numpy oracle in the CPU tests.
The shared library is built with gcc (``-O3 -fopenmp``) into ``oracle/c/_build/``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "c", "bruss_oracle.c")
OUT = os.path.join(HERE, "c", "_build", "libbruss_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the shared library when it is missing or older than its source."""
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        tmp = OUT + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-o", tmp, SRC], check=True)
        os.replace(tmp, OUT)
    return OUT


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        dp, i64 = C.POINTER(C.c_double), C.c_int64
        L.bruss_ssprk33.argtypes = [i64, i64, dp, dp, C.c_double, dp, dp, dp, C.c_double, C.c_double, i64, C.c_int]
        L.bruss_ssprk33.restype = C.c_int
        L.bruss_rhs.argtypes = [i64, i64, dp, dp, C.c_double, dp, dp, dp, dp, C.c_double]
        L.bruss_rhs.restype = None
        L.bruss_max_threads.argtypes = []
        L.bruss_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Brusselator:
    """The grid, weights and parameter of a lowered periodic Brusselator problem."""

    def __init__(self, lw):
        ops = {t["dim"]: t["op"] for t in lw.terms if t["kind"] == 1 and t["field"] == 0}
        self.wx = np.ascontiguousarray(lw.ops[ops[0]].interior, dtype=np.float64)
        self.wy = np.ascontiguousarray(lw.ops[ops[1]].interior, dtype=np.float64)
        assert self.wx.size == 3 and self.wy.size == 3, "three-point second derivatives expected"
        self.x = np.ascontiguousarray(lw.grids[0][lw.lower[0]:], dtype=np.float64)
        self.y = np.ascontiguousarray(lw.grids[1][lw.lower[1]:], dtype=np.float64)
        self.nx, self.ny = self.x.size, self.y.size
        assert 2 * self.nx * self.ny == lw.n_unknowns
        self.alpha = float(lw.param_values[0])

    def rhs(self, u: np.ndarray, t: float) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty_like(u)
        lib().bruss_rhs(self.nx, self.ny, _ptr(self.wx), _ptr(self.wy), self.alpha, _ptr(self.x), _ptr(self.y),
                        _ptr(u), _ptr(out), float(t))
        return out

    def ssprk33(self, u: np.ndarray, t0: float, dt: float, nsteps: int, nthreads: int = 0) -> np.ndarray:
        s = np.array(u, dtype=np.float64, copy=True)
        st = lib().bruss_ssprk33(self.nx, self.ny, _ptr(self.wx), _ptr(self.wy), self.alpha, _ptr(self.x),
                                 _ptr(self.y), _ptr(s), float(t0), float(dt), int(nsteps), int(nthreads))
        if st != 0:
            raise MemoryError("bruss_ssprk33: scratch allocation failed")
        return s


def max_threads() -> int:
    return int(lib().bruss_max_threads())
