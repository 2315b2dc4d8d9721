"""ctypes binding of the oracle's C/OpenMP restatements (``oracle/c``):

- ``bruss_oracle.c``: the 2-D periodic Brusselator semi-discretisation and its fixed-step
  SSPRK33 solve;
- ``adr_oracle.c``: the 3-D advection-diffusion-reaction semi-discretisation (x, y periodic,
  z Dirichlet) and its fixed-step SSPRK33 solve.

Test infrastructure, like the rest of ``oracle/``: these are the multi-core CPU baselines of
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) and are checked against
the numpy oracle in the CPU tests.  Both sources are built with gcc (``-O3 -fopenmp``, no
machine-specific flags, so x86 and Arm hosts compile the same code) into one shared library
under ``oracle/c/_build/``.  The numeric tables (weights, the diffusivity at the faces) are
inputs, taken from the lowered problem, so the arithmetic uses the same doubles as the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "c", "bruss_oracle.c"), os.path.join(HERE, "c", "adr_oracle.c")]
OUT = os.path.join(HERE, "c", "_build", "libmol_oracle_c.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the shared library when it is missing or older than a source."""
    newest = max(os.path.getmtime(s) for s in SRCS)
    if force or not os.path.exists(OUT) or os.path.getmtime(OUT) < newest:
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        tmp = OUT + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c11", "-o", tmp] + SRCS, check=True)
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
        ip = C.POINTER(C.c_int64)
        L.adr_rhs.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.adr_rhs.restype = None
        L.adr_ssprk33.argtypes = [ip, dp, dp, dp, dp, dp, dp, dp, dp, dp, C.c_double, i64, C.c_int]
        L.adr_ssprk33.restype = C.c_int
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


class ADR3D:
    """The tables of a lowered 3-D advection-diffusion-reaction problem (problems.adr3d):
    the half-offset weights and the face diffusivities of the three nonlinear-Laplacian
    terms, the centered weights of the mixed term, the backward upwind weights, and the
    equation's constants (0.3, 1.0, 0.5) and parameter lambda."""

    def __init__(self, lw, cmix: float = 0.3, cx: float = 1.0, cy: float = 0.5):
        assert len(lw.ivs) == 3 and len(lw.fields) == 1
        assert list(lw.consts) == [cmix, cx, cy], "not the adr3d equation"
        n = [lw.npts[j] - lw.lower[j] - lw.upper[j] for j in range(3)]
        self.n = np.array(n, dtype=np.int64)
        wi, wo, K = np.zeros(6), np.zeros(6), [None] * 3
        for t in lw.terms:
            if t["kind"] != 4:
                continue
            j = t["dim"]
            wo[2 * j:2 * j + 2] = lw.ops[t["op"]].interior
            wi[2 * j:2 * j + 2] = lw.ops[t["op2"]].interior
            ext = [lw.npts[k] + (1 if k == j else 0) for k in range(3)]
            full = lw.aux[t["aux0"]].reshape(ext, order="F")
            sl = [slice(lw.lower[k], lw.npts[k] - lw.upper[k]) for k in range(3)]
            sl[j] = slice(lw.lower[j], lw.lower[j] + n[j] + 1)      # left face of every cell + the last right face
            K[j] = np.ascontiguousarray(full[tuple(sl)].reshape(-1, order="F"))
        mixed = [t for t in lw.terms if t["kind"] == 2][0]
        wm = np.concatenate([lw.ops[mixed["op"]].interior, lw.ops[mixed["op2"]].interior])
        wb = np.zeros(4)
        for t in lw.terms:
            if t["kind"] == 1 and lw.ops[t["op"]].omin == -1:      # the backward (positive-wind) stencil
                wb[2 * t["dim"]:2 * t["dim"] + 2] = lw.ops[t["op"]].interior
        self.wi, self.wo, self.wm, self.wb = wi, wo, np.ascontiguousarray(wm, dtype=np.float64), wb
        self.coef = np.array([cmix, cx, cy, float(lw.param_values[0])])
        self.K = K

    def _args(self):
        return (self.n.ctypes.data_as(C.POINTER(C.c_int64)), _ptr(self.wi), _ptr(self.wo), _ptr(self.wm),
                _ptr(self.wb), _ptr(self.coef), _ptr(self.K[0]), _ptr(self.K[1]), _ptr(self.K[2]))

    def rhs(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty_like(u)
        lib().adr_rhs(*self._args(), _ptr(u), _ptr(out))
        return out

    def ssprk33(self, u: np.ndarray, dt: float, nsteps: int, nthreads: int = 0, out: np.ndarray = None):
        s = np.array(u, dtype=np.float64, copy=True) if out is None else out
        if out is not None:
            s[...] = u
        st = lib().adr_ssprk33(*self._args(), _ptr(s), float(dt), int(nsteps), int(nthreads))
        if st != 0:
            raise MemoryError("adr_ssprk33: scratch allocation failed")
        return s


def max_threads() -> int:
    return int(lib().bruss_max_threads())
