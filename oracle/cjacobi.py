"""ORACLE (test infrastructure only): ctypes binding of oracle/jacobi_ref.c.

``build()`` compiles the C restatement into oracle/_build/ with gcc (done by
``__graft_entry__.build()`` and on first use).  Only tests, the smoke check
and the CPU-baseline legs of bench.py use this module.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
_SRC = _HERE / "jacobi_ref.c"
_LIB = _HERE / "_build" / "liboracle_jacobi.so"
_lib = None

_f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_f64 = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> pathlib.Path:
    if force or not _LIB.exists() or _LIB.stat().st_mtime < _SRC.stat().st_mtime:
        _LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = _LIB.with_suffix(f".{os.getpid()}.tmp")
        subprocess.run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        str(_SRC), "-o", str(tmp), "-lm"], check=True)
        os.replace(tmp, _LIB)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(str(build()))
        c_int, c_i64 = ctypes.c_int, ctypes.c_int64
        _lib.oracle_grid_sweeps.argtypes = [c_int, c_int, _i32, _f32, _f32, _f32, c_int, c_int]
        _lib.oracle_grid_sweeps.restype = c_int
        _lib.oracle_grid_residual.argtypes = [c_int, c_int, _i32, _f32, _f32, _f64, ctypes.c_void_p]
        _lib.oracle_clip_u8.argtypes = [c_i64, _f32, _u8]
        _lib.oracle_equ_sweeps.argtypes = [c_int, _i32, _f32, _f32, _f32, c_int, c_int]
        _lib.oracle_equ_sweeps.restype = c_int
        _lib.oracle_equ_residual.argtypes = [c_int, _i32, _f32, _f32, _f64]
        _lib.oracle_equ_rb_sweeps.argtypes = [c_int, c_int, _i32, _f32, _f32, c_int, c_int]
        _lib.oracle_equ_rb_sweeps.restype = None
    return _lib


def threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


class CGrid:
    """Grid Jacobi state held in numpy arrays, swept by the C restatement."""

    def __init__(self, mask, tgt, grad, nthreads: int | None = None):
        self.mask = np.ascontiguousarray(mask, dtype=np.int32)
        self.n, self.m = self.mask.shape
        self.x = np.array(tgt, dtype=np.float32, order="C", copy=True)
        self.tmp = np.empty_like(self.x)
        self.g = np.ascontiguousarray(grad, dtype=np.float32)
        self.nthreads = nthreads or threads()

    def sweep(self, k: int) -> None:
        if k <= 0:
            return
        if lib().oracle_grid_sweeps(self.n, self.m, self.mask, self.x, self.tmp, self.g, k, self.nthreads):
            self.x, self.tmp = self.tmp, self.x

    def err64(self) -> np.ndarray:
        e = np.zeros(3, np.float64)
        lib().oracle_grid_residual(self.n, self.m, self.mask, self.x, self.g, e, None)
        return e

    def image(self) -> np.ndarray:
        out = np.empty(self.x.shape, np.uint8)
        lib().oracle_clip_u8(self.x.size, self.x, out)
        return out


class CEqu:
    """Equation Jacobi state held in numpy arrays, swept by the C restatement."""

    def __init__(self, A, X, B, nthreads: int | None = None):
        self.A = np.ascontiguousarray(A, dtype=np.int32)
        self.N = self.A.shape[0]
        self.X = np.array(X, dtype=np.float32, order="C", copy=True)
        self.tmp = np.empty_like(self.X)
        self.B = np.ascontiguousarray(B, dtype=np.float32)
        self.nthreads = nthreads or threads()

    def sweep(self, k: int) -> None:
        if k <= 0:
            return
        if lib().oracle_equ_sweeps(self.N, self.A, self.X, self.tmp, self.B, k, self.nthreads):
            self.X, self.tmp = self.tmp, self.X

    def err64(self) -> np.ndarray:
        e = np.zeros(3, np.float64)
        lib().oracle_equ_residual(self.N, self.A, self.X, self.B, e)
        return e

    def image(self) -> np.ndarray:
        out = np.empty(self.X.shape, np.uint8)
        lib().oracle_clip_u8(self.X.size, self.X, out)
        return out


class CEquRedBlack(CEqu):
    """Red-black Gauss-Seidel (the reference's OpenMP EquSolver order) by the
    C restatement: rows 1..n_mid-1 then n_mid..N-1, in place."""

    def __init__(self, A, X, B, n_mid: int, nthreads: int | None = None):
        super().__init__(A, X, B, nthreads)
        self.n_mid = int(n_mid)

    def sweep(self, k: int) -> None:
        if k > 0:
            lib().oracle_equ_rb_sweeps(self.N, self.n_mid, self.A, self.X, self.B, k, self.nthreads)
