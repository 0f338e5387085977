"""ORACLE (test infrastructure only): numpy restatement of fpie's Jacobi solvers.

Restates the reference's strict-Jacobi numpy backend, the one every backend
here is checked against at equal sweep counts:

* ``GridJacobi`` -- np_solver.GridSolver, fpie/np_solver.py:57-101
* ``EquJacobi``  -- np_solver.EquSolver,  fpie/np_solver.py:6-54

and the red-black Gauss-Seidel order of the reference's OpenMP EquSolver:

* ``red_black_ids`` -- OpenMPEquSolver::partition, fpie/core/openmp/equ.cc:22-56
* ``EquRedBlack``   -- OpenMPEquSolver::step, fpie/core/openmp/equ.cc:67-80, 107-118

Arithmetic order is kept exactly, so float32 states are bit-identical to the
reference's: grid update ``(grad + up + down + left + right) / 4``, grid
residual ``4x - grad - up - down - left - right``, equation update
``(B + X[A0] + X[A1] + X[A2] + X[A3]) / 4`` and residual
``B + sum X[A] - 4X``.  The per-channel error is the sum of |residual| over
the unknowns; ``err64`` accumulates it in float64 (order-free to ~1e-16),
``err32`` in float32 the way numpy does.  Only tests, the smoke check and the
CPU-baseline leg of the benchmark may use this module.
"""

from __future__ import annotations

import numpy as np


def _neighbour_sum(x: np.ndarray, first: np.ndarray) -> np.ndarray:
    """first + up + down + left + right, neighbours outside the array read 0."""
    p = np.pad(x, ((1, 1), (1, 1), (0, 0)))
    acc = first + p[:-2, 1:-1]
    acc = acc + p[2:, 1:-1]
    acc = acc + p[1:-1, :-2]
    acc = acc + p[1:-1, 2:]
    return acc


class GridJacobi:
    """Strict Jacobi on the cropped grid (float32 state)."""

    def __init__(self, mask: np.ndarray, tgt: np.ndarray, grad: np.ndarray):
        self.on = np.asarray(mask) != 0
        self.x = np.array(tgt, dtype=np.float32, copy=True)
        self.g = np.array(grad, dtype=np.float32, copy=True)

    def sweep(self, n: int) -> None:
        for _ in range(n):
            new = _neighbour_sum(self.x, self.g) / np.float32(4.0)
            self.x = np.where(self.on[..., None], new, self.x).astype(np.float32)

    def residual(self) -> np.ndarray:
        """Per-pixel residual 4x - grad - up - down - left - right (float32)."""
        p = np.pad(self.x, ((1, 1), (1, 1), (0, 0)))
        r = np.float32(4.0) * self.x - self.g
        r = r - p[:-2, 1:-1]
        r = r - p[2:, 1:-1]
        r = r - p[1:-1, :-2]
        r = r - p[1:-1, 2:]
        return r

    def err64(self) -> np.ndarray:
        return np.abs(self.residual()[self.on]).astype(np.float64).sum(axis=0)

    def err32(self) -> np.ndarray:
        return np.abs(self.residual()[self.on]).sum(axis=0)

    def image(self) -> np.ndarray:
        """Clip to [0,255] and truncate to uint8 (the processor's store)."""
        return np.clip(self.x, 0, 255).astype(np.uint8)


class EquJacobi:
    """Strict Jacobi on the relabelled unknowns; row 0 is the constant 0."""

    def __init__(self, A: np.ndarray, X: np.ndarray, B: np.ndarray):
        self.A = np.asarray(A, dtype=np.int64)
        self.X = np.array(X, dtype=np.float32, copy=True)
        self.B = np.array(B, dtype=np.float32, copy=True)

    def _gsum(self) -> np.ndarray:
        s = self.B + self.X[self.A[:, 0]]
        s = s + self.X[self.A[:, 1]]
        s = s + self.X[self.A[:, 2]]
        s = s + self.X[self.A[:, 3]]
        return s

    def sweep(self, n: int) -> None:
        for _ in range(n):
            self.X = (self._gsum() / np.float32(4.0)).astype(np.float32)

    def residual(self) -> np.ndarray:
        return self._gsum() - np.float32(4.0) * self.X

    def err64(self) -> np.ndarray:
        return np.abs(self.residual()).astype(np.float64).sum(axis=0)

    def err32(self) -> np.ndarray:
        return np.abs(self.residual()).sum(axis=0)

    def image(self) -> np.ndarray:
        return np.clip(self.X, 0, 255).astype(np.uint8)


def red_black_ids(mask: np.ndarray) -> tuple[np.ndarray, int]:
    """ids of the reference's OpenMP EquSolver.partition: cells with odd
    row + col get 1, 2, ... in row-major order, then cells with even row + col
    continue the count; 0 where mask <= 0.  Returns (ids, n_mid), n_mid = the
    first even id (odd count + 1)."""
    mask = np.asarray(mask)
    n, m = mask.shape
    ii, jj = np.indices((n, m))
    on = mask > 0
    odd = on & ((ii + jj) % 2 == 1)
    even = on & ((ii + jj) % 2 == 0)
    ids = np.zeros((n, m), np.int64)
    n_odd, n_even = int(odd.sum()), int(even.sum())
    ids[odd] = np.arange(1, n_odd + 1)  # boolean indexing visits row-major
    ids[even] = np.arange(n_odd + 1, n_odd + n_even + 1)
    return ids, n_odd + 1


class EquRedBlack(EquJacobi):
    """Red-black Gauss-Seidel of the reference's OpenMP EquSolver: a sweep
    updates rows 1..n_mid-1 in place, then rows n_mid..N-1 reading the new
    values, each as (B + X[A0] + X[A1] + X[A2] + X[A3]) / 4 in that order.
    Rows of one colour only read rows of the other colour (or row 0), so each
    half is computed at once here as in the reference's parallel loops."""

    def __init__(self, A: np.ndarray, X: np.ndarray, B: np.ndarray, n_mid: int):
        super().__init__(A, X, B)
        self.n_mid = int(n_mid)
        N = self.A.shape[0]
        assert 1 <= self.n_mid <= N
        red = np.arange(N) < self.n_mid
        nb = self.A[1:]
        same = (nb != 0) & (red[nb] == red[1:, None])
        assert not same.any(), "a row reads a row of its own colour"

    def _half(self, lo: int, hi: int) -> None:
        if hi <= lo:
            return
        a = self.A[lo:hi]
        s = self.B[lo:hi] + self.X[a[:, 0]]
        s = s + self.X[a[:, 1]]
        s = s + self.X[a[:, 2]]
        s = s + self.X[a[:, 3]]
        self.X[lo:hi] = s / np.float32(4.0)

    def sweep(self, n: int) -> None:
        for _ in range(n):
            self._half(1, self.n_mid)
            self._half(self.n_mid, self.A.shape[0])
