"""ORACLE (test infrastructure only): restatement of fpie's host-side set-up.

This module restates, in plain numpy, how the reference processors turn
(source, mask, target, offsets) into solver inputs.  Only tests, the smoke
check and the CPU-baseline leg of the benchmark may import it; the backend
never calls it.

* ``threshold_mask``      -- fpie/process.py:209-217 (also :338-346)
* ``crop_box``            -- fpie/process.py:219-224 / :348-351
* ``mix``                 -- BaseProcessor.mixgrad, fpie/process.py:113-122
* ``grid_inputs``         -- GridProcessor.reset, fpie/process.py:321-386
* ``equ_inputs``          -- EquProcessor.mask2index + reset,
                             fpie/process.py:180-190, 192-271 with
                             np_solver.EquSolver.partition (np_solver.py:14-16)

Pinned against vectors produced by the reference itself
(tests/golden/*.npz, made by tests/golden/make_golden.py).
"""

from __future__ import annotations

import numpy as np


def threshold_mask(mask: np.ndarray) -> np.ndarray:
    """uint8/any mask -> int32 0/1, frame zeroed.

    A 3-channel mask is averaged over channels first (float64 mean), then
    compared with 128.  For integer masks the mean test equals
    ``channel sum >= 384`` exactly, which is how it is computed here.
    """
    if mask.ndim == 3:
        if np.issubdtype(mask.dtype, np.integer):
            on = mask.astype(np.int64).sum(axis=-1) >= 384
        else:
            on = mask.mean(axis=-1) >= 128
    else:
        on = mask >= 128
    out = on.astype(np.int32)
    out[[0, -1], :] = 0
    out[:, [0, -1]] = 0
    return out


def crop_box(mask01: np.ndarray) -> tuple[int, int, int, int]:
    """Bounding box of the set pixels grown by one pixel: (x0, x1, y0, y1)."""
    rows = np.flatnonzero(mask01.any(axis=1))
    cols = np.flatnonzero(mask01.any(axis=0))
    if rows.size == 0:
        raise ValueError("mask selects no pixel")
    return int(rows[0]) - 1, int(rows[-1]) + 2, int(cols[0]) - 1, int(cols[-1]) + 2


def mix(a: np.ndarray, b: np.ndarray, mode: str) -> np.ndarray:
    """Gradient mixing of source difference a and target difference b."""
    if mode == "src":
        return a
    if mode == "avg":
        return (a + b) / 2
    return np.where(np.abs(a) < np.abs(b), b, a)


def grid_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, mode):
    """Return (mask int32[n,m], tgt f32[n,m,3], grad f32[n,m,3], (x0,x1,y0,y1) on tgt)."""
    m01 = threshold_mask(mask)
    x0, x1, y0, y1 = crop_box(m01)
    mc = m01[x0:x1, y0:y1]
    s = src[mask_on_src[0] + x0 : mask_on_src[0] + x1, mask_on_src[1] + y0 : mask_on_src[1] + y1].astype(np.float32)
    t = tgt[mask_on_tgt[0] + x0 : mask_on_tgt[0] + x1, mask_on_tgt[1] + y0 : mask_on_tgt[1] + y1].astype(np.float32)
    n, m = mc.shape
    grad = np.zeros((n, m, 3), np.float32)
    # For every pixel, the four mixed differences "centre minus neighbour"
    # are accumulated in the order up, down, left, right; a neighbour outside
    # the crop contributes nothing.
    for (di, dj) in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        ci = slice(max(0, -di), n - max(0, di))
        cj = slice(max(0, -dj), m - max(0, dj))
        ni = slice(max(0, di), n - max(0, -di))
        nj = slice(max(0, dj), m - max(0, -dj))
        grad[ci, cj] += mix(s[ci, cj] - s[ni, nj], t[ci, cj] - t[ni, nj], mode)
    grad[mc == 0] = 0
    box = (mask_on_tgt[0] + x0, mask_on_tgt[0] + x1, mask_on_tgt[1] + y0, mask_on_tgt[1] + y1)
    return mc, t, grad, box


def equ_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, mode, order: str = "row"):
    """Return dict with ids, A int32[N,4], X f32[N,3], B f32[N,3], N, and target pixel indices.

    order "row": ids row-major (np_solver / core_cuda partition); "red_black":
    the OpenMP EquSolver's odd-then-even ids (fpie/core/openmp/equ.cc:22-56),
    with n_mid = the first even id in the result."""
    m01 = threshold_mask(mask)
    x0, x1, y0, y1 = crop_box(m01)
    mc = m01[x0:x1, y0:y1]
    n, m = mc.shape
    n_mid = None
    if order == "red_black":
        from .np_jacobi import red_black_ids

        ids, n_mid = red_black_ids(mc)
    else:
        assert order == "row", order
        ids = np.zeros((n, m), np.int64)
        flat = mc.reshape(-1) > 0
        ids.reshape(-1)[flat] = np.arange(1, int(flat.sum()) + 1)
    px, py = np.nonzero(mc)
    sel = np.argsort(ids[px, py], kind="stable")  # unknowns in id order
    px, py = px[sel], py[sel]
    N = px.size + 1
    so = (mask_on_src[0] + x0, mask_on_src[1] + y0)
    to = (mask_on_tgt[0] + x0, mask_on_tgt[1] + y0)

    def at(img, off, dx, dy):
        return img[px + off[0] + dx, py + off[1] + dy].astype(np.float32)

    g = np.zeros((N - 1, 3), np.float32)
    for (dx, dy) in ((0, -1), (0, 1), (-1, 0), (1, 0)):  # left, right, up, down
        g = g + mix(at(src, so, 0, 0) - at(src, so, dx, dy), at(tgt, to, 0, 0) - at(tgt, to, dx, dy), mode)
    A = np.zeros((N, 4), np.int32)
    X = np.zeros((N, 3), np.float32)
    B = np.zeros((N, 3), np.float32)
    X[1:] = at(tgt, to, 0, 0)
    for k, (dx, dy) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1))):  # up, down, left, right
        A[1:, k] = ids[px + dx, py + dy]
    B[1:] = g
    for (dx, dy) in ((-1, 0), (0, -1), (0, 1), (1, 0)):  # up, left, right, down
        outside = mc[px + dx, py + dy] == 0
        B[1:][outside] += at(tgt, to, dx, dy)[outside]
    return {
        "ids": ids.astype(np.int32),
        "A": A,
        "X": X,
        "B": B,
        "N": N,
        "tgt_index": (px + to[0], py + to[1]),
        "mask": mc,
        "n_mid": n_mid,
    }
