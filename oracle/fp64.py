"""ORACLE (test infrastructure only): the converged FP64 solution of a grid problem.

The grid form's fixed point (the limit of the Jacobi sweeps of
fpie/np_solver.py:79-101) solves, for every masked pixel p and channel,

    4 x_p - sum_{masked q ~ p} x_q = grad_p + sum_{unmasked q ~ p} x_q,

where unmasked neighbours hold their fixed target values and neighbours
outside the crop contribute nothing.  ``direct`` solves it with scipy's
sparse LU in float64 (small and medium grids); ``cg_torch`` runs a
matrix-free float64 conjugate-gradient on a torch device (CUDA for the
10M-unknown workload), and is checked against ``direct`` in the tests.
Only tests and the benchmark scripts use this module.
"""

from __future__ import annotations

import numpy as np


def _system(mask: np.ndarray, tgt: np.ndarray, grad: np.ndarray):
    on = np.asarray(mask) != 0
    n, m = on.shape
    idx = -np.ones((n, m), np.int64)
    px, py = np.nonzero(on)
    idx[px, py] = np.arange(px.size)
    rhs = grad[px, py].astype(np.float64)
    rows, cols = [np.arange(px.size)], [np.arange(px.size)]
    vals = [np.full(px.size, 4.0)]
    for dx, dy in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        qx, qy = px + dx, py + dy
        inside = (qx >= 0) & (qx < n) & (qy >= 0) & (qy < m)
        qxi, qyi = np.where(inside, qx, 0), np.where(inside, qy, 0)
        nb_on = inside & on[qxi, qyi]
        rows.append(np.nonzero(nb_on)[0])
        cols.append(idx[qxi[nb_on], qyi[nb_on]])
        vals.append(np.full(int(nb_on.sum()), -1.0))
        fixed = inside & ~on[qxi, qyi]
        rhs[fixed] += tgt[qxi[fixed], qyi[fixed]].astype(np.float64)
    return (np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)), rhs, (px, py)


def direct(mask, tgt, grad) -> np.ndarray:
    """FP64 solution as an [n, m, 3] array (unmasked pixels = tgt)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    (r, c, v), rhs, (px, py) = _system(mask, tgt, grad)
    A = sp.csc_matrix((v, (r, c)), shape=(px.size, px.size))
    lu = spl.splu(A)
    out = np.array(tgt, dtype=np.float64, copy=True)
    out[px, py] = lu.solve(rhs)
    return out


def cg_torch(mask, tgt, grad, device="cuda", rtol=1e-12, max_iter=200000, check=200):
    """Matrix-free FP64 CG on the masked 5-point operator; returns [n, m, 3] float64."""
    import torch

    on = torch.from_numpy(np.asarray(mask) != 0).to(device)
    t = torch.from_numpy(np.asarray(tgt, np.float64)).to(device).permute(2, 0, 1)
    g = torch.from_numpy(np.asarray(grad, np.float64)).to(device).permute(2, 0, 1)
    onf = on.to(torch.float64)[None]

    def nbsum(z):
        p = torch.nn.functional.pad(z, (1, 1, 1, 1))
        return p[:, :-2, 1:-1] + p[:, 2:, 1:-1] + p[:, 1:-1, :-2] + p[:, 1:-1, 2:]

    fixed = t * (1 - onf)
    b = (g + nbsum(fixed)) * onf

    def A(z):
        return (4 * z - nbsum(z * onf)) * onf

    x = t * onf
    r = b - A(x)
    p = r.clone()
    rs = (r * r).sum(dim=(1, 2))
    b2 = (b * b).sum(dim=(1, 2)).clamp_min(1e-300)
    for it in range(max_iter):
        Ap = A(p)
        alpha = rs / (p * Ap).sum(dim=(1, 2)).clamp_min(1e-300)
        x += alpha[:, None, None] * p
        r -= alpha[:, None, None] * Ap
        rs_new = (r * r).sum(dim=(1, 2))
        if it % check == 0 and bool((rs_new <= (rtol ** 2) * b2).all()):
            break
        p = r + (rs_new / rs.clamp_min(1e-300))[:, None, None] * p
        rs = rs_new
    out = (x * onf + fixed).permute(1, 2, 0).contiguous()
    return out.cpu().numpy()
