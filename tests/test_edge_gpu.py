"""Edge cases of the grid and equation solvers against the numpy oracle.

Degenerate and thin grids, no set pixel, every pixel set (borders included,
so neighbours outside the grid read 0 as in the numpy backend), and sweep
counts that are not multiples of any kernel's depth -- for every sweep
kernel.  States bit for bit, images exactly, err rtol 1e-5.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import np_jacobi

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (1, 7), (7, 1), (2, 2), (3, 3), (2, 300), (300, 3), (5, 129), (131, 130)]
KERNELS = ["sweep1", "p16w8k8", "p16w8k16", "p8w16k16", "p8w8k8", "p16w8k16t", "p16w8k16d",
           "p16w8k12d", "p16w8k16dp", "p16w8k12dp"]


def _case(shape, kind, seed):
    rng = np.random.default_rng(seed)
    n, m = shape
    if kind == "none":
        mask = np.zeros(shape, np.int32)
    elif kind == "all":
        mask = np.ones(shape, np.int32)
    else:
        mask = (rng.random(shape) > 0.4).astype(np.int32)
    tgt = rng.uniform(-20, 275, (n, m, 3)).astype(np.float32)  # values outside [0,255] clip
    grad = rng.uniform(-50, 50, (n, m, 3)).astype(np.float32)
    return mask, tgt, grad


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", ["none", "all", "random"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_grid_edge_cases(shape, kind, kernel):
    from fpie_gb300 import backend

    mask, tgt, grad = _case(shape, kind, hash((shape, kind)) % 1000)
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.reset(mask.size, mask, tgt, grad)
    o = np_jacobi.GridJacobi(mask, tgt, grad)
    for k in (1, 17, 70):
        img, err = s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.x)
        np.testing.assert_array_equal(img, o.image())
        np.testing.assert_allclose(err, o.err64(), rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("n_unknowns", [1, 2, 33, 1000])
def test_equ_edge_cases(n_unknowns):
    """Random neighbour tables, including self-references and row 0 links."""
    from fpie_gb300 import backend

    rng = np.random.default_rng(n_unknowns)
    N = n_unknowns
    A = rng.integers(0, N, (N, 4)).astype(np.int32)
    X = rng.uniform(-10, 270, (N, 3)).astype(np.float32)
    B = rng.uniform(-30, 30, (N, 3)).astype(np.float32)
    s = backend.EquSolver(64)
    s.reset(N, A, X, B)
    o = np_jacobi.EquJacobi(A, X, B)
    for k in (1, 5, 64, 3):
        x, err = s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.X)
        np.testing.assert_array_equal(x, o.image())
        np.testing.assert_allclose(err, o.err64(), rtol=1e-5, atol=1e-4)


def test_fp32_probe_rate_is_plausible():
    """The roofline's denominator: the packed-add rate lies between 25% and
    200% of SMs x 128 lanes x 2.5 GHz (one operation per value)."""
    torch = pytest.importorskip("torch")
    from fpie_gb300 import _abi

    sms = torch.cuda.get_device_properties(0).multi_processor_count
    nominal = sms * 128 * 2.5e9
    for kind in ("fadd2", "ffma2", "fadd"):
        rate = _abi.fp32_rate(kind, iters=2000)
        assert 0.25 * nominal < rate < 2.0 * nominal, (kind, rate, nominal)
