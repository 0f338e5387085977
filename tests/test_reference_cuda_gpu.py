"""The reference's own CUDA solvers as the GPU comparison arm (oracle/ref_cuda.py).

Their kernels update in place, so their results are not bit-comparable with
Jacobi; these tests check that the harness runs them as the reference's step
does: the uint8 image is the clip of the returned state, the residual falls,
and per sweep it falls at least as fast as Jacobi's (the reference's own
documentation reports a far lower error than numpy Jacobi at equal sweeps).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import cjacobi, ref_cuda

pytestmark = [
    pytest.mark.gpu,
    pytest.mark.skipif(ref_cuda.unavailable_reason() is not None,
                       reason=str(ref_cuda.unavailable_reason())),
]


@pytest.fixture(scope="module")
def circle():
    from fpie_gb300 import prep, workloads

    pb = workloads.circle256()
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    return pb, mc, t, g


def _grid_residual(mc, t, g, x):
    o = cjacobi.CGrid(mc, t, g)
    o.x = np.ascontiguousarray(x, dtype=np.float32)
    return o.err64()


def test_reference_grid_step(circle):
    _, mc, t, g = circle
    r = ref_cuda.RefCudaGrid(8, 8)
    r.reset(mc, t, g)
    img, err = r.step(200)
    x = r.state()
    assert np.isfinite(x).all()
    o = cjacobi.CGrid(mc, t, g)
    o.x = x
    np.testing.assert_array_equal(img, o.image())
    # Unmasked pixels are never written.
    np.testing.assert_array_equal(x[mc == 0], t[mc == 0])
    res = _grid_residual(mc, t, g, x)
    res0 = _grid_residual(mc, t, g, t)
    assert res.sum() < 0.5 * res0.sum()
    jac = cjacobi.CGrid(mc, t, g)
    jac.sweep(200)
    assert res.sum() <= 1.05 * jac.err64().sum(), (res, jac.err64())
    assert err.shape == (3,) and np.isfinite(err).all()


def test_reference_grid_sweeps_continue(circle):
    """step(a) then step(b) continues from the same state (the reference keeps
    its state on the device between steps)."""
    _, mc, t, g = circle
    r = ref_cuda.RefCudaGrid(8, 8)
    r.reset(mc, t, g)
    r.step(100)
    a = _grid_residual(mc, t, g, r.state()).sum()
    r.step(100)
    b = _grid_residual(mc, t, g, r.state()).sum()
    assert b < a


def test_reference_grid_rejects_masked_frame(circle):
    _, mc, t, g = circle
    bad = mc.copy()
    bad[0, 5] = 1
    r = ref_cuda.RefCudaGrid(8, 8)
    with pytest.raises(ValueError):
        r.reset(bad, t, g)


def test_reference_equ_step(circle):
    from fpie_gb300 import backend, prep

    pb, _, _, _ = circle
    sysm = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                           backend.EquSolver(256).partition)
    q = ref_cuda.RefCudaEqu(1024)
    q.reset(sysm.N, sysm.A, sysm.X, sysm.B)
    img, err = q.step(200)
    X = q.state()
    assert np.isfinite(X).all()
    o = cjacobi.CEqu(sysm.A, sysm.X, sysm.B)
    res0 = o.err64().sum()
    o.X = X
    np.testing.assert_array_equal(img[1:], o.image()[1:])
    assert o.err64().sum() < 0.5 * res0
    jac = cjacobi.CEqu(sysm.A, sysm.X, sysm.B)
    jac.sweep(200)
    assert o.err64().sum() <= 1.05 * jac.err64().sum()
