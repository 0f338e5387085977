"""The batched persistent form against GridSolver runs of each job alone.

Every job's FP32 state must equal, bit for bit, a GridSolver run of the same
sweeps (the kernels share the tile arithmetic); images exactly; err within
rtol 1e-5.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(seed=5):
    from fpie_gb300 import prep, workloads

    rng = np.random.default_rng(seed)
    out = []
    for pb in workloads.job_mix(n_jobs=10, seed=seed, min_box=8, max_box=300, it_lo=1, it_hi=700):
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        out.append((mc, t, g, pb.iterations))
    # plus a job with border pixels set and a single-pixel job
    n, m = 37, 45
    mask = (rng.random((n, m)) > 0.5).astype(np.int32)
    t = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    g = rng.uniform(-20, 20, (n, m, 3)).astype(np.float32)
    out.append((mask, t, g, 333))
    one = np.zeros((3, 3), np.int32)
    one[1, 1] = 1
    out.append((one, np.full((3, 3, 3), 7, np.float32), np.ones((3, 3, 3), np.float32), 17))
    return out


def _alone(mc, t, g, iters):
    from fpie_gb300 import backend

    s = backend.GridSolver(8, 8)
    s.reset(mc.size, mc, t, g)
    img, err = s.step(iters)
    return s.state(), img, err


@pytest.mark.parametrize("kernel", ["auto", "p16w8k16", "p8w16k16", "p16w8k8"])
def test_batch_equals_jobs_alone(kernel):
    from fpie_gb300.batch import BatchSolver

    jobs = _jobs()
    b = BatchSolver(4e9)
    if kernel != "auto":
        b.set_kernel(kernel)
    ids = [b.add(mc, t, g, it) for mc, t, g, it in jobs]
    b.run()
    for jid, (mc, t, g, it) in zip(ids, jobs):
        assert b.progress(jid) == (it, it)
        state, img, err = _alone(mc, t, g, it)
        np.testing.assert_array_equal(b.state(jid), state)
        bimg, berr = b.result(jid)
        np.testing.assert_array_equal(bimg, img)
        np.testing.assert_allclose(berr, err, rtol=1e-5, atol=1e-4)


def test_batch_in_steps_and_slot_reuse():
    from fpie_gb300.batch import BatchSolver

    jobs = _jobs(seed=9)
    b = BatchSolver(4e9)
    ids = [b.add(mc, t, g, it) for mc, t, g, it in jobs]
    b.run(100)
    b.run(250)
    b.run()
    for jid, (mc, t, g, it) in zip(ids, jobs):
        np.testing.assert_array_equal(b.state(jid), _alone(mc, t, g, it)[0])
    b.remove(ids[0])
    mc, t, g, _ = jobs[3]
    new = b.add(mc, t, g, 90)
    assert new == ids[0]  # the freed slot is reused
    b.run()
    np.testing.assert_array_equal(b.state(new), _alone(mc, t, g, 90)[0])


def test_budget_refuses_a_job_that_does_not_fit():
    from fpie_gb300 import _abi
    from fpie_gb300.batch import BatchSolver

    mc, t, g, it = _jobs()[0]
    need = BatchSolver.job_bytes(*mc.shape)
    b = BatchSolver(need * 1.5)
    b.add(mc, t, g, it)
    with pytest.raises(_abi.FpieError):
        b.add(mc, t, g, it)
    used, budget = b.memory()
    assert used == need and budget == pytest.approx(need * 1.5)


def test_dependency_wait_times_out_without_hanging():
    """A spin limit of 1 makes the level-1 waits run out: the call returns a
    timeout error and the GPU stays usable."""
    from fpie_gb300 import _abi
    from fpie_gb300.batch import BatchSolver

    rng = np.random.default_rng(1)
    n, m = 600, 600
    mask = np.ones((n, m), np.int32)
    mask[[0, -1]] = 0
    mask[:, [0, -1]] = 0
    t = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    g = np.zeros((n, m, 3), np.float32)
    b = BatchSolver(4e9)
    b.set_kernel("p16w8k8")
    b.set_spin_limit(1)
    b.add(mask, t, g, 400)
    with pytest.raises(_abi.FpieTimeoutError):
        b.run()
    b.close()
    state, img, err = _alone(mask, t, g, 20)  # the context still works
    assert np.isfinite(state).all()


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
@pytest.mark.parametrize("kernel", ["p16w8k16", "p16w8k8"])
def test_mixed_batch_equals_mixed_solver(precision, kernel):
    """Same correction kernel, same cycle boundaries: the batched mixed form
    reproduces a mixed-precision GridSolver bit for bit."""
    from fpie_gb300 import backend
    from fpie_gb300.batch import BatchSolver

    jobs = _jobs(seed=13)
    b = BatchSolver(4e9, precision=precision)
    b.set_kernel(kernel)
    ids = [b.add(mc, t, g, it) for mc, t, g, it in jobs]
    b.run(200)
    b.run()
    for jid, (mc, t, g, it) in zip(ids, jobs):
        s = backend.GridSolver(8, 8)
        s.set_precision(precision)
        s.set_kernel(kernel)
        s.reset(mc.size, mc, t, g)
        s.step(min(it, 200))
        if it > 200:
            s.step(it - 200)
        np.testing.assert_array_equal(b.state(jid), s.state())


def test_mixed_batch_needs_precision_before_jobs():
    from fpie_gb300 import _abi
    from fpie_gb300.batch import BatchSolver

    mc, t, g, it = _jobs()[0]
    b = BatchSolver(4e9)
    b.add(mc, t, g, it)
    with pytest.raises(_abi.FpieError):
        _abi.call("fpie_batch_set_precision", b._h, 1)


@pytest.mark.parametrize("gradient", ["src", "avg", "max"])
def test_add_images_equals_host_built_inputs(gradient):
    """A job added from uint8 images (3-channel mask, offsets on both images)
    holds the inputs the host construction of GridProcessor.reset gives, and
    its result equals a GridSolver reset from those inputs."""
    from fpie_gb300 import prep, workloads
    from fpie_gb300.batch import BatchSolver

    rng = np.random.default_rng(3)
    src = workloads.smooth_image(21, 140, 150, 12)
    tgt = workloads.smooth_image(22, 160, 170, 12)
    mask = np.zeros((90, 100, 3), np.uint8)
    mask[10:80, 15:90] = rng.integers(100, 256, (70, 75, 3), dtype=np.uint8)
    mos, mot = (20, 30), (40, 35)
    mc, t, g, box = prep.grid_inputs(src, mask, tgt, mos, mot, gradient)
    b = BatchSolver(4e9)
    jid, jbox = b.add_images(src, mask, tgt, mos, mot, gradient, 333)
    assert jbox == (box.x0, box.x1, box.y0, box.y1)
    b.run()
    state, img, err = _alone(mc, t, g, 333)
    np.testing.assert_array_equal(b.state(jid), state)
    bimg, berr = b.result(jid)
    np.testing.assert_array_equal(bimg, img)
    np.testing.assert_allclose(berr, err, rtol=1e-5)


def test_add_images_rejects_bad_input():
    from fpie_gb300 import _abi, workloads
    from fpie_gb300.batch import BatchSolver

    src = workloads.smooth_image(1, 64, 64, 8)
    b = BatchSolver(4e9)
    empty = np.zeros((32, 32), np.uint8)
    with pytest.raises(_abi.FpieArgumentError, match="no pixel"):
        b.add_images(src, empty, src, (0, 0), (0, 0), "max", 10)
    full = np.full((32, 32), 255, np.uint8)
    with pytest.raises(_abi.FpieArgumentError, match="leaves"):
        b.add_images(src, full, src, (50, 0), (0, 0), "max", 10)
    assert b.memory()[0] == 0
