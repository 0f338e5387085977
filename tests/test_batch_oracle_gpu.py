"""The batched and served forms against the oracle at the batched workload's
real sizes.

Sixteen jobs of the 256-job mix (boxes log-uniform 32..1024: the largest,
1024x1024, and fifteen others spread over the sizes, circles / squares /
blobs, 'src' and 'max' gradients, 2000-10000 sweeps each) run in one
BatchSolver.  Every job is compared with the oracle's C restatement of the
reference's Jacobi grid solver (fpie/np_solver.py:79-101) after the job's own
sweep count: FP32 state and uint8 image bit for bit, err within rtol 1e-5
(the oracle sums in double in another order).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import cjacobi

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(600)]


def pick_jobs(n_pick: int = 16, seed: int = 7):
    """The largest job of the 256-job mix and n_pick - 1 others evenly spaced
    in box size; both gradients are present."""
    from fpie_gb300 import prep, workloads

    mix = workloads.job_mix(n_jobs=256, seed=seed)
    order = sorted(range(len(mix)), key=lambda k: mix[k].mask.shape[0] * mix[k].mask.shape[1])
    idx = sorted({order[-1], *(order[int(round(q))] for q in np.linspace(0, len(order) - 2, n_pick - 1))})
    jobs = []
    for k in idx:
        pb = mix[k]
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        jobs.append((pb, mc, t, g))
    return jobs


@pytest.fixture(scope="module")
def jobs():
    js = pick_jobs()
    assert {pb.gradient for pb, *_ in js} == {"src", "max"}
    assert max(pb.mask.shape[0] for pb, *_ in js) == 1024
    return js


@pytest.fixture(scope="module")
def oracle_results(jobs):
    out = []
    for pb, mc, t, g in jobs:
        o = cjacobi.CGrid(mc, t, g)
        o.sweep(pb.iterations)
        out.append((o.x.copy(), o.image(), o.err64()))
    return out


def test_batch_jobs_equal_the_oracle(jobs, oracle_results):
    from fpie_gb300.batch import BatchSolver

    b = BatchSolver(40e9)
    ids = [b.add(mc, t, g, pb.iterations) for pb, mc, t, g in jobs]
    b.run()
    for jid, (pb, mc, t, g), (x, img, err) in zip(ids, jobs, oracle_results):
        assert b.progress(jid) == (pb.iterations, pb.iterations)
        np.testing.assert_array_equal(b.state(jid), x, err_msg=pb.name)
        bimg, berr = b.result(jid)
        np.testing.assert_array_equal(bimg, img, err_msg=pb.name)
        np.testing.assert_allclose(berr, err, rtol=1e-5, err_msg=pb.name)


def test_batch_in_epochs_equals_the_oracle(jobs, oracle_results):
    """The serving engine's use: the same jobs advanced in 256-sweep runs."""
    from fpie_gb300.batch import BatchSolver

    b = BatchSolver(40e9)
    ids = [b.add(mc, t, g, pb.iterations) for pb, mc, t, g in jobs]
    while any(b.progress(j)[0] < b.progress(j)[1] for j in ids):
        b.run(256)
    for jid, (pb, *_), (x, img, err) in zip(ids, jobs, oracle_results):
        np.testing.assert_array_equal(b.state(jid), x, err_msg=pb.name)


def test_served_results_equal_the_oracle(jobs):
    """The same sixteen jobs as serving requests (images in, inputs built on
    the GPU, 256-sweep epochs, stop at max |r| <= 1e-3 per channel or 10000
    sweeps): every result equals the oracle after the request's own sweeps."""
    from fpie_gb300.serve import Request, Server

    srv = Server(budget_bytes=40e9, epoch_sweeps=256, tol=1e-3, max_sweeps=10000)
    for k, (pb, *_) in enumerate(jobs):
        srv.submit(Request(k, problem=pb))
    t = iter(range(10**9))
    srv.drain(lambda: float(next(t)))
    assert len(srv.finished) == len(jobs)
    for r in srv.finished:
        pb, mc, t, g = jobs[r.rid]
        assert r.max_residual <= 1e-3 or r.sweeps == 10000
        o = cjacobi.CGrid(mc, t, g)
        o.sweep(r.sweeps)
        np.testing.assert_array_equal(r.img, o.image(), err_msg=pb.name)
        np.testing.assert_allclose(r.err, o.err64(), rtol=1e-5, err_msg=pb.name)
