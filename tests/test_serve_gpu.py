"""Serving loop on the GPU: each result is the same alone and in the mix, and
equals the oracle's at the request's own sweep count."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(300)]


def _requests():
    from fpie_gb300.serve import make_requests

    return make_requests(6, seed=3, max_box=160)


def _serve(reqs, **kw):
    from fpie_gb300.serve import Server

    srv = Server(**kw)
    for r in reqs:
        srv.submit(r)
    t = iter(range(10**9))
    srv.drain(lambda: float(next(t)))
    return {r.rid: r for r in srv.finished}, srv


def test_alone_equals_in_the_mix():
    kw = dict(budget_bytes=4e9, epoch_sweeps=128, tol=1e-3, max_sweeps=3000)
    mixed, _ = _serve(_requests(), **kw)
    assert len(mixed) == 6
    for rid in range(6):
        alone, _ = _serve([_requests()[rid]], **kw)
        a, b = alone[rid], mixed[rid]
        assert a.sweeps == b.sweeps
        np.testing.assert_array_equal(a.img, b.img)
        np.testing.assert_array_equal(a.err, b.err)


def test_results_match_the_oracle_and_stop_rule():
    """Requests carry images; the server builds the inputs on the GPU.  Each
    result equals the oracle's C restatement of the reference's Jacobi grid
    solver run on the host-built inputs (GridProcessor.reset semantics) for
    the request's own sweep count: image bit for bit, err rtol 1e-5."""
    from fpie_gb300 import prep
    from oracle import cjacobi

    res, srv = _serve(_requests(), budget_bytes=4e9, epoch_sweeps=128, tol=1e-3, max_sweeps=3000)
    for rid, r in res.items():
        assert r.max_residual <= 1e-3 or r.sweeps == 3000
        assert r.sweeps % 128 == 0 or r.sweeps == 3000
        pb = r.problem
        mc, t, g, box = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                         pb.gradient)
        assert r.box == (box.x0, box.x1, box.y0, box.y1)
        o = cjacobi.CGrid(mc, t, g)
        o.sweep(r.sweeps)
        np.testing.assert_array_equal(r.img, o.image())
        np.testing.assert_allclose(r.err, o.err64(), rtol=1e-5)


def test_prebuilt_requests_equal_image_requests():
    from fpie_gb300.serve import make_requests

    kw = dict(budget_bytes=4e9, epoch_sweeps=128, tol=1e-3, max_sweeps=3000)
    a, _ = _serve(_requests(), **kw)
    b, _ = _serve(make_requests(6, seed=3, max_box=160, prebuilt=True), **kw)
    for rid in a:
        assert a[rid].sweeps == b[rid].sweeps
        np.testing.assert_array_equal(a[rid].img, b[rid].img)
        np.testing.assert_array_equal(a[rid].err, b[rid].err)


def test_budget_limits_concurrency():
    from fpie_gb300.batch import BatchSolver

    reqs = _requests()
    biggest = max(BatchSolver.job_bytes(*r.size_bound()) for r in reqs)
    res, srv = _serve(reqs, budget_bytes=2.2 * biggest, epoch_sweeps=256, tol=1e-2, max_sweeps=2000)
    assert len(res) == 6 and srv.peak_active <= 2


def test_poisson_replay_reports_latency_percentiles():
    from fpie_gb300.serve import run_workload

    stats = run_workload(_requests(), rate=200.0, budget_bytes=4e9, epoch_sweeps=256, tol=1e-2,
                         max_sweeps=2000)
    assert stats["requests"] == 6
    lat = stats["latency_ms"]
    assert 0 < lat["p50"] <= lat["p95"] <= lat["p99"] <= lat["max"]


def test_unservable_request_is_rejected_and_the_rest_served():
    """An image request whose mask selects nothing (after its frame is
    cleared) is refused at admission with the engine's message; the other
    requests are served as usual."""
    from fpie_gb300.serve import Request

    reqs = _requests()[:3]
    bad = reqs[1].problem
    bad = type(bad)(bad.name, bad.src, bad.mask * 0, bad.tgt, bad.mask_on_src, bad.mask_on_tgt,
                    bad.gradient, bad.iterations)
    reqs[1] = Request(reqs[1].rid, problem=bad)
    res, srv = _serve(reqs, budget_bytes=4e9, epoch_sweeps=128, tol=1e-3, max_sweeps=3000)
    assert [r.rid for r in srv.rejected] == [reqs[1].rid]
    assert "no pixel" in srv.rejected[0].error
    assert sorted(res) == sorted(r.rid for r in reqs if r.rid != reqs[1].rid)
