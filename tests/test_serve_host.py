"""Host logic of the serving loop, driven by a fake batch engine (no GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from fpie_gb300.serve import Request, Server


class FakeBatch:
    """Residual of job j halves every epoch from its own start value."""

    def __init__(self, budget):
        self.budget, self.used, self.jobs, self.next_id = budget, 0, {}, 0
        self.run_calls = []

    precision = "fp32"

    def memory(self):
        return self.used, self.budget

    def add(self, mask, tgt, grad, iterations):
        jid = self.next_id
        self.next_id += 1
        self.jobs[jid] = {"done": 0, "total": iterations, "r0": float(tgt.flat[0]), "n": mask.size}
        self.used += mask.size
        return jid

    def run(self, limit):
        self.run_calls.append(sorted(self.jobs))
        for j in self.jobs.values():
            j["done"] = min(j["total"], j["done"] + limit)

    def norms(self, ids):
        out = np.zeros((len(ids), 6))
        for k, jid in enumerate(ids):
            j = self.jobs[jid]
            out[k, :3] = j["r0"] * 0.5 ** (j["done"] // 100)
        return out

    def progress(self, jid):
        return self.jobs[jid]["done"], self.jobs[jid]["total"]

    def result(self, jid):
        return np.zeros((1, 1, 3), np.uint8), np.zeros(3, np.float32)

    def remove(self, jid):
        self.used -= self.jobs.pop(jid)["n"]


def _req(rid, side, r0):
    mask = np.ones((side, side), np.int32)
    return Request(rid, mask, np.full((side, side, 3), r0, np.float32), np.zeros((side, side, 3), np.float32))


def test_admission_respects_budget_and_everything_finishes():
    fb = FakeBatch(budget=250)
    srv = Server(epoch_sweeps=100, tol=1e-3, max_sweeps=10000, batch=fb, job_bytes=lambda n, m: n * m)
    for k in range(6):
        srv.submit(_req(k, 10, r0=2.0 ** (k + 3)))  # 100 "bytes" each: at most 2 active
    t = iter(range(10**6))
    srv.drain(lambda: float(next(t)))
    assert len(srv.finished) == 6 and not srv.active and fb.used == 0
    assert srv.peak_active == 2
    assert all(len(c) <= 2 for c in fb.run_calls)
    for r in srv.finished:  # stopped at the first epoch whose residual met tol
        assert r.max_residual <= 1e-3 and r.max_residual > 1e-3 * 0.5 - 1e-12


def test_sweep_cap_retires_unconverged_requests():
    fb = FakeBatch(budget=1000)
    srv = Server(epoch_sweeps=256, tol=1e-30, max_sweeps=600, batch=fb, job_bytes=lambda n, m: n * m)
    srv.submit(_req(0, 5, r0=1.0))
    t = iter(range(10**6))
    srv.drain(lambda: float(next(t)))
    (r,) = srv.finished
    assert r.sweeps == 600 and r.max_residual > 1e-30


def test_request_larger_than_budget_is_rejected_and_the_rest_served():
    fb = FakeBatch(budget=30)
    srv = Server(epoch_sweeps=100, tol=1e-3, max_sweeps=10000, batch=fb, job_bytes=lambda n, m: n * m)
    srv.submit(_req(0, 6, r0=1.0))   # 36 "bytes": can never fit
    srv.submit(_req(1, 5, r0=8.0))   # 25: fits
    t = iter(range(10**6))
    srv.drain(lambda: float(next(t)))
    assert [r.rid for r in srv.rejected] == [0] and "budget" in srv.rejected[0].error
    assert [r.rid for r in srv.finished] == [1] and srv.finished[0].error is None


def test_request_the_engine_refuses_is_rejected():
    from fpie_gb300._abi import FpieArgumentError

    class Refusing(FakeBatch):
        def add(self, mask, tgt, grad, iterations):
            if not mask.any():
                raise FpieArgumentError("the mask selects no pixel")
            return super().add(mask, tgt, grad, iterations)

    fb = Refusing(budget=1000)
    srv = Server(epoch_sweeps=100, tol=1e-3, max_sweeps=10000, batch=fb, job_bytes=lambda n, m: n * m)
    empty = _req(0, 5, r0=1.0)
    empty.mask[:] = 0
    srv.submit(empty)
    srv.submit(_req(1, 5, r0=4.0))
    t = iter(range(10**6))
    srv.drain(lambda: float(next(t)))
    assert [r.rid for r in srv.rejected] == [0] and "no pixel" in srv.rejected[0].error
    assert [r.rid for r in srv.finished] == [1]
