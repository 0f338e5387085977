"""Serving form: continuous batching of paste requests on one GPU.

Requests (grid problems from ``prep.grid_inputs``) arrive over time.  The
server admits a request when the HBM budget has room for it, keeps its
state on the device (``BatchSolver``), and advances every admitted request
together in epochs of ``epoch_sweeps`` sweeps -- one persistent kernel
launch per epoch -- so requests that arrive while others run join the next
epoch instead of waiting for the batch to drain.  After each epoch the FP64
residual norms decide which requests are done: max |r| <= ``tol`` in every
channel, or ``max_sweeps`` reached.  Done requests are read back and their
memory is freed for the queue.

A request's schedule depends only on itself: it advances exactly
``epoch_sweeps`` per epoch from its admission and is checked at the same
sweep counts, so its result is bit-identical whether it runs alone or in
any mix (the kernels are deterministic).

Latency = completion time - arrival time.  ``run_workload`` replays a
seeded Poisson arrival stream in real time and reports throughput and
p50/p95/p99 latency.  Command line:

    python -m fpie_gb300.serve --rate 500 --jobs 128
"""

from __future__ import annotations

import argparse
import collections
import dataclasses
import json
import time

import numpy as np

from .batch import BatchSolver


@dataclasses.dataclass
class Request:
    rid: int
    mask: np.ndarray
    tgt: np.ndarray
    grad: np.ndarray
    arrival: float = 0.0
    admitted: float | None = None
    done: float | None = None
    sweeps: int = 0
    img: np.ndarray | None = None
    err: np.ndarray | None = None
    max_residual: float | None = None
    job: int | None = None


class Server:
    def __init__(self, budget_bytes: float = 40e9, epoch_sweeps: int = 256, tol: float = 1e-3,
                 max_sweeps: int = 10000, kernel: str = "auto", batch=None,
                 job_bytes=None, precision: str = "fp32") -> None:
        if epoch_sweeps <= 0 or max_sweeps <= 0:
            raise ValueError("epoch_sweeps and max_sweeps must be positive")
        # `batch` / `job_bytes` replace the GPU engine (tests of the host logic).
        self.batch = batch if batch is not None else BatchSolver(budget_bytes, precision)
        self.job_bytes = job_bytes or self.batch.job_bytes_for
        if kernel != "auto":
            self.batch.set_kernel(kernel)
        self.budget = budget_bytes
        self.epoch = epoch_sweeps
        self.tol = tol
        self.max_sweeps = max_sweeps
        self.queue: collections.deque[Request] = collections.deque()
        self.active: dict[int, Request] = {}
        self.finished: list[Request] = []
        self.epochs = 0
        self.peak_active = 0

    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _admit(self, now: float) -> None:
        while self.queue:
            req = self.queue[0]
            need = self.job_bytes(*req.mask.shape)
            used, budget = self.batch.memory()
            if used + need > budget:
                if not self.active:
                    raise RuntimeError(f"request {req.rid} needs {need} B, more than the whole budget")
                return
            self.queue.popleft()
            req.job = self.batch.add(req.mask, req.tgt, req.grad, self.max_sweeps)
            req.admitted = now
            self.active[req.job] = req
        self.peak_active = max(self.peak_active, len(self.active))

    def step(self, clock) -> int:
        """Admit what fits, run one epoch, retire converged requests; returns retired count."""
        self._admit(clock())
        if not self.active:
            return 0
        self.batch.run(self.epoch)
        self.epochs += 1
        ids = list(self.active)
        norms = self.batch.norms(ids)
        retired = 0
        for jid, nrm in zip(ids, norms):
            req = self.active[jid]
            done, total = self.batch.progress(jid)
            req.sweeps = done
            req.max_residual = float(nrm[:3].max())
            if req.max_residual <= self.tol or done >= total:
                req.img, req.err = self.batch.result(jid)
                req.done = clock()
                self.batch.remove(jid)
                del self.active[jid]
                self.finished.append(req)
                retired += 1
        return retired

    def drain(self, clock) -> None:
        while self.queue or self.active:
            self.step(clock)


def percentile(xs, q):
    return float(np.percentile(np.asarray(xs, np.float64), q)) if xs else None


def run_workload(requests: list[Request], rate: float, seed: int = 0, **server_kw) -> dict:
    """Replay Poisson arrivals at `rate` requests/s in real time; return stats."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(requests))
    arrivals = np.cumsum(gaps)
    srv = Server(**server_kw)
    t0 = time.perf_counter()
    clock = lambda: time.perf_counter() - t0  # noqa: E731
    pending = collections.deque(zip(arrivals, requests))
    while pending or srv.queue or srv.active:
        now = clock()
        while pending and pending[0][0] <= now:
            at, req = pending.popleft()
            req.arrival = float(at)
            srv.submit(req)
        if not srv.queue and not srv.active:
            if pending:
                time.sleep(max(0.0, pending[0][0] - clock()))
            continue
        srv.step(clock)
    wall = clock()
    lat = [r.done - r.arrival for r in srv.finished]
    unknowns = sum(int((r.mask != 0).sum()) * r.sweeps for r in srv.finished)
    return {
        "requests": len(srv.finished),
        "rate_per_s": rate,
        "wall_s": wall,
        "throughput_req_per_s": len(srv.finished) / wall,
        "pixel_updates_per_s": unknowns / wall,
        "latency_ms": {"p50": 1e3 * percentile(lat, 50), "p95": 1e3 * percentile(lat, 95),
                       "p99": 1e3 * percentile(lat, 99), "max": 1e3 * max(lat)},
        "epochs": srv.epochs,
        "peak_active": srv.peak_active,
        "sweeps_mean": float(np.mean([r.sweeps for r in srv.finished])),
        "converged": sum(1 for r in srv.finished if r.max_residual <= srv.tol),
        "kernel": srv.batch.kernel,
        "precision": srv.batch.precision,
    }


def make_requests(n_jobs: int, seed: int = 7, max_box: int = 1024) -> list[Request]:
    """Requests drawn from the batched-jobs distribution (workloads.job_mix)."""
    from . import prep, workloads

    reqs = []
    for k, pb in enumerate(workloads.job_mix(n_jobs=n_jobs, seed=seed, max_box=max_box)):
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        reqs.append(Request(k, mc, t, g))
    return reqs


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--rate", type=float, default=500.0, help="arrivals per second")
    ap.add_argument("--jobs", type=int, default=128)
    ap.add_argument("--epoch", type=int, default=256)
    ap.add_argument("--budget-gb", type=float, default=40.0)
    ap.add_argument("--max-box", type=int, default=1024)
    ap.add_argument("--precision", choices=["fp32", "fp16", "bf16"], default="fp32")
    args = ap.parse_args()
    reqs = make_requests(args.jobs, max_box=args.max_box)
    stats = run_workload(reqs, args.rate, budget_bytes=args.budget_gb * 1e9, epoch_sweeps=args.epoch,
                         precision=args.precision)
    print(json.dumps(stats))


if __name__ == "__main__":
    main()
