"""Serving form: continuous batching of paste requests on one GPU.

A request is a paste job as a user submits it: the source, mask and target
images, the offsets and the gradient mode.  The server admits a request
when the HBM budget has room for it (the mask image's size bounds the
crop), builds its solver inputs on the GPU (``BatchSolver.add_images``: the
mask threshold and crop on the host, gradient mixing and layout on the
device), keeps its state on the device, and advances every admitted request
together in epochs of ``epoch_sweeps`` sweeps -- one persistent kernel
launch per epoch.  Each epoch is queued without waiting, followed by the
FP64 residual norms of its requests and one copy of them to pinned host
memory; while it runs, requests that arrived meanwhile are admitted (their
inputs are built behind the epoch on the device and they join the next
one).  Then the norms decide which requests are done: max |r| <= ``tol`` in
every channel, or ``max_sweeps`` reached.  Done requests are read back and
their memory returns to the pool once the device is past them.

A request's schedule depends only on itself: it advances exactly
``epoch_sweeps`` per epoch from its admission and is checked at the same
sweep counts, so its result is bit-identical whether it runs alone or in
any mix (the kernels are deterministic).

Latency = completion time - arrival time, so it includes the queueing
before admission and the construction of the solver inputs.
``run_workload`` replays a seeded Poisson arrival stream in real time and
reports throughput and p50/p95/p99 latency.  Command line:

    python -m fpie_gb300.serve --rate 500 --requests 1000
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
    """A paste request: ``problem`` (images in), or prebuilt grid inputs
    (``mask``, ``tgt``, ``grad``, as GridSolver.reset takes them)."""

    rid: int
    mask: np.ndarray | None = None
    tgt: np.ndarray | None = None
    grad: np.ndarray | None = None
    problem: object | None = None
    arrival: float = 0.0
    admitted: float | None = None
    done: float | None = None
    sweeps: int = 0
    img: np.ndarray | None = None
    err: np.ndarray | None = None
    max_residual: float | None = None
    job: int | None = None
    box: tuple | None = None
    error: str | None = None  # why the request was rejected (then img is None)

    def size_bound(self) -> tuple[int, int]:
        """Rows and columns of a grid at least as large as the request's crop."""
        if self.problem is not None:
            return tuple(self.problem.mask.shape[:2])
        return tuple(self.mask.shape)


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
        self.rejected: list[Request] = []  # refused at admission (req.error says why)
        self.epochs = 0
        self.peak_active = 0

    def submit(self, req: Request) -> None:
        self.queue.append(req)

    def _reject(self, req: Request, now: float, why: str) -> None:
        req.error = why
        req.done = now
        self.rejected.append(req)

    def _admit(self, now: float) -> None:
        from ._abi import FpieArgumentError

        while self.queue:
            req = self.queue[0]
            need = self.job_bytes(*req.size_bound())
            used, budget = self.batch.memory()
            if need > budget:  # can never fit: refuse it, serve the rest
                self.queue.popleft()
                self._reject(req, now, f"needs {need} B, more than the whole budget of {budget:.0f} B")
                continue
            if used + need > budget:
                return  # waits for running requests to free memory
            self.queue.popleft()
            try:
                if req.problem is not None:
                    pb = req.problem
                    req.job, req.box = self.batch.add_images(pb.src, pb.mask, pb.tgt, pb.mask_on_src,
                                                             pb.mask_on_tgt, pb.gradient,
                                                             self.max_sweeps)
                else:
                    req.job = self.batch.add(req.mask, req.tgt, req.grad, self.max_sweeps)
            except FpieArgumentError as exc:  # e.g. an empty mask, a crop off the image
                self._reject(req, now, str(exc))
                continue
            req.admitted = now
            self.active[req.job] = req
        self.peak_active = max(self.peak_active, len(self.active))

    def step(self, clock, poll=None) -> int:
        """Admit what fits, run one epoch, retire converged requests; returns
        retired count.  ``poll`` (optional) is called while the epoch runs on
        the device; it may submit newly arrived requests, which are admitted
        then and join the next epoch."""
        self._admit(clock())
        if not self.active:
            return 0
        ids = list(self.active)
        before = {jid: self.active[jid].sweeps for jid in ids}
        if hasattr(self.batch, "run_async"):
            self.batch.run_async(self.epoch)
            self.batch.norms_async(ids)
            if poll is not None:
                poll()
                self._admit(clock())
            norms = self.batch.norms_wait()
            self.batch.wait()
        else:
            self.batch.run(self.epoch)
            norms = self.batch.norms(ids)
        self.epochs += 1
        retired = 0
        for jid, nrm in zip(ids, norms):
            req = self.active[jid]
            done, total = self.batch.progress(jid)
            if done <= before[jid] and done < total:
                raise RuntimeError(f"request {req.rid} made no progress in an epoch")
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

    def poll():
        now = clock()
        while pending and pending[0][0] <= now:
            at, req = pending.popleft()
            req.arrival = float(at)
            srv.submit(req)

    while pending or srv.queue or srv.active:
        poll()
        if not srv.queue and not srv.active:
            if pending:
                time.sleep(max(0.0, pending[0][0] - clock()))
            continue
        srv.step(clock, poll)
    wall = clock()
    lat = [r.done - r.arrival for r in srv.finished]
    wait = [r.admitted - r.arrival for r in srv.finished]
    unknowns = sum(_unknowns(r) * r.sweeps for r in srv.finished)

    def pct(xs):
        if not xs:
            return {"p50": None, "p95": None, "p99": None, "max": None}
        return {"p50": 1e3 * percentile(xs, 50), "p95": 1e3 * percentile(xs, 95),
                "p99": 1e3 * percentile(xs, 99), "max": 1e3 * max(xs)}

    return {
        "requests": len(srv.finished),
        "rejected": len(srv.rejected),
        "rate_per_s": rate,
        "wall_s": wall,
        "throughput_req_per_s": len(srv.finished) / wall,
        "pixel_updates_per_s": unknowns / wall,
        "latency_ms": pct(lat),
        "admission_wait_ms": pct(wait),
        "epochs": srv.epochs,
        "peak_active": srv.peak_active,
        "sweeps_mean": float(np.mean([r.sweeps for r in srv.finished])),
        "converged": sum(1 for r in srv.finished if r.max_residual <= srv.tol),
        "kernel": srv.batch.kernel,
        "precision": srv.batch.precision,
    }


def _unknowns(req: Request) -> int:
    """Masked pixels of a request (the reference's threshold, frame cleared)."""
    if req.problem is None:
        return int((req.mask != 0).sum())
    m = np.asarray(req.problem.mask)
    on = (m.astype(np.int32).sum(axis=2) >= 384) if m.ndim == 3 else (m >= 128)
    return int(on[1:-1, 1:-1].sum())


def make_requests(n_requests: int, seed: int = 7, max_box: int = 1024, pool: int | None = None,
                  prebuilt: bool = False) -> list[Request]:
    """Requests drawn from the batched-jobs distribution (workloads.job_mix).

    With ``pool`` the requests are drawn (seeded, with replacement) from
    ``pool`` generated jobs instead of generating every one; ``prebuilt``
    builds the grid inputs on the host (``prep.grid_inputs``) instead of
    carrying the images."""
    from . import prep, workloads

    jobs = workloads.job_mix(n_jobs=pool or n_requests, seed=seed, max_box=max_box)
    if pool:
        rng = np.random.default_rng(seed + 1)
        jobs = [jobs[int(k)] for k in rng.integers(0, len(jobs), size=n_requests)]
    reqs = []
    for k, pb in enumerate(jobs):
        if prebuilt:
            mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                           pb.gradient)
            reqs.append(Request(k, mc, t, g))
        else:
            reqs.append(Request(k, problem=pb))
    return reqs


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--rate", type=float, default=500.0, help="arrivals per second")
    ap.add_argument("--requests", type=int, default=1000)
    ap.add_argument("--pool", type=int, default=256, help="distinct generated jobs to draw from")
    ap.add_argument("--epoch", type=int, default=256)
    ap.add_argument("--budget-gb", type=float, default=40.0)
    ap.add_argument("--max-box", type=int, default=1024)
    ap.add_argument("--precision", choices=["fp32", "fp16", "bf16"], default="fp32")
    args = ap.parse_args()
    reqs = make_requests(args.requests, max_box=args.max_box, pool=args.pool)
    stats = run_workload(reqs, args.rate, budget_bytes=args.budget_gb * 1e9, epoch_sweeps=args.epoch,
                         precision=args.precision)
    print(json.dumps(stats))


if __name__ == "__main__":
    main()
