#!/usr/bin/env python3
"""Benchmark of the GB300 Jacobi backend on the square800 paste workload.

Workload (one step): the fpie GridSolver path on the 'square800' problem --
an 800x800 square (640,000 unknowns, 802x802 crop) pasted from a 900^2
source into a 1024^2 target with the 'max' gradient -- reset from inputs
already resident in HBM, then 5000 FP32 Jacobi sweeps, the residual and the
uint8 image.  Metric: pixel-updates/s = unknowns x sweeps / time.

Printed JSON line (rank 0):
* ``value``     device-timed (CUDA events on the launching stream), inputs in
                HBM; L2 is flushed between steps (a 512 MiB write), outside
                the timed events;
* ``e2e``       the same work through the plugin API a user calls:
                ``GridSolver.reset`` from pinned host arrays (H2D inside) and
                ``GridSolver.step(5000)`` returning the uint8 image (D2H);
* ``roofline``  the sweep kernel: algorithmic bytes per launch / its average
                launch duration, against the measured HBM copy bandwidth;
* ``cpu_baseline`` the oracle's C restatement (OpenMP, all host threads) on a
                bounded number of sweeps of the same problem;
* ``equ``       the EquSolver form of the same problem, device-timed;
* ``mixed_fp16`` the FP16-correction refinement form, device-timed;
* ``error_vs_fp64`` (with the CPU baseline) how far the 5000-sweep result is
                from the converged FP64 solution of the same system;
* ``reference_cuda`` (with the CPU baseline) the reference's own CUDA
                solvers on the same GPU: step time at 5000 sweeps, residual
                sum and error against the converged solution, and the GB300
                solvers' sweeps and time to the same error and to the same
                residual sum.

``--impl reference`` times the CPU implementation of the path instead (the
C restatement of the reference's Jacobi solvers, all host threads), on a
bounded sample of each step, and prints the same metric.  Under torchrun
with N>1 every rank runs an independent replica (the path has no exchange
step); the reference arm runs on rank 0 only.
"""

from __future__ import annotations

import argparse
import json
import re
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SWEEPS = 5000
GRID_BYTES_PER_PX = 37   # read x 12 + read grad 12 + write x 12 + mask 1 (FP32 sweep)
EQU_BYTES_PER_UNKNOWN = 52  # A 16 + B 12 + read X 12 + write X 12
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--sweeps", type=int, default=SWEEPS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-equ", action="store_true")
    p.add_argument("--kernel", default="auto",
                   help="grid sweep kernel ('auto' = autotuned; a name pins one, e.g. for profiling)")
    p.add_argument("--workload", choices=["square800", "batch", "serve"], default="square800",
                   help="square800 (default, the headline line); batch: 256 uneven jobs in one "
                        "persistent launch vs one GridSolver per job; serve: Poisson arrivals")
    p.add_argument("--jobs", type=int, default=256)
    p.add_argument("--rates", default="50,200,500,1000,2000")
    p.add_argument("--precision", choices=["fp32", "fp16", "bf16"], default="fp32",
                   help="batch/serve workloads: FP32 or a mixed form")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def job_time_max(ms: float, world: int, device=None) -> float:
    """The whole job's time: the max over ranks of each rank's timed
    milliseconds (with N > 1 every rank runs an independent replica; the
    path has no exchange step).  `device` None = a CPU tensor (gloo)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_step: float, steps: int, world: int, ms: float) -> float:
    """Units all ranks processed (each rank the same replica work) per second
    of the slowest rank's time."""
    return units_per_step * steps * world / (ms / 1e3)


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def kernel_shape(kernel: str, sweeps: int):
    """(sweeps per launch, launches per step, region passes per launch) of a
    grid sweep kernel, from its name: "sweep1"; "r/p<R>w<W>k<K>[s|t]" (K
    sweeps per launch); "p16w8k16d" (dependency flow: the whole step in one
    launch, a pass per 16-sweep level); "res16w8k4" (resident: the whole step
    in one launch, one region load)."""
    if kernel == "sweep1":
        return 1, sweeps, 1
    depth = int(re.search(r"k(\d+)", kernel).group(1))
    if kernel.endswith("d"):
        return sweeps, 1, -(-sweeps // depth)
    if kernel.startswith("res"):
        return sweeps, 1, 1
    return depth, -(-sweeps // depth), 1


def profiled_traffic(name: str):
    """dram bytes per launch from a committed ncu summary, if there is one."""
    f = ROOT / "profiles" / f"{name}.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi samples (every 100 ms) while the timed region runs."""

    FIELDS = ["index", "clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={','.join(self.FIELDS)}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) == len(self.FIELDS):
                    rows.append(parts)
        os.unlink(self.out.name)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "", 1).isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "", 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "", 1).isdigit()), default=None)}


def square800_inputs():
    from fpie_gb300 import prep, workloads

    pb = workloads.square800(SWEEPS)
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    return pb, mc, t, g


def cpu_baseline_grid(mc, t, g, budget_s: float = 10.0):
    """The oracle's C restatement timed on a bounded number of sweeps."""
    from oracle import cjacobi

    th = host_threads()
    o = cjacobi.CGrid(mc, t, g, nthreads=th)
    o.sweep(3)
    t0 = time.perf_counter()
    o.sweep(20)
    per = (time.perf_counter() - t0) / 20
    n_sw = int(max(20, min(SWEEPS, budget_s / max(per, 1e-9))))
    o = cjacobi.CGrid(mc, t, g, nthreads=th)
    t0 = time.perf_counter()
    o.sweep(n_sw)
    o.err64()
    o.image()
    dt = time.perf_counter() - t0
    unknowns = int((mc != 0).sum())
    return {"value": unknowns * n_sw / dt, "unit": "pixel-updates/s", "cores": th, "kind": "port",
            "sample": f"{n_sw} of {SWEEPS} sweeps of square800 GridSolver (640,000 unknowns) + residual + "
                      f"clip, oracle C restatement (OpenMP), {th} threads, {dt:.2f} s"}


def fp64_solution(mc, t, g):
    """The converged solution of the grid system (oracle FP64 conjugate
    gradient, checked against a direct solve in the tests) and its time."""
    from oracle import fp64

    t0 = time.perf_counter()
    x64 = fp64.cg_torch(mc, t, g, device="cuda", rtol=1e-12)
    return x64, time.perf_counter() - t0


def err_stats(x, x64, mc) -> dict:
    """max and mean |x - x64| over masked pixels, in intensity units (LSB)."""
    d = np.abs(np.asarray(x, np.float64) - x64)[np.asarray(mc) != 0]
    return {"max_abs": float(d.max()), "mean_abs": float(d.mean())}


def equ_on_grid(X, sysm, origin, shape):
    """An EquSolver state (rows 1..N-1) placed on the crop grid."""
    x = np.zeros(shape, np.float32)
    r, c = sysm.tgt_index
    x[r - origin[0], c - origin[1]] = np.asarray(X)[1:]
    return x


def error_vs_fp64(x, x64, mc, seconds) -> dict:
    """How far a result is from the converged solution."""
    return {**err_stats(x, x64, mc), "unit": "intensity (LSB)", "sweeps": SWEEPS,
            "reference": "FP64 conjugate gradient, rtol 1e-12", "seconds": round(seconds, 2),
            "note": "the benchmark's 5000 Jacobi sweeps are far from converged on an "
                    "800x800 paste; the precision study runs to <= 0.5 LSB"}


def _median_step_s(reset, step, n: int, reps: int = 3) -> float:
    """Median wall time of step(n) from a fresh reset (step synchronizes)."""
    ts = []
    for _ in range(reps):
        reset()
        t0 = time.perf_counter()
        step(n)
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def _first_reaching(reset, step, value, target: float, start: int, chunk: int, cap: int):
    """The first sweep count start + j * chunk (at most cap) after which
    value() <= target, and that value."""
    reset()
    step(start)
    n, v = start, value()
    while v > target and n < cap:
        step(chunk)
        n += chunk
        v = value()
    return n, v


def reference_cuda(mc, t, g, sysm, x64, origin) -> dict:
    """The reference's own CUDA solvers on this GPU -- its kernels, compiled
    from its sources (oracle/ref_cuda.py), driven by a restatement of its
    step loop -- beside the GB300 backend on the same problem.

    Reported for each: the 5000-sweep step time, the residual sum (the
    reference's err) and the error against the converged FP64 solution.
    The reference's kernels update in place, which damps the high
    frequencies that dominate the residual sum far faster than Jacobi does,
    while the error against the converged solution is set by the slowest
    (low-frequency) modes, which in-place and Jacobi sweeps reduce at nearly
    the same rate per sweep.  So two comparisons are given: at matched error
    (the GB300 Jacobi sweeps whose max |x - x64| is <= the reference's after
    5000) and at matched residual sum."""
    from fpie_gb300 import backend, prep, workloads
    from oracle import cjacobi, ref_cuda

    why = ref_cuda.unavailable_reason()
    if why:
        return {"unavailable": why}
    unknowns = int((mc != 0).sum())
    cap = 40 * SWEEPS
    r = ref_cuda.RefCudaGrid(8, 8)
    r.reset(mc, t, g)
    r.step(SWEEPS)  # warm-up
    ref_s = _median_step_s(lambda: r.reset(mc, t, g), r.step, SWEEPS)
    o = cjacobi.CGrid(mc, t, g)
    o.x = r.state()
    ref_res = float(o.err64().sum())
    ref_err = err_stats(o.x, x64, mc)

    s = backend.GridSolver(8, 8)
    g_reset = lambda: s.reset(mc.size, mc, t, g)  # noqa: E731

    last = {}

    def g_step_keep(n):
        last["err"] = s.step(n)[1]

    def g_res():  # the solver's own residual sum of its last step
        return float(np.asarray(last["err"], np.float64).sum())

    def g_err():
        return err_stats(s.state(), x64, mc)["max_abs"]

    n_err, v_err = _first_reaching(g_reset, s.step, g_err, ref_err["max_abs"], SWEEPS // 2, 50, cap)
    t_err = _median_step_s(g_reset, s.step, n_err)
    n_res, v_res = _first_reaching(g_reset, g_step_keep, g_res, ref_res, SWEEPS, 250, cap)
    t_res = _median_step_s(g_reset, s.step, n_res)
    out = {
        "grid": {
            "reference": {"value": unknowns * SWEEPS / ref_s, "unit": "pixel-updates/s",
                          "ms_per_step": ref_s * 1e3, "sweeps": SWEEPS, "residual_sum": ref_res,
                          "error_vs_fp64": ref_err,
                          "kernel": "iter_grid_kernel, one launch per sweep, 8x8 blocks, in place"},
            "matched_error": {"gb300_sweeps": n_err, "gb300_ms": t_err * 1e3, "gb300_max_abs": v_err,
                              "reference_ms": ref_s * 1e3},
            "matched_residual": {"gb300_sweeps": n_res, "gb300_ms": t_res * 1e3,
                                 "gb300_residual_sum": v_res, "reference_ms": ref_s * 1e3,
                                 "gb300_error_vs_fp64": err_stats(s.state(), x64, mc)},
        },
        "note": "the reference's fpie/core/cuda kernels compiled from its sources for sm_103a, host "
                "step loop restated over the driver API; wall times of step(n) from a reset, incl. "
                "the image and err copies back, median of 3; matched_* = the first GB300 sweep count "
                "(steps of 50 for the error, 250 for the residual) reaching the reference's value "
                "after 5000",
    }
    if sysm is None:
        return out

    # EquSolver: the reference's in-place kernel, the GB300 Jacobi and the
    # GB300 red-black order (the reference's OpenMP iteration, own numbering).
    q = ref_cuda.RefCudaEqu(1024)
    q.reset(sysm.N, sysm.A, sysm.X, sysm.B)
    q.step(SWEEPS)
    qref_s = _median_step_s(lambda: q.reset(sysm.N, sysm.A, sysm.X, sysm.B), q.step, SWEEPS)
    qo = cjacobi.CEqu(sysm.A, sysm.X, sysm.B)
    qo.X = q.state()
    qref_res = float(qo.err64().sum())
    qref_err = err_stats(equ_on_grid(qo.X, sysm, origin, t.shape), x64, mc)
    equ = {"reference": {"value": (sysm.N - 1) * SWEEPS / qref_s, "unit": "pixel-updates/s",
                         "ms_per_step": qref_s * 1e3, "sweeps": SWEEPS, "residual_sum": qref_res,
                         "error_vs_fp64": qref_err,
                         "kernel": "iter_equ_kernel, one launch per sweep, blocks of 1024, in place"}}
    pb = workloads.square800(SWEEPS)
    rb = backend.EquSolver(1024, order="red_black")
    rsys = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                           rb.partition)
    for name, solver, system in (("gb300_jacobi", backend.EquSolver(1024), sysm),
                                 ("gb300_red_black", rb, rsys)):
        e_reset = (lambda solver=solver, system=system:  # noqa: E731
                   solver.reset(system.N, system.A, system.X, system.B))
        elast = {}

        def e_step_keep(n, solver=solver, elast=elast):
            elast["err"] = solver.step(n)[1]

        def e_res(elast=elast):
            return float(np.asarray(elast["err"], np.float64).sum())

        def e_err(solver=solver, system=system):
            return err_stats(equ_on_grid(solver.state(), system, origin, t.shape), x64, mc)["max_abs"]

        e_reset()
        solver.step(SWEEPS)
        at5000 = err_stats(equ_on_grid(solver.state(), system, origin, t.shape), x64, mc)
        t5000 = _median_step_s(e_reset, solver.step, SWEEPS)
        ne, ve = _first_reaching(e_reset, solver.step, e_err, qref_err["max_abs"], 50, 50, cap)
        te = _median_step_s(e_reset, solver.step, ne)
        nr, vr = _first_reaching(e_reset, e_step_keep, e_res, qref_res, 250, 250, cap)
        tr = _median_step_s(e_reset, solver.step, nr)
        equ[name] = {"value": (system.N - 1) * SWEEPS / t5000, "unit": "pixel-updates/s",
                     "ms_per_step": t5000 * 1e3, "error_vs_fp64": at5000, "kernel": solver.kernel,
                     "matched_error": {"sweeps": ne, "ms": te * 1e3, "max_abs": ve},
                     "matched_residual": {"sweeps": nr, "ms": tr * 1e3, "residual_sum": vr}}
    out["equ"] = equ
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import cjacobi

    pb, mc, t, g = square800_inputs()
    unknowns = int((mc != 0).sum())
    th = host_threads()
    o = cjacobi.CGrid(mc, t, g, nthreads=th)
    o.sweep(2)
    t0 = time.perf_counter()
    o.sweep(10)
    per = (time.perf_counter() - t0) / 10
    # Each step is a bounded sample so the whole run stays within ~2 minutes.
    budget = 120.0 / max(1, args.steps + args.warmup)
    n_sw = int(max(10, min(args.sweeps, budget / max(per, 1e-9))))

    def one_step():
        s = cjacobi.CGrid(mc, t, g, nthreads=th)  # reset: copy the inputs
        s.sweep(n_sw)
        s.err64()
        s.image()

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    dt = time.perf_counter() - t0
    value = unknowns * n_sw * args.steps / dt
    line = {
        "impl": "reference", "metric": "pixel-updates/s", "value": value, "unit": "pixel-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "square800 GridSolver FP32 Jacobi ('max' gradient, 640,000 unknowns, "
                               "802x802 crop)", "sweeps_per_step": n_sw, "sweeps_of_full_step": args.sweeps},
        "cpu_baseline": {"value": value, "unit": "pixel-updates/s", "cores": th, "kind": "port",
                         "sample": f"{n_sw} of {args.sweeps} sweeps per step, oracle C restatement of the "
                                   f"reference's Jacobi grid solver (OpenMP, {th} threads)"},
        "e2e": {"value": value, "unit": "pixel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gb300(args):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    from fpie_gb300 import backend, prep

    pb, mc, t, g = square800_inputs()
    n, m = mc.shape
    unknowns = int((mc != 0).sum())
    crop_px = n * m
    sweeps = args.sweeps
    stream = torch.cuda.current_stream()

    dm = torch.from_numpy(mc).to(dev)
    dt_ = torch.from_numpy(t).to(dev)
    dg = torch.from_numpy(g).to(dev)
    img = torch.empty((n, m, 3), dtype=torch.uint8, device=dev)
    err = torch.empty(3, dtype=torch.float32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    s = backend.GridSolver(8, 8)
    s.set_stream(stream.cuda_stream)
    if args.kernel != "auto":
        s.set_kernel(args.kernel)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def device_steps(k, solver, reset, finish, record):
        ev = []
        for _ in range(k):
            flush.zero_()  # L2 flush, outside the timed events
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            reset()
            solver.sweeps(sweeps)
            e1.record(stream)
            finish()
            e2.record(stream)
            ev.append((e0, e1, e2))
        if record:
            torch.cuda.synchronize()
            return [(a.elapsed_time(c), a.elapsed_time(b)) for a, b, c in ev]
        return None

    grid_reset = lambda: s.reset_tensors(dm, dt_, dg)  # noqa: E731
    grid_finish = lambda: s.step_tensors(0, img, err)  # noqa: E731

    device_steps(args.warmup, s, grid_reset, grid_finish, False)
    torch.cuda.synchronize()
    clocks = ClockSampler(local).start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    l0 = s.launches
    w0 = time.perf_counter()
    times = device_steps(args.steps, s, grid_reset, grid_finish, True)
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - w0
    launches = s.launches - l0
    clk = clocks.stop()

    step_ms = sum(a for a, _ in times)
    sweep_ms = sum(b for _, b in times)
    step_ms = job_time_max(step_ms, world, dev)
    value = whole_job_value(unknowns * sweeps, args.steps, world, step_ms)

    # Parity spot check of the timed path's output against a fresh solve.
    check = backend.GridSolver(8, 8)
    check.reset(crop_px, mc, t, g)
    ref_img, ref_err = check.step(sweeps)
    same = bool(np.array_equal(img.cpu().numpy(), ref_img))

    # End to end through the plugin API: pinned host inputs, H2D + D2H inside.
    pin_m = torch.from_numpy(mc).pin_memory()
    pin_t = torch.from_numpy(t).pin_memory()
    pin_g = torch.from_numpy(g).pin_memory()
    hm, ht, hg = pin_m.numpy(), pin_t.numpy(), pin_g.numpy()
    e2e_solver = backend.GridSolver(8, 8)
    for _ in range(max(1, min(args.warmup, 3))):
        e2e_solver.reset(crop_px, hm, ht, hg)
        e2e_solver.step(sweeps)
    e2e_steps = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_solver.reset(crop_px, hm, ht, hg)
        out_img, out_err = e2e_solver.step(sweeps)
    e2e_dt = (time.perf_counter() - t0) / e2e_steps
    barrier()

    # End to end from the uint8 images (GPU-side reset: threshold, crop,
    # gradient mixing on the device), pinned host images in, image out.
    pin_src = torch.from_numpy(pb.src).pin_memory().numpy()
    pin_msk = torch.from_numpy(pb.mask).pin_memory().numpy()
    pin_tgt = torch.from_numpy(pb.tgt).pin_memory().numpy()
    img_solver = backend.GridSolver(8, 8)
    for _ in range(max(1, min(args.warmup, 3))):
        img_solver.reset_images(pin_src, pin_msk, pin_tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
        img_solver.step(sweeps)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        img_solver.reset_images(pin_src, pin_msk, pin_tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
        out_img2, _ = img_solver.step(sweeps)
    e2e_img_dt = (time.perf_counter() - t0) / e2e_steps

    peak, peak_kind = measured_peak()
    kernel = s.kernel
    per_launch, launches_per_step, passes = kernel_shape(kernel, sweeps)
    avg_launch_s = sweep_ms / 1e3 / (args.steps * launches_per_step)
    # Algorithmic bytes of one launch: 37 B per crop pixel per sweep, times
    # the sweeps one launch performs (the temporally blocked kernels do
    # `depth` sweeps per launch on register-resident state; the flow and
    # resident kernels a whole step).
    alg_bytes = GRID_BYTES_PER_PX * crop_px * per_launch
    achieved = alg_bytes / avg_launch_s / 1e9
    # Compulsory: one read of x/grad/mask and one write of x per pass over
    # the regions (one per launch, or one per 16-sweep level of the flow
    # kernel).
    compulsory = GRID_BYTES_PER_PX * crop_px * passes / avg_launch_s / 1e9

    line = {
        "metric": "pixel-updates/s", "value": value, "unit": "pixel-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms / args.steps,
        "wall_ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "square800 GridSolver FP32 Jacobi, 5000 sweeps, 'max' gradient "
                               "(640,000 unknowns, 802x802 crop; 1024^2 target, 900^2 source)",
                   "unknowns": unknowns, "crop": [n, m], "sweeps": sweeps,
                   "step": "device reset from HBM-resident inputs + 5000 sweeps + residual + uint8 image",
                   "l2": "flushed between steps by a 512 MiB write outside the timed events",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "gpu_launches": launches,
        "e2e": {"value": unknowns * sweeps / e2e_dt, "unit": "pixel-updates/s",
                "h2d_bytes_per_step": int(mc.nbytes + t.nbytes + g.nbytes),
                "d2h_bytes_per_step": int(out_img.nbytes + out_err.nbytes),
                "api": "GridSolver.reset(pinned host arrays) + GridSolver.step(5000)",
                "ms_per_step": e2e_dt * 1e3},
        "e2e_from_images": {"value": unknowns * sweeps / e2e_img_dt, "unit": "pixel-updates/s",
                            "h2d_bytes_per_step": int(pb.src.nbytes + pb.mask.nbytes + pb.tgt.nbytes),
                            "d2h_bytes_per_step": int(out_img2.nbytes + 12),
                            "api": "GridSolver.reset_images(pinned uint8 src/mask/tgt) + "
                                   "GridSolver.step(5000)",
                            "ms_per_step": e2e_img_dt * 1e3},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": profiled_traffic(f"grid_{kernel}_square800"),
                     "kernel": kernel, "sweeps_per_launch": per_launch,
                     "region_passes_per_launch": passes, "bytes_per_launch": alg_bytes,
                     "avg_launch_us": avg_launch_s * 1e6, "peak_source": f"hbm_gbs ({peak_kind})",
                     "compulsory_gbs": compulsory, "compulsory_frac": compulsory / peak,
                     "note": "achieved counts 37 B/pixel for every sweep a launch performs; "
                             "compulsory counts one read of x/grad/mask and one write of x "
                             "per pass over the regions"},
        "clocks": clk,
        "parity": {"timed_output_equals_fresh_solve": same},
    }

    # The FP16 refinement form on the same workload (same step structure).
    m = backend.GridSolver(8, 8)
    m.set_stream(stream.cuda_stream)
    m.set_precision("fp16")
    m_reset = lambda: m.reset_tensors(dm, dt_, dg)  # noqa: E731
    m_finish = lambda: m.step_tensors(0, img, err)  # noqa: E731
    device_steps(args.warmup, m, m_reset, m_finish, False)
    msteps = max(3, args.steps // 4)
    mt = device_steps(msteps, m, m_reset, m_finish, True)
    m_ms = sum(a for a, _ in mt) / msteps
    line["mixed_fp16"] = {"value": unknowns * sweeps / (m_ms / 1e3), "unit": "pixel-updates/s",
                          "ms_per_step": m_ms, "steps": msteps, "kernel": m.kernel,
                          "note": "FP16 correction + FP32 residual every 64 sweeps; equals FP32 "
                                  "up to the correction's rounding (see the precision study)"}

    if not args.no_equ:
        from fpie_gb300 import backend as B

        q = B.EquSolver(256)
        q.set_stream(stream.cuda_stream)
        sysm = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                               q.partition)
        qa = torch.from_numpy(sysm.A).to(dev)
        qx = torch.from_numpy(sysm.X).to(dev)
        qb = torch.from_numpy(sysm.B).to(dev)
        qimg = torch.empty((sysm.N, 3), dtype=torch.uint8, device=dev)
        q_reset = lambda: q.reset_tensors(sysm.N, qa, qx, qb)  # noqa: E731
        q_finish = lambda: q.step_tensors(0, qimg, err)  # noqa: E731
        device_steps(args.warmup, q, q_reset, q_finish, False)
        qsteps = max(3, args.steps // 4)
        qt = device_steps(qsteps, q, q_reset, q_finish, True)
        q_ms = sum(a for a, _ in qt)
        q_sweep = sum(b for _, b in qt) / 1e3 / (qsteps * sweeps)
        line["equ"] = {"value": (sysm.N - 1) * sweeps * qsteps / (q_ms / 1e3), "unit": "pixel-updates/s",
                       "ms_per_step": q_ms / qsteps, "steps": qsteps, "kernel": q.kernel,
                       "sweep_kernel_achieved_gbs": EQU_BYTES_PER_UNKNOWN * sysm.N / q_sweep / 1e9,
                       "note": "reset_tensors (A/X/B from HBM; the placement on a grid is "
                               "re-checked on the device) + 5000 sweeps + residual + uint8 "
                               "values; 'grid:<k>' = the system is a 4-neighbour raster "
                               "stencil swept by grid kernel k"}

    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_grid(mc, t, g)
        if sweeps == SWEEPS:
            x64, secs = fp64_solution(mc, t, g)
            line["error_vs_fp64"] = error_vs_fp64(check.state(), x64, mc, secs)
            origin = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                      pb.gradient)[3]
            try:
                line["reference_cuda"] = reference_cuda(mc, t, g, sysm if not args.no_equ else None,
                                                        x64, (origin.x0, origin.y0))
            except Exception as exc:  # the comparison arm must not cost the bench line
                line["reference_cuda"] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_batch(args):
    """256 uneven paste jobs (boxes log-uniform 32..1024, 2000-10000 sweeps each):
    one persistent batched launch vs the same jobs run one at a time."""
    import torch

    from fpie_gb300 import backend, prep, workloads
    from fpie_gb300.batch import BatchSolver

    jobs = []
    for pb in workloads.job_mix(n_jobs=args.jobs, seed=7):
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        jobs.append((mc, t, g, pb.iterations))
    work = sum(int((mc != 0).sum()) * it for mc, t, g, it in jobs)
    crop_px = sum(mc.size for mc, *_ in jobs)
    b = BatchSolver(40e9, precision=args.precision)
    ids = [b.add(mc, t, g, it) for mc, t, g, it in jobs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b.run()
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t0
    launches = b.launches
    # The same jobs, one GridSolver each with the batch's kernel, back to back.
    def solo(mc, t, g):
        s = backend.GridSolver(8, 8)
        s.set_precision(args.precision)
        s.set_kernel(b.kernel)
        s.reset(mc.size, mc, t, g)
        return s

    t0 = time.perf_counter()
    for mc, t, g, it in jobs:
        s = solo(mc, t, g)
        s.sweeps(it)
        s.sync()
        s.close()
    seq_s = time.perf_counter() - t0
    # Spot parity: three jobs against a GridSolver run of the same kernel.
    # FP32 results are bit-identical whatever the kernel; the mixed forms
    # round the correction where the kernel's depth puts launch boundaries
    # (the tuner ran other depths for 64 sweeps each), so they are compared
    # within the mixed forms' tolerance (0.25 FP16, 2.0 BF16 intensity units).
    same, worst = True, 0.0
    tol = {"fp32": 0.0, "fp16": 0.25, "bf16": 2.0}[args.precision]
    for k in (0, len(jobs) // 2, len(jobs) - 1):
        mc, t, g, it = jobs[k]
        s = solo(mc, t, g)
        s.step(it)
        diff = float(np.abs(s.state() - b.state(ids[k])).max())
        worst = max(worst, diff)
        same &= diff <= tol
    line = {"metric": "pixel-updates/s", "value": work / batch_s, "unit": "pixel-updates/s",
            "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": batch_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"{len(jobs)} paste jobs, boxes log-uniform 32..1024, circles/"
                                   "squares/blobs, src|max gradient, 2000-10000 sweeps each",
                       "precision": args.precision,
                       "unknown_sweeps": work, "crop_pixels": crop_px,
                       "batch_kernel": b.kernel, "includes_autotuning": True},
            "sequential_gridsolver": {"value": work / seq_s, "seconds": seq_s},
            "batched_seconds": batch_s, "speedup_vs_sequential": seq_s / batch_s,
            "gpu_launches": launches, "parity_spot_check": same, "parity_max_abs_diff": worst}
    # Algorithmic bytes of the whole run: 37 B per crop pixel per sweep (FP32;
    # the mixed forms' inner sweeps move 25 B) over every job's sweeps.
    per_px = GRID_BYTES_PER_PX if args.precision == "fp32" else 25
    alg = sum(per_px * mc.size * it for mc, t, g, it in jobs)
    peak, peak_kind = measured_peak()
    line["roofline"] = {"bound": "hbm", "achieved": alg / batch_s / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": alg / batch_s / 1e9 / peak, "traffic": None,
                        "peak_source": peak_kind,
                        "note": f"{per_px} B per crop pixel per sweep over all jobs' sweeps, "
                                "divided by the batched wall time (autotuning included); above 1 "
                                "because each pass keeps a region in registers for 16 sweeps"}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Poisson arrivals of the batched-job distribution; each job stops at a
    max residual of 1e-3 per channel or 10000 sweeps; 40 GB HBM budget."""
    from fpie_gb300.serve import make_requests, run_workload

    out = {}
    for rate in [float(r) for r in args.rates.split(",")]:
        reqs = make_requests(args.jobs, seed=11)
        out[str(int(rate))] = run_workload(reqs, rate, seed=int(rate), budget_bytes=40e9,
                                           epoch_sweeps=256, tol=1e-3, max_sweeps=10000,
                                           precision=args.precision)
        print(json.dumps({"rate": rate, **out[str(int(rate))]}), flush=True)
    best = max(out.values(), key=lambda r: r["throughput_req_per_s"])
    line = {"metric": "p99 latency ms (and throughput)", "value": best["latency_ms"]["p99"],
            "unit": "ms", "higher_is_better": False, "n_gpus": 1, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"serving: {args.jobs} requests per rate, Poisson arrivals, "
                                   "stop at max|r| <= 1e-3 or 10000 sweeps, 40 GB budget, "
                                   "256-sweep epochs", "precision": args.precision},
            "rates": out}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
