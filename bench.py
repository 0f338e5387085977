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
WORKLOAD = ("square800 GridSolver FP32 Jacobi, 5000 sweeps, 'max' gradient "
            "(640,000 unknowns, 802x802 crop; 1024^2 target, 900^2 source)")


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
    p.add_argument("--workload", choices=["square800", "batch", "serve", "precision", "large",
                                          "steps"],
                   default="square800",
                   help="square800 (default, the headline line, which also carries the precision, "
                        "batch, serving and large-grid legs); batch: 256 uneven jobs in one "
                        "persistent launch vs one GridSolver per job; serve: Poisson arrivals; "
                        "precision: FP32 vs the mixed forms to <= 0.5 LSB on --problem; "
                        "large: the circle1800 FP32 leg alone; steps: --steps timed steps of "
                        "--sweeps sweeps of --problem (--kernel, --precision)")
    p.add_argument("--problem", default="circle450", help="precision workload: circle450 or circle1800")
    p.add_argument("--forms", default="fp32,fp16,bf16")
    p.add_argument("--chunk", type=int, default=4096, help="precision checkpoint spacing (sweeps)")
    p.add_argument("--max-sweeps", type=int, default=2_000_000)
    p.add_argument("--no-extras", action="store_true",
                   help="headline line only: skip the precision, batch, serving and large-grid legs")
    p.add_argument("--jobs", type=int, default=256, help="batch: jobs; serve: requests per rate")
    p.add_argument("--rates", default="50,500,2000")
    p.add_argument("--epoch", type=int, default=256, help="serve: sweeps per epoch")
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
    grid sweep kernel, from its name: "sweep1"; "p<R>w<W>k<K>[t]" (K sweeps
    per launch); "p16w8k16d" / "p16w8k12d" (and their "dp" forms) /
    "rb16w8k8d" (dependency flow: the whole step in one launch, a pass per
    level)."""
    if kernel == "sweep1":
        return 1, sweeps, 1
    depth = int(re.search(r"k(\d+)", kernel).group(1))
    if re.search(r"k\d+dp?$", kernel):
        return sweeps, 1, -(-sweeps // depth)
    return depth, -(-sweeps // depth), 1


FP32_OPS_PER_UPDATE = 15  # per pixel update: 4 additions + 1 multiplication, 3 channels


def apron_factor(kernel: str) -> float:
    """Region pixels a temporally blocked kernel sweeps per tile pixel it
    writes: regions are W*R rows x 128 columns, tiles lose K pixels (2K for
    red-black levels) on every side; 1 for the one-sweep kernel."""
    m = re.match(r"(rb|p)(\d+)w(\d+)k(\d+)", kernel)
    if not m:
        return 1.0
    r, w, k = (int(v) for v in m.groups()[1:])
    k = 2 * k if m.group(1) == "rb" else k
    rows = r * w
    return rows * 128 / ((rows - 2 * k) * (128 - 2 * k))


def fp32_peaks(stream_handle: int) -> dict:
    """Measured FP32 rates of this GPU (operations per second, one per
    value), from the library's probe kernel timed with CUDA events."""
    from fpie_gb300 import _abi

    return {k: _abi.fp32_rate(k, stream=stream_handle) for k in ("fadd2", "ffma2", "fadd")}


def grid_roofline(kernel: str, crop_px: int, unknowns: int, sweeps: int, avg_launch_s: float,
                  peaks: dict, traffic) -> dict:
    """Roofline object of a grid sweep kernel.  The bound is FP32 issue: the
    useful work of a launch is 15 FP32 operations per pixel update (masked
    pixels only), divided by the launch's average duration, against the
    measured packed-add rate.  The 37 B/pixel HBM figures are kept beside it
    as `hbm_effective` (algorithmic bytes of every sweep, above the copy
    bandwidth when sweeps stay in registers) and `hbm_compulsory` (one read
    of x/grad/mask and one write of x per pass over the regions)."""
    per_launch, _, passes = kernel_shape(kernel, sweeps)
    hbm, hbm_kind = measured_peak()
    ops = FP32_OPS_PER_UPDATE * unknowns * per_launch
    achieved = ops / avg_launch_s
    peak = peaks["fadd2"]
    af = apron_factor(kernel)
    alg_bytes = GRID_BYTES_PER_PX * crop_px * per_launch
    eff = alg_bytes / avg_launch_s / 1e9
    comp = GRID_BYTES_PER_PX * crop_px * passes / avg_launch_s / 1e9
    return {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "kernel": kernel,
            "sweeps_per_launch": per_launch, "ops_per_launch": ops,
            "ops_per_pixel_update": FP32_OPS_PER_UPDATE, "avg_launch_us": avg_launch_s * 1e6,
            "peak_source": "packed FP32 add rate measured in this run (fpie_probe_fp32_rate, "
                           "one operation per value)",
            "fp32_rates_tops": {k: v / 1e12 for k, v in peaks.items()},
            "apron_factor": af,
            "issued_frac": achieved * af * crop_px / unknowns / peak,
            "hbm_effective": {"achieved_gbs": eff, "peak_gbs": hbm, "frac": eff / hbm,
                              "peak_source": f"hbm_gbs ({hbm_kind})",
                              "bytes_per_launch": alg_bytes,
                              "note": "37 B per crop pixel for every sweep a launch performs; "
                                      "an effective figure, not a bound: the state stays in "
                                      "registers for K sweeps"},
            "hbm_compulsory": {"achieved_gbs": comp, "frac": comp / hbm,
                               "region_passes_per_launch": passes},
            "note": "useful FP32 operations (masked pixels, 15 per update) per second of the "
                    "sweep kernel; issued_frac adds the apron and the unmasked pixels of active "
                    "tiles that the kernel also computes"}


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


PRECISION_TARGET = 0.5  # max |x - x_fp64| over the unknowns, intensity units (LSB)


def precision_run(form: str, mc, t, g, x64, chunk: int, max_sweeps: int, stream,
                  target: float = PRECISION_TARGET, stall_checkpoints: int = 16) -> dict:
    """One form (fp32 / fp16 / bf16) from the initial state, in chunks of
    `chunk` sweeps: after each chunk the max error against the converged
    FP64 solution over the unknowns.  Device time counts the sweeps only
    (CUDA events on the solver's stream around each chunk); the error checks
    run between the events.  Stops at `target`, at `max_sweeps`, or -- plain
    FP32 Jacobi -- when the error has not improved for `stall_checkpoints`
    checkpoints (a sweep's change then rounds away at every pixel)."""
    import torch

    from fpie_gb300 import backend

    on = np.asarray(mc) != 0
    ref = x64[on]
    # Tuning happens on a throwaway solver of the same shape (the choice is
    # cached per shape), so that the measured run starts from the initial
    # state and its first chunk holds no tuning sweeps.
    w = backend.GridSolver(8, 8)
    w.set_stream(stream.cuda_stream)
    w.set_precision(form)
    w.reset(mc.size, mc, t, g)
    w.step(65536)
    w.close()
    s = backend.GridSolver(8, 8)
    s.set_stream(stream.cuda_stream)
    s.set_precision(form)
    s.reset(mc.size, mc, t, g)
    done, dev_ms, curve, hit, stalled = 0, 0.0, [], None, None
    best, best_at = float("inf"), 0
    while done < max_sweeps:
        k = min(chunk, max_sweeps - done)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.sweeps(k)
        e1.record(stream)
        e1.synchronize()
        dev_ms += e0.elapsed_time(e1)
        done += k
        err = float(np.abs(s.state()[on].astype(np.float64) - ref).max())
        curve.append((done, round(dev_ms, 3), err))
        if err < best:
            best, best_at = err, len(curve)
        if err <= target:
            hit = (done, dev_ms)
            break
        if len(curve) - best_at >= stall_checkpoints:
            stalled = done
            break
    out = {"kernel": s.kernel, "us_per_sweep": dev_ms * 1e3 / done, "sweeps_run": done,
           "sweeps_to_target": hit[0] if hit else None,
           "ms_to_target": hit[1] if hit else None,
           "best_max_err": best, "stalled_at_sweeps": stalled, "curve": curve}
    s.close()
    return out


def first_reaching(curve, level: float):
    """(sweeps, device ms) of the first checkpoint with error <= level."""
    for sw, ms, err in curve:
        if err <= level:
            return sw, ms
    return None, None


def precision_study(pb, forms=("fp32", "fp16", "bf16"), chunk: int = 4096,
                    max_sweeps: int = 2_000_000) -> dict:
    """Plain FP32 Jacobi against the mixed forms (FP16 / BF16 correction,
    FP32 residual every 64 sweeps) on one paste problem: sweeps and device
    time to <= 0.5 LSB of the converged FP64 solution, FP32's error floor
    and each form's time to that floor, and the cost per sweep."""
    import torch

    from fpie_gb300 import prep
    from oracle import fp64

    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                   pb.gradient)
    t0 = time.perf_counter()
    x64 = fp64.cg_torch(mc, t, g, device="cuda", rtol=1e-13)
    cg_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    runs = {f: precision_run(f, mc, t, g, x64, chunk, max_sweeps, stream) for f in forms}
    out = {"workload": f"{pb.name}: {pb.src.shape[0]}x{pb.src.shape[1]} images, crop "
                       f"{mc.shape[0]}x{mc.shape[1]}, {int((mc != 0).sum())} unknowns, "
                       f"'{pb.gradient}' gradient",
           "target_max_err": PRECISION_TARGET, "checkpoint_sweeps": chunk,
           "reference": f"FP64 conjugate gradient on the GPU (oracle), rtol 1e-13, {cg_s:.1f} s",
           "forms": {}}
    floor = runs["fp32"]["best_max_err"] if "fp32" in runs else None
    if floor is not None:
        out["fp32_floor"] = floor
    fl_sw, fl_ms = first_reaching(runs["fp32"]["curve"], floor) if floor is not None else (None, None)
    for f, r in runs.items():
        d = {k: v for k, v in r.items() if k != "curve"}
        if floor is not None:
            sw, ms = first_reaching(r["curve"], floor)
            d["sweeps_to_fp32_floor"], d["ms_to_fp32_floor"] = sw, ms
            if f != "fp32" and ms and fl_ms:
                d["speedup_to_fp32_floor"] = fl_ms / ms
        if f != "fp32" and "fp32" in runs:
            d["fp32_reaches_target"] = runs["fp32"]["sweeps_to_target"] is not None
        # Every 8th checkpoint and the last: (sweeps, device ms, max error).
        d["curve"] = r["curve"][7::8] + ([r["curve"][-1]] if len(r["curve"]) % 8 else [])
        out["forms"][f] = d
    return out


def run_precision(args):
    """--workload precision: the precision comparison on --problem."""
    import torch

    from fpie_gb300 import workloads

    torch.cuda.set_device(0)
    pb = workloads.WORKLOADS[args.problem]()
    res = precision_study(pb, forms=tuple(args.forms.split(",")), chunk=args.chunk,
                          max_sweeps=args.max_sweeps)
    print(json.dumps({"metric": "device ms to <= 0.5 LSB of the FP64 solution", **res}), flush=True)


def cpu_equ_baselines(sysm, rsys, n_mid: int, budget_s: float = 8.0) -> dict:
    """The oracle's C restatements of the reference's EquSolver iterations on
    the square800 system, all host threads, each on a bounded number of
    sweeps: the numpy EquSolver's Jacobi (fpie/np_solver.py:31-54) and the
    OpenMP EquSolver's red-black order (fpie/core/openmp/equ.cc:107-125)."""
    from oracle import cjacobi

    th = host_threads()
    out = {}
    for name, make in (("jacobi", lambda: cjacobi.CEqu(sysm.A, sysm.X, sysm.B, nthreads=th)),
                       ("red_black", lambda: cjacobi.CEquRedBlack(rsys.A, rsys.X, rsys.B, n_mid,
                                                                  nthreads=th))):
        o = make()
        o.sweep(3)
        t0 = time.perf_counter()
        o.sweep(20)
        per = (time.perf_counter() - t0) / 20
        n_sw = int(max(20, min(SWEEPS, budget_s / 2 / max(per, 1e-9))))
        o = make()
        t0 = time.perf_counter()
        o.sweep(n_sw)
        o.err64()
        o.image()
        dt = time.perf_counter() - t0
        out[name] = {"value": (sysm.N - 1) * n_sw / dt, "unit": "pixel-updates/s", "cores": th,
                     "kind": "port", "sample": f"{n_sw} of {SWEEPS} sweeps + residual + clip, "
                                               f"{th} threads, {dt:.2f} s"}
    return out


def config0_leg(stream) -> dict:
    """The reference's CPU-runnable case (circle256: 256x256 images, circle of
    radius 96, 'src' gradient, 5000 sweeps): the GB300 GridSolver through its
    public API (reset from host arrays + step(5000), wall time, median of 5)
    beside the numpy GridSolver's iteration (the oracle's numpy restatement
    of fpie/np_solver.py:79-101, one core) on a bounded number of sweeps."""
    from fpie_gb300 import backend, prep, workloads
    from oracle import np_jacobi

    pb = workloads.circle256()
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                   pb.gradient)
    unknowns = int((mc != 0).sum())
    s = backend.GridSolver(8, 8)
    s.set_stream(stream.cuda_stream)
    for _ in range(2):
        s.reset(mc.size, mc, t, g)
        s.step(SWEEPS)
    ts = []
    for _ in range(5):
        t0 = time.perf_counter()
        s.reset(mc.size, mc, t, g)
        img, _ = s.step(SWEEPS)
        ts.append(time.perf_counter() - t0)
    gpu_s = statistics.median(ts)
    o = np_jacobi.GridJacobi(mc, t, g)
    o.sweep(5)
    t0 = time.perf_counter()
    o.sweep(20)
    per = (time.perf_counter() - t0) / 20
    n_sw = int(max(20, min(SWEEPS, 4.0 / max(per, 1e-9))))
    o = np_jacobi.GridJacobi(mc, t, g)
    t0 = time.perf_counter()
    o.sweep(n_sw)
    o.err64()
    o.image()
    cpu_s = time.perf_counter() - t0
    kernel = s.kernel
    s.close()
    return {"workload": f"circle256 GridSolver FP32 Jacobi, 5000 sweeps, 'src' gradient "
                        f"({unknowns} unknowns, {mc.shape[0]}x{mc.shape[1]} crop)",
            "gpu": {"value": unknowns * SWEEPS / gpu_s, "unit": "pixel-updates/s",
                    "ms_per_step": gpu_s * 1e3, "kernel": kernel,
                    "api": "GridSolver.reset(host arrays) + step(5000), wall time"},
            "cpu_baseline": {"value": unknowns * n_sw / cpu_s, "unit": "pixel-updates/s",
                             "cores": 1, "kind": "port",
                             "sample": f"{n_sw} of {SWEEPS} sweeps + residual + clip, numpy "
                                       f"restatement of the reference's numpy GridSolver, "
                                       f"{cpu_s:.2f} s"}}


def large_grid_leg(stream, steps: int = 3, kernel: str = "auto") -> dict:
    """FP32 Jacobi on circle1800 (4096x4096 images, radius 1800, 10.2 M
    unknowns): a working set of ~480 MB, well above the 129 MB L2, so HBM
    figures mean something here.  Device-timed steps of 5000 sweeps (reset
    from HBM-resident inputs + sweeps + residual + image), same structure as
    the headline step."""
    import torch

    from fpie_gb300 import backend, prep, workloads

    pb = workloads.circle1800()
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                   pb.gradient)
    unknowns, crop_px = int((mc != 0).sum()), int(mc.size)
    dev = torch.device("cuda", torch.cuda.current_device())
    dm, dt_, dg = (torch.from_numpy(a).to(dev) for a in (mc, t, g))
    img = torch.empty((*mc.shape, 3), dtype=torch.uint8, device=dev)
    err = torch.empty(3, dtype=torch.float32, device=dev)
    s = backend.GridSolver(8, 8)
    s.set_stream(stream.cuda_stream)
    if kernel != "auto":
        s.set_kernel(kernel)
    s.reset_tensors(dm, dt_, dg)
    s.sweeps(SWEEPS)  # tuning on real sweeps
    s.step_tensors(0, img, err)
    torch.cuda.synchronize()
    l0 = s.launches
    ev = []
    for _ in range(steps):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        s.reset_tensors(dm, dt_, dg)
        s.sweeps(SWEEPS)
        e1.record(stream)
        s.step_tensors(0, img, err)
        e2.record(stream)
        ev.append((e0, e1, e2))
    torch.cuda.synchronize()
    step_ms = statistics.median(a.elapsed_time(c) for a, _, c in ev)
    sweep_ms = sum(a.elapsed_time(b) for a, b, _ in ev) / steps
    kernel = s.kernel
    _, launches_per_step, _ = kernel_shape(kernel, SWEEPS)
    avg_launch_s = sweep_ms / 1e3 / launches_per_step
    out = {"workload": f"circle1800 GridSolver FP32 Jacobi, 5000 sweeps, 'max' gradient "
                       f"({unknowns} unknowns, {mc.shape[0]}x{mc.shape[1]} crop)",
           "value": unknowns * SWEEPS / (step_ms / 1e3), "unit": "pixel-updates/s",
           "ms_per_step": step_ms, "us_per_sweep": sweep_ms * 1e3 / SWEEPS, "steps": steps,
           "kernel": kernel, "gpu_launches": (s.launches - l0) // steps,
           "l2": "not flushed: the ~480 MB working set is larger than L2",
           "roofline": grid_roofline(kernel, crop_px, unknowns, SWEEPS, avg_launch_s,
                                     fp32_peaks(stream.cuda_stream),
                                     profiled_traffic(f"grid_{kernel}_circle1800"))}
    s.close()
    return out


def _leg(line: dict, key: str, fn) -> None:
    """Runs one extra leg into line[key]; a failure is recorded there and
    does not cost the headline line."""
    t0 = time.perf_counter()
    try:
        line[key] = fn()
    except Exception as exc:
        line[key] = {"unavailable": f"{type(exc).__name__}: {exc}"}
    if isinstance(line[key], dict):
        line[key]["leg_seconds"] = round(time.perf_counter() - t0, 1)


def extra_legs(line: dict, args, pb, stream, sysm) -> None:
    """The legs beside the headline number (rank 0, one GPU): the CPU rows of
    the EquSolver forms and of the CPU-runnable circle256 case, the FP32
    sweep on a grid larger than L2, the precision comparison, the batched
    form and the serving form."""
    from fpie_gb300 import backend, prep, workloads

    if sysm is not None and "equ" in line and not args.no_cpu_baseline:
        def equ_cpu():
            rb = backend.EquSolver(1024, order="red_black")
            rsys = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                   pb.gradient, rb.partition)
            return cpu_equ_baselines(sysm, rsys, rb.n_mid)
        _leg(line["equ"], "cpu_baseline", equ_cpu)
    if not args.no_cpu_baseline:
        _leg(line, "config0", lambda: config0_leg(stream))
    _leg(line, "large_grid", lambda: large_grid_leg(stream))
    _leg(line, "precision", lambda: precision_study(workloads.circle450()))
    mix = workloads.job_mix(n_jobs=256, seed=7)
    _leg(line, "batch", lambda: {f: batch_study(batch_jobs(mix=mix), f, sequential=True)
                                 for f in ("fp32", "fp16")})
    _leg(line, "serve", lambda: serve_study(mix))


def serve_study(mix, n_requests: int = 1000, rates=(50.0, 500.0, 2000.0),
                forms=("fp32", "fp16"), epoch: int = 256) -> dict:
    """Poisson arrivals of paste requests drawn (seeded, with replacement)
    from the 256-job mix, images in: each request's inputs are built on the
    GPU at admission, inside its latency.  Each request stops at a max
    residual of 1e-3 per channel or 10000 sweeps; 40 GB HBM budget;
    `epoch`-sweep epochs (the stop rule is checked after each)."""
    from fpie_gb300.serve import Request, run_workload

    rng = np.random.default_rng(11)
    draws = rng.integers(0, len(mix), size=n_requests)
    out = {"workload": f"{n_requests} requests per rate drawn from the 256-job mix (boxes "
                       "log-uniform 32..1024, circles/squares/blobs, src|max gradient), images "
                       "in; stop at max|r| <= 1e-3 per channel or 10000 sweeps; 40 GB budget; "
                       f"{epoch}-sweep epochs; Poisson arrivals",
           "latency": "arrival to result on the host, input construction included"}
    for form in forms:
        for rate in rates:
            reqs = [Request(k, problem=mix[int(d)]) for k, d in enumerate(draws)]
            r = run_workload(reqs, rate, seed=int(rate), budget_bytes=40e9, epoch_sweeps=epoch,
                             tol=1e-3, max_sweeps=10000, precision=form)
            out[f"{form}@{int(rate)}"] = r
    return out


def run_steps(args):
    """--workload steps: `--steps` device-timed steps of `--sweeps` sweeps of
    --problem with a pinned or tuned --kernel and --precision (a small,
    fixed sequence of launches for profiling and for comparing kernels)."""
    import torch

    from fpie_gb300 import backend, prep, workloads

    torch.cuda.set_device(0)
    stream = torch.cuda.current_stream()
    pb = workloads.WORKLOADS[args.problem]()
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                   pb.gradient)
    s = backend.GridSolver(8, 8)
    s.set_stream(stream.cuda_stream)
    s.set_precision(args.precision)
    if args.kernel != "auto":
        s.set_kernel(args.kernel)
    s.reset(mc.size, mc, t, g)
    for _ in range(args.warmup):
        s.sweeps(args.sweeps)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.sweeps(args.sweeps)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    unknowns = int((mc != 0).sum())
    med = statistics.median(ms)
    print(json.dumps({"workload": f"{pb.name} ({unknowns} unknowns, crop {mc.shape[0]}x{mc.shape[1]})",
                      "precision": args.precision, "kernel": s.kernel, "sweeps": args.sweeps,
                      "steps": args.steps, "ms_median": med, "us_per_sweep": med * 1e3 / args.sweeps,
                      "pixel_updates_per_s": unknowns * args.sweeps / (med / 1e3)}), flush=True)


def run_large(args):
    """--workload large: the FP32 leg on circle1800 alone."""
    import torch

    torch.cuda.set_device(0)
    print(json.dumps(large_grid_leg(torch.cuda.current_stream(), steps=args.steps,
                                    kernel=args.kernel)), flush=True)


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
        "config": {"workload": WORKLOAD, "sweeps_per_step": n_sw, "sweeps_of_full_step": args.sweeps},
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

    kernel = s.kernel
    per_launch, launches_per_step, passes = kernel_shape(kernel, sweeps)
    avg_launch_s = sweep_ms / 1e3 / (args.steps * launches_per_step)
    peaks = fp32_peaks(stream.cuda_stream)

    line = {
        "metric": "pixel-updates/s", "value": value, "unit": "pixel-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms / args.steps,
        "wall_ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD,
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
        "roofline": grid_roofline(kernel, crop_px, unknowns, sweeps, avg_launch_s, peaks,
                                  profiled_traffic(f"grid_{kernel}_square800")),
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
    if rank == 0 and world == 1 and not args.no_extras and sweeps == SWEEPS:
        extra_legs(line, args, pb, stream, sysm if not args.no_equ else None)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def batch_jobs(n_jobs: int = 256, seed: int = 7, mix=None):
    """The batched-jobs mix (workloads.job_mix, or `mix`) as solver inputs
    built on the host: [(mask, tgt, grad, sweeps)]."""
    from fpie_gb300 import prep, workloads

    jobs = []
    for pb in mix if mix is not None else workloads.job_mix(n_jobs=n_jobs, seed=seed):
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        jobs.append((mc, t, g, pb.iterations))
    return jobs


def batch_study(jobs, precision: str = "fp32", sequential: bool = True) -> dict:
    """All jobs in one persistent launch (BatchSolver.run to completion) vs
    one GridSolver per job back to back.  The autotuner (64 real sweeps of
    every job per candidate) runs on a first batch of the same jobs and is
    timed on its own; the timed batch is pinned to the tuned kernel."""
    import torch

    from fpie_gb300 import backend
    from fpie_gb300.batch import BatchSolver

    work = sum(int((mc != 0).sum()) * it for mc, t, g, it in jobs)
    crop_px = sum(mc.size for mc, *_ in jobs)
    tune = BatchSolver(40e9, precision=precision)
    for mc, t, g, it in jobs:
        tune.add(mc, t, g, it)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tune.run(256)  # 3 candidates x 64 sweeps + 64 more
    torch.cuda.synchronize()
    tune_s = time.perf_counter() - t0
    kernel = tune.kernel
    tune.close()
    b = BatchSolver(40e9, precision=precision)
    b.set_kernel(kernel)
    ids = [b.add(mc, t, g, it) for mc, t, g, it in jobs]
    torch.cuda.synchronize()
    l0 = b.launches
    t0 = time.perf_counter()
    b.run()
    torch.cuda.synchronize()
    batch_s = time.perf_counter() - t0
    launches = b.launches - l0
    out = {"workload": f"{len(jobs)} paste jobs, boxes log-uniform 32..1024, circles/squares/"
                       "blobs, src|max gradient, 2000-10000 sweeps each",
           "precision": precision, "value": work / batch_s, "unit": "pixel-updates/s",
           "seconds": batch_s, "unknown_sweeps": work, "crop_pixels": crop_px,
           "kernel": kernel, "gpu_launches": launches,
           "autotune_seconds": tune_s, "includes_autotuning": False}
    per_px = GRID_BYTES_PER_PX if precision == "fp32" else 25
    alg = sum(per_px * mc.size * it for mc, t, g, it in jobs)
    out["hbm_effective_gbs"] = alg / batch_s / 1e9
    if sequential:
        t0 = time.perf_counter()
        for mc, t, g, it in jobs:
            s = backend.GridSolver(8, 8)
            s.set_precision(precision)
            s.set_kernel(kernel)
            s.reset(mc.size, mc, t, g)
            s.sweeps(it)
            s.sync()
            s.close()
        seq_s = time.perf_counter() - t0
        out["sequential_gridsolver"] = {"value": work / seq_s, "seconds": seq_s,
                                        "note": "one GridSolver per job with the batch's kernel, "
                                                "reset from host arrays + sweeps, back to back"}
        out["speedup_vs_sequential"] = seq_s / batch_s
    # Spot parity against a GridSolver of the same kernel (the full parity
    # check against the oracle is in the tests): FP32 bit for bit; the mixed
    # forms round the correction where the kernel puts launch boundaries,
    # so within their tolerance (0.25 FP16, 2.0 BF16 intensity units).
    tol = {"fp32": 0.0, "fp16": 0.25, "bf16": 2.0}[precision]
    worst = 0.0
    for k in (0, len(jobs) // 2, len(jobs) - 1):
        mc, t, g, it = jobs[k]
        s = backend.GridSolver(8, 8)
        s.set_precision(precision)
        s.set_kernel(kernel)
        s.reset(mc.size, mc, t, g)
        s.step(it)
        worst = max(worst, float(np.abs(s.state() - b.state(ids[k])).max()))
        s.close()
    out["parity_spot_check"] = worst <= tol
    out["parity_max_abs_diff"] = worst
    b.close()
    return out


def run_batch(args):
    """--workload batch: the batched form alone, as its own JSON line."""
    import torch

    torch.cuda.set_device(0)
    r = batch_study(batch_jobs(args.jobs), args.precision)
    peak, peak_kind = measured_peak()
    line = {"metric": "pixel-updates/s", "value": r["value"], "unit": "pixel-updates/s",
            "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": r["seconds"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": r["workload"], "precision": args.precision},
            "gpu_launches": r["gpu_launches"], "batch": r,
            "roofline": {"bound": "hbm", "achieved": r["hbm_effective_gbs"], "peak": peak,
                         "unit": "GB/s", "frac": r["hbm_effective_gbs"] / peak, "traffic": None,
                         "peak_source": peak_kind,
                         "note": "effective: 37 B (FP32) / 25 B (mixed) per crop pixel per sweep "
                                 "over all jobs' sweeps, divided by the batched wall time"}}
    print(json.dumps(line), flush=True)


def run_serve(args):
    """--workload serve: the serving form alone, one JSON line per rate and a
    summary line."""
    import torch

    from fpie_gb300 import workloads

    torch.cuda.set_device(0)
    mix = workloads.job_mix(n_jobs=256, seed=7)
    rates = tuple(float(r) for r in args.rates.split(","))
    res = serve_study(mix, n_requests=args.jobs, rates=rates, forms=(args.precision,),
                      epoch=args.epoch)
    best = max((v for k, v in res.items() if isinstance(v, dict)),
               key=lambda r: r["throughput_req_per_s"])
    line = {"metric": "p99 latency ms (and throughput)", "value": best["latency_ms"]["p99"],
            "unit": "ms", "higher_is_better": False, "n_gpus": 1, "dtype": "f32",
            "data": "synthetic", "config": {"workload": res["workload"], "precision": args.precision},
            "serve": res}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "precision":
        run_precision(args)
    elif args.workload == "large":
        run_large(args)
    elif args.workload == "steps":
        run_steps(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
