#!/usr/bin/env python3
"""Precision study: sweeps and GPU time to reach <= 0.5 LSB of the FP64 solution.

For a circle paste (default: circle1800, 4096x4096 images, radius 1800,
about 10.2 M unknowns, 'max' gradient) this script

1. computes the converged FP64 solution with the oracle's matrix-free FP64
   conjugate gradient on the GPU (oracle/fp64.py, test infrastructure);
2. runs plain FP32 Jacobi and the mixed forms (FP16 / BF16 correction,
   FP32 residual every 64 sweeps) in chunks, recording after each chunk the
   max |x - x64| over masked pixels and the device time of the sweeps
   (CUDA events on the solver's stream);
3. reports, per form, the first checkpoint whose error is <= 0.5 and the
   sweeps and milliseconds it took, plus the per-sweep time.

It is a measurement script (run on a GPU), not a pytest module.
Usage: python tests/precision_study.py [--radius R] [--size S] [--chunk C] [--max-sweeps M]
"""

from __future__ import annotations

import argparse
import json
import pathlib
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--radius", type=float, default=1800)
    ap.add_argument("--chunk", type=int, default=262144)
    ap.add_argument("--max-sweeps", type=int, default=16_000_000)
    ap.add_argument("--forms", default="fp32,fp16,bf16")
    ap.add_argument("--target", type=float, default=0.5)
    args = ap.parse_args()

    import torch

    from fpie_gb300 import backend, prep, workloads
    from oracle import fp64

    if args.size == 4096 and args.radius == 1800:
        pb = workloads.circle1800()
    else:
        src = workloads.smooth_image(5, args.size, args.size, 16)
        tgt = workloads.smooth_image(6, args.size, args.size, 16)
        pb = workloads.Problem("circle", src, workloads.disk_mask(args.size, args.size, args.radius),
                               tgt, (0, 0), (0, 0), "max", 0)
    mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    on = mc != 0
    unknowns = int(on.sum())
    t0 = time.time()
    x64 = fp64.cg_torch(mc, t, g, device="cuda", rtol=1e-13)
    cg_s = time.time() - t0
    dev = torch.device("cuda", 0)
    x64_d = torch.from_numpy(x64).to(dev)
    on_d = torch.from_numpy(on).to(dev)
    print(json.dumps({"problem": pb.name, "crop": list(mc.shape), "unknowns": unknowns,
                      "fp64_cg_seconds": round(cg_s, 1)}), flush=True)

    results = {}
    stream = torch.cuda.current_stream()
    for form in args.forms.split(","):
        s = backend.GridSolver(8, 8)
        s.set_stream(stream.cuda_stream)
        s.set_precision(form)
        s.reset(mc.size, mc, t, g)
        s.step(4096)  # autotune on real sweeps
        done, dev_ms = 4096, 0.0
        curve = []
        hit = None
        while done < args.max_sweeps:
            k = min(args.chunk, args.max_sweeps - done)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.sweeps(k)
            e1.record(stream)
            torch.cuda.synchronize()
            dev_ms += e0.elapsed_time(e1)
            done += k
            x = torch.from_numpy(s.state()).to(dev)
            err = float((x - x64_d).abs()[on_d].max())
            mx, _ = s.residual_norms()
            curve.append({"sweeps": done, "max_err": err, "max_residual": float(mx.max())})
            print(json.dumps({"form": form, **curve[-1]}), flush=True)
            if err <= args.target:
                hit = done
                break
            # Stagnation: no 1% improvement over the last four checkpoints
            # (plain FP32 Jacobi stalls once a sweep's change rounds away).
            if len(curve) >= 5 and curve[-1]["max_err"] > 0.99 * curve[-5]["max_err"]:
                results.setdefault("_stalled", {})[form] = {"sweeps": done, "max_err": err}
                break
        per_sweep_ms = dev_ms / max(1, done - 4096)
        stalled = results.get("_stalled", {}).get(form)
        results[form] = {"kernel": s.kernel, "sweeps_to_target": hit,
                         "stalled_at": stalled,
                         "best_max_err": min(c["max_err"] for c in curve),
                         "ms_per_sweep": per_sweep_ms,
                         "ms_to_target": per_sweep_ms * hit if hit else None,
                         "px_updates_per_s": unknowns / (per_sweep_ms / 1e3),
                         "curve": curve}
        s.close()
    results.pop("_stalled", None)
    base = results.get("fp32", {}).get("ms_to_target")
    for form, r in results.items():
        if base and r["ms_to_target"]:
            r["speedup_vs_fp32"] = base / r["ms_to_target"]
    print(json.dumps({"summary": {f: {k: v for k, v in r.items() if k != "curve"}
                                  for f, r in results.items()}}), flush=True)


if __name__ == "__main__":
    main()
