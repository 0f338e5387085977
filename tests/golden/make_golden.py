#!/usr/bin/env python3
"""Generate golden vectors by running the reference fpie itself.

Needs the reference source tree ($FPIE_REFERENCE, by default the read-only
copy this script was written against, /root/reference) and, for the OpenMP vectors, its compiled modules from
oracle/build_ref.sh.  Writes tests/golden/*.npz; the tests only read those
files, so they run where the reference is absent.

Each file holds a paste problem (src, mask, tgt, offsets, gradient), the
solver inputs the reference processors built from it, and the reference
solvers' outputs after the listed sweep counts: uint8 image (the crop of the
target the solver updates, rows x0:x1 and columns y0:y1) and float32 err
from ``step``, plus the unclipped float32 state of the numpy solver after the
last count.

Usage: python tests/golden/make_golden.py
"""

from __future__ import annotations

import os
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle.ref_import import import_reference  # noqa: E402


def _workloads():
    import fpie_gb300.workloads as W

    return W


def run_case(P, name, src, mask, tgt, mos, mot, gradient, checkpoints, omp=False, omp_grid=(1, 1)):
    out = {"src": src, "mask": mask, "tgt": tgt, "mask_on_src": np.array(mos), "mask_on_tgt": np.array(mot),
           "gradient": np.array(gradient), "checkpoints": np.array(checkpoints)}
    g = P.GridProcessor(gradient=gradient, backend="numpy")
    n = g.reset(src, mask, tgt.copy(), mos, mot)
    out["grid_n"] = np.array(n)
    out["grid_mask"] = g.core.mask.astype(np.int32)
    out["grid_tgt"] = g.core.tgt.copy()
    out["grid_grad"] = g.core.grad.copy()
    out["grid_box"] = np.array([g.x0, g.x1, g.y0, g.y1])
    e = P.EquProcessor(gradient=gradient, backend="numpy")
    N = e.reset(src, mask, tgt.copy(), mos, mot)
    out["equ_N"] = np.array(N)
    out["equ_A"] = e.core.A.astype(np.int32)
    out["equ_X"] = e.core.X.copy()
    out["equ_B"] = e.core.B.copy()
    out["equ_tgt_index"] = np.stack(e.tgt_index)
    mc = out["grid_mask"]
    ids = e.core.partition(mc)
    ids[mc == 0] = 0
    out["equ_ids"] = ids.astype(np.int32)
    go = eo = None
    if omp and "openmp" in P.ALL_BACKEND:
        go = P.GridProcessor(gradient=gradient, backend="openmp", n_cpu=4, grid_x=omp_grid[0], grid_y=omp_grid[1])
        go.reset(src, mask, tgt.copy(), mos, mot)
        # The OpenMP EquSolver: red-black Gauss-Seidel on odd-then-even ids.
        eo = P.EquProcessor(gradient=gradient, backend="openmp", n_cpu=4)
        eo.reset(src, mask, tgt.copy(), mos, mot)
        rb = np.asarray(eo.core.partition(mc)).astype(np.int32)  # same mask: same n_mid
        rb[mc == 0] = 0
        out["omp_equ_ids"] = rb
    # Images are stored as the solver-updated crop of the target only.
    x0, x1, y0, y1 = g.x0, g.x1, g.y0, g.y1
    done = 0
    for k in checkpoints:
        img, err = g.step(k - done)
        out[f"grid_img_{k}"] = img[x0:x1, y0:y1].copy()
        out[f"grid_err_{k}"] = np.asarray(err, np.float32)
        if k == checkpoints[-1]:
            out[f"grid_state_{k}"] = g.core.tgt.copy()
        img, err = e.step(k - done)
        out[f"equ_img_{k}"] = img[x0:x1, y0:y1].copy()
        out[f"equ_err_{k}"] = np.asarray(err, np.float32)
        if k == checkpoints[-1]:
            out[f"equ_state_{k}"] = e.core.X.copy()
        if go is not None:
            img, err = go.step(k - done)
            out[f"omp_img_{k}"] = img[x0:x1, y0:y1].copy()
            out[f"omp_err_{k}"] = np.asarray(err, np.float32)
            img, err = eo.step(k - done)
            out[f"omp_equ_img_{k}"] = img[x0:x1, y0:y1].copy()
            out[f"omp_equ_err_{k}"] = np.asarray(err, np.float32)
        done = k
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: grid crop {mc.shape}, N={N}, checkpoints {checkpoints}")


def main() -> None:
    P = import_reference(os.environ.get("FPIE_REFERENCE", "/root/reference"))
    if P is None:
        sys.exit("reference tree not found; set FPIE_REFERENCE")
    W = _workloads()

    # 1. The reference smoke test's 6x6 problem (tests/test_smoke.py:19-24).
    src = np.zeros((6, 6, 3), np.uint8)
    mask = np.zeros((6, 6), np.uint8)
    mask[2:4, 2:4] = 255
    tgt = np.ones((6, 6, 3), np.uint8) * 10
    run_case(P, "smoke6", src, mask, tgt, (0, 0), (0, 0), "max", [2, 5])

    # 2. The reference's OpenMP-vs-numpy pin (tests/test_smoke.py:48-66).
    rng = np.random.default_rng(0)
    src = rng.integers(0, 256, size=(24, 24, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(24, 24, 3), dtype=np.uint8)
    mask = np.zeros((24, 24), dtype=np.uint8)
    mask[2:-2, 2:-2] = (rng.random((20, 20)) > 0.35).astype(np.uint8) * 255
    run_case(P, "rand24", src, mask, tgt, (0, 0), (0, 0), "max", [5, 50], omp=True)

    # 3. circle256 workload (256x256, radius-96 circle, 'src'), to 5000 sweeps.
    pb = W.circle256()
    run_case(P, "circle256", pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
             [1, 100, 5000], omp=True, omp_grid=(8, 8))

    # 4. 'avg' gradient, offsets, 3-channel mask with values at the threshold.
    rng = np.random.default_rng(1)
    src = rng.integers(0, 256, size=(50, 47, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(44, 52, 3), dtype=np.uint8)
    mask3 = np.zeros((36, 33, 3), np.uint8)
    mask3[3:30, 4:28] = 255
    mask3[10:14, 6:9] = (128, 128, 127)   # sum 383: off
    mask3[15:19, 10:13] = (128, 128, 128)  # sum 384: on
    mask3[20:22, 2:4] = 255
    run_case(P, "avg_offsets", src, mask3, tgt, (5, 7), (4, 9), "avg", [3, 40], omp=True)

    # 5. 'src' gradient with a random blob mask reaching the frame.
    rng = np.random.default_rng(2)
    src = rng.integers(0, 256, size=(40, 40, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(40, 40, 3), dtype=np.uint8)
    mask = (rng.random((40, 40)) > 0.3).astype(np.uint8) * 255
    run_case(P, "blob_frame", src, mask, tgt, (0, 0), (0, 0), "src", [7, 70], omp=True)

    # 6. Solver level, mask set on the crop border: neighbours outside the
    #    grid contribute nothing (numpy semantics of np_solver.GridSolver).
    from fpie import np_solver

    rng = np.random.default_rng(3)
    m = (rng.random((11, 13)) > 0.4).astype(np.int32)
    t = rng.uniform(0, 255, size=(11, 13, 3)).astype(np.float32)
    gr = rng.uniform(-40, 40, size=(11, 13, 3)).astype(np.float32)
    gr[m == 0] = 0
    s = np_solver.GridSolver()
    s.reset(m.size, m, t.copy(), gr)
    out = {"mask": m, "tgt": t, "grad": gr}
    for k in (1, 6, 30):
        img, err = s.step(1 if k == 1 else (5 if k == 6 else 24))
        out[f"img_{k}"] = np.clip(img, 0, 255).astype(np.uint8)
        out[f"err_{k}"] = np.asarray(err, np.float32)
        out[f"state_{k}"] = s.tgt.copy()
    np.savez_compressed(HERE / "grid_border.npz", **out)
    print("grid_border: solver-level grid with border pixels set")


if __name__ == "__main__":
    main()
