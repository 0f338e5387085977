"""The oracle (numpy and C restatements) against the reference's own vectors."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, problem_args
from oracle import cjacobi, np_jacobi, prep


def test_prep_matches_reference(golden):
    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    mc, t, g, box = prep.grid_inputs(src, mask, tgt, mos, mot, grad)
    np.testing.assert_array_equal(mc, d["grid_mask"])
    np.testing.assert_array_equal(t, d["grid_tgt"])
    np.testing.assert_array_equal(g, d["grid_grad"])
    assert box == tuple(int(v) for v in d["grid_box"])
    e = prep.equ_inputs(src, mask, tgt, mos, mot, grad)
    assert e["N"] == int(d["equ_N"])
    np.testing.assert_array_equal(e["A"], d["equ_A"])
    np.testing.assert_array_equal(e["X"], d["equ_X"])
    np.testing.assert_array_equal(e["B"], d["equ_B"])
    np.testing.assert_array_equal(e["ids"], d["equ_ids"])
    np.testing.assert_array_equal(np.stack(e["tgt_index"]), d["equ_tgt_index"])


def _crop(img_full, d):
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    return img_full[x0:x1, y0:y1]


@pytest.mark.parametrize("impl", ["numpy", "c"])
def test_grid_jacobi_matches_reference(golden, impl):
    name, d = golden
    cls = np_jacobi.GridJacobi if impl == "numpy" else cjacobi.CGrid
    o = cls(d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    done = 0
    cps = [int(k) for k in d["checkpoints"]]
    for k in cps:
        o.sweep(k - done)
        done = k
        # uint8 image of the reference processor (crop of the updated target)
        np.testing.assert_array_equal(o.image(), d[f"grid_img_{k}"])
        np.testing.assert_allclose(o.err64(), d[f"grid_err_{k}"], rtol=1e-5, atol=1e-3)
        if impl == "numpy":
            np.testing.assert_array_equal(o.err32(), d[f"grid_err_{k}"])
    np.testing.assert_array_equal(o.x, d[f"grid_state_{cps[-1]}"])


@pytest.mark.parametrize("impl", ["numpy", "c"])
def test_equ_jacobi_matches_reference(golden, impl):
    name, d = golden
    cls = np_jacobi.EquJacobi if impl == "numpy" else cjacobi.CEqu
    o = cls(d["equ_A"], d["equ_X"], d["equ_B"])
    done = 0
    cps = [int(k) for k in d["checkpoints"]]
    idx = d["equ_tgt_index"]
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    for k in cps:
        o.sweep(k - done)
        done = k
        img = o.image()
        ref = d[f"equ_img_{k}"]
        np.testing.assert_array_equal(img[1:], ref[idx[0] - x0, idx[1] - y0])
        np.testing.assert_allclose(o.err64(), d[f"equ_err_{k}"], rtol=1e-5, atol=1e-3)
        if impl == "numpy":
            np.testing.assert_array_equal(o.err32(), d[f"equ_err_{k}"])
    state = o.X
    np.testing.assert_array_equal(state, d[f"equ_state_{cps[-1]}"])


OMP_EQU_CASES = ["rand24", "circle256", "avg_offsets", "blob_frame"]


@pytest.mark.parametrize("name", OMP_EQU_CASES)
@pytest.mark.parametrize("impl", ["numpy", "c"])
def test_red_black_matches_reference_openmp(name, impl):
    """The red-black restatement against the reference's compiled OpenMP
    EquSolver: its odd-then-even ids exactly, its uint8 images exactly at
    every checkpoint, its float32 err within rtol 1e-5 (it sums in float32
    sequentially; the oracle's sum is float64)."""
    d = load_golden(name)
    src, mask, tgt, mos, mot, grad = problem_args(d)
    e = prep.equ_inputs(src, mask, tgt, mos, mot, grad, order="red_black")
    np.testing.assert_array_equal(e["ids"], d["omp_equ_ids"])
    cls = np_jacobi.EquRedBlack if impl == "numpy" else cjacobi.CEquRedBlack
    o = cls(e["A"], e["X"], e["B"], e["n_mid"])
    idx = e["tgt_index"]
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    done = 0
    for k in (int(v) for v in d["checkpoints"]):
        o.sweep(k - done)
        done = k
        ref = d[f"omp_equ_img_{k}"]
        np.testing.assert_array_equal(o.image()[1:], ref[idx[0] - x0, idx[1] - y0])
        np.testing.assert_allclose(o.err64(), d[f"omp_equ_err_{k}"], rtol=1e-5, atol=1e-2)


def test_red_black_numpy_equals_c_and_differs_from_jacobi():
    d = load_golden("circle256")
    e = prep.equ_inputs(*problem_args(d), order="red_black")
    a = np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    b = cjacobi.CEquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    j = np_jacobi.EquJacobi(e["A"], e["X"], e["B"])
    for o in (a, b, j):
        o.sweep(40)
    np.testing.assert_array_equal(a.X, b.X)
    assert a.err64().sum() < j.err64().sum()


def test_red_black_rejects_same_colour_neighbours():
    d = load_golden("rand24")
    e = prep.equ_inputs(*problem_args(d), order="red_black")
    with pytest.raises(AssertionError):
        np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"] + 1)


def test_grid_border_semantics():
    """Set pixels on the grid border: outside neighbours contribute nothing."""
    d = load_golden("grid_border")
    for impl in (np_jacobi.GridJacobi, cjacobi.CGrid):
        o = impl(d["mask"], d["tgt"], d["grad"])
        done = 0
        for k in (1, 6, 30):
            o.sweep(k - done)
            done = k
            np.testing.assert_array_equal(o.x, d[f"state_{k}"])
            np.testing.assert_array_equal(o.image(), d[f"img_{k}"])
            np.testing.assert_allclose(o.err64(), d[f"err_{k}"], rtol=1e-5, atol=1e-3)


def test_reference_openmp_within_one_lsb():
    """The reference's OpenMP grid solver adds in another order: <=1 LSB."""
    d = load_golden("circle256")
    for k in (1, 100, 5000):
        diff = np.abs(d[f"omp_img_{k}"].astype(int) - d[f"grid_img_{k}"].astype(int))
        assert diff.max() <= 1
        np.testing.assert_allclose(d[f"omp_err_{k}"], d[f"grid_err_{k}"], rtol=1e-3)


def test_oracle_catches_a_planted_error():
    """A one-ulp change in one grad value must change the oracle's state."""
    d = load_golden("rand24")
    g = d["grid_grad"].copy()
    on = np.argwhere(d["grid_mask"] != 0)[0]
    g[on[0], on[1], 0] = np.nextafter(g[on[0], on[1], 0], np.float32(1e9))
    a = cjacobi.CGrid(d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    b = cjacobi.CGrid(d["grid_mask"], d["grid_tgt"], g)
    a.sweep(5)
    b.sweep(5)
    assert not np.array_equal(a.x, b.x)


def test_reference_cuda_harness_builds():
    """The host side of the reference's CUDA solvers (oracle/ref_cuda_host.c)
    compiles and exports its entry points; running it needs a GPU."""
    import shutil
    import subprocess

    from oracle import ref_cuda

    if not (ref_cuda.cuda_home() / "include" / "cuda.h").is_file() or shutil.which("nm") is None:
        pytest.skip("no CUDA headers or nm")
    so = ref_cuda.build()
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True,
                         check=True).stdout
    for sym in ("refcuda_load", "refcuda_grid_sweeps", "refcuda_grid_step", "refcuda_equ_sweeps",
                "refcuda_equ_step"):
        assert sym in out, sym
