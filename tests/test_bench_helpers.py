"""Host logic of bench.py's comparison legs (no GPU): the error statistics,
the placement of an equation state on the crop grid, and the search for
the first sweep count that reaches a target."""

from __future__ import annotations

import pathlib
import sys

import numpy as np

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent.parent))
import bench  # noqa: E402


def test_err_stats_counts_masked_pixels_only():
    mc = np.array([[0, 1], [1, 0]], np.int32)
    x = np.zeros((2, 2, 3), np.float32)
    x64 = np.zeros((2, 2, 3))
    x[0, 1] = 2.0
    x[1, 0] = -1.0
    x[0, 0] = 100.0  # unmasked: ignored
    s = bench.err_stats(x, x64, mc)
    assert s["max_abs"] == 2.0
    assert s["mean_abs"] == 1.5


def test_equ_on_grid_places_rows_by_target_index():
    class Sys:
        tgt_index = (np.array([5, 6]), np.array([7, 9]))

    X = np.array([[0, 0, 0], [1, 2, 3], [4, 5, 6]], np.float32)  # row 0: the constant
    g = bench.equ_on_grid(X, Sys, (5, 7), (3, 4, 3))
    np.testing.assert_array_equal(g[0, 0], [1, 2, 3])
    np.testing.assert_array_equal(g[1, 2], [4, 5, 6])
    assert g.sum() == 21


def test_first_reaching_steps_until_the_target():
    state = {"n": 0}

    def reset():
        state["n"] = 0

    def step(k):
        state["n"] += k

    def value():  # falls by 1 per sweep from 1000
        return 1000.0 - state["n"]

    n, v = bench._first_reaching(reset, step, value, 640.0, 100, 50, 10_000)
    assert n == 400 and v == 600.0  # 100, 150, ... the first multiple reaching <= 640
    n, v = bench._first_reaching(reset, step, value, -1e9, 100, 50, 300)
    assert n == 300  # capped


def test_median_step_time_resets_before_each_step():
    calls = []
    s = bench._median_step_s(lambda: calls.append("r"), lambda k: calls.append(k), 7, reps=3)
    assert calls == ["r", 7, "r", 7, "r", 7] and s >= 0.0


def test_kernel_shape_and_apron_of_every_grid_kernel_name():
    """Sweeps per launch, launches per step and region passes per launch,
    and the apron factor, from the kernel names the solver reports."""
    assert bench.kernel_shape("sweep1", 5000) == (1, 5000, 1)
    assert bench.kernel_shape("p16w8k16", 5000) == (16, 313, 1)
    for name, depth in (("p16w8k16d", 16), ("p16w8k12d", 12), ("p16w8k16dp", 16),
                        ("p16w8k12dp", 12), ("rb16w8k8d", 8)):
        assert bench.kernel_shape(name, 5000) == (5000, 1, -(-5000 // depth)), name
    assert abs(bench.apron_factor("p16w8k16d") - 128 * 128 / (96 * 96)) < 1e-12
    assert abs(bench.apron_factor("p16w8k12dp") - 128 * 128 / (104 * 104)) < 1e-12
    assert abs(bench.apron_factor("rb16w8k8d") - 128 * 128 / (96 * 96)) < 1e-12
    assert bench.apron_factor("sweep1") == 1.0
