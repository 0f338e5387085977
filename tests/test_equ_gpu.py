"""EquSolver on the GPU against the oracle, through the C ABI.

States bit for bit (numpy order B + X[A0] + X[A1] + X[A2] + X[A3]); uint8
images exactly; err within rtol 1e-5 of the oracle's float64 sum.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden, problem_args
from oracle import cjacobi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from fpie_gb300 import backend as b

    return b


def test_partition_matches_reference(backend, golden):
    name, d = golden
    s = backend.EquSolver(256)
    mc = d["grid_mask"]
    ids = s.partition(mc)
    assert ids.dtype == np.int32 and ids.shape == mc.shape
    np.testing.assert_array_equal(np.where(mc > 0, ids, 0), d["equ_ids"])
    np.testing.assert_array_equal(ids[mc > 0], np.cumsum((mc > 0).reshape(-1)).reshape(mc.shape)[mc > 0])


def test_golden_cases(backend, golden):
    name, d = golden
    s = backend.EquSolver(1024)
    N = int(d["equ_N"])
    s.reset(N, d["equ_A"], d["equ_X"], d["equ_B"])
    idx = d["equ_tgt_index"]
    x0, y0 = int(d["grid_box"][0]), int(d["grid_box"][2])
    done = 0
    cps = [int(k) for k in d["checkpoints"]]
    for k in cps:
        x, err = s.step(k - done)
        done = k
        assert x.dtype == np.uint8 and x.shape == (N, 3)
        np.testing.assert_array_equal(x[1:], d[f"equ_img_{k}"][idx[0] - x0, idx[1] - y0])
        np.testing.assert_allclose(err, d[f"equ_err_{k}"], rtol=1e-4, atol=1e-3)
    np.testing.assert_array_equal(s.state(), d[f"equ_state_{cps[-1]}"])


def test_square800_5000_sweeps_bit_exact(backend):
    from fpie_gb300 import prep, workloads

    pb = workloads.square800()
    s = backend.EquSolver(256)
    sysm = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient, s.partition)
    s.reset(sysm.N, sysm.A, sysm.X, sysm.B)
    x, err = s.step(5000)
    o = cjacobi.CEqu(sysm.A, sysm.X, sysm.B)
    o.sweep(5000)
    np.testing.assert_array_equal(s.state(), o.X)
    np.testing.assert_array_equal(x, o.image())
    np.testing.assert_allclose(err, o.err64(), rtol=1e-5)


def test_out_of_range_neighbour_is_rejected(backend):
    from fpie_gb300 import _abi

    d = load_golden("smoke6")
    A = d["equ_A"].copy()
    A[2, 1] = int(d["equ_N"])  # one past the end
    s = backend.EquSolver(256)
    with pytest.raises(_abi.FpieArgumentError):
        s.reset(int(d["equ_N"]), A, d["equ_X"], d["equ_B"])
    A[2, 1] = -1
    with pytest.raises(_abi.FpieArgumentError):
        s.reset(int(d["equ_N"]), A, d["equ_X"], d["equ_B"])
    x, err = s.step(3)  # the rejected reset left no state: empty result
    assert x.shape == (0, 3)


def test_continuation(backend):
    d = load_golden("blob_frame")
    args = (int(d["equ_N"]), d["equ_A"], d["equ_X"], d["equ_B"])
    a, b = backend.EquSolver(128), backend.EquSolver(1024)
    a.reset(*args)
    b.reset(*args)
    for k in (3, 64, 1, 2):
        a.step(k)
    b.step(70)
    np.testing.assert_array_equal(a.state(), b.state())
    np.testing.assert_array_equal(a.state(), d["equ_state_70"])


def _two_disks_system():
    n0, m0 = 300, 420
    mask = np.zeros((n0, m0), np.uint8)
    yy, xx = np.mgrid[:n0, :m0]
    mask[(yy - 90) ** 2 + (xx - 100) ** 2 < 70 ** 2] = 255
    mask[(yy - 200) ** 2 + (xx - 300) ** 2 < 90 ** 2] = 255
    mask[250:260, 20:60] = 255
    from fpie_gb300 import workloads
    from oracle import prep

    src = workloads.smooth_image(8, n0, m0, 8)
    tgt = workloads.smooth_image(9, n0, m0, 8)
    return prep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), "max")


def _same_as_gather(backend, N, A, X, B):
    """A raster system swept by the grid kernels ("auto") and by the gather
    kernel: identical states, images and err at every checkpoint."""
    g = backend.EquSolver(256)
    g.reset(N, A, X, B)
    assert g.kernel.startswith("grid:")
    q = backend.EquSolver(256)
    q.set_kernel("gather")
    q.reset(N, A, X, B)
    assert q.kernel == "gather"
    for k in (1, 16, 33, 200):
        xg, eg = g.step(k)
        xq, eq = q.step(k)
        np.testing.assert_array_equal(xg, xq)
        np.testing.assert_array_equal(eg, eq)
        np.testing.assert_array_equal(g.state(), q.state())


def test_grid_placement_equals_gather_golden(backend, golden):
    _, d = golden
    _same_as_gather(backend, int(d["equ_N"]), d["equ_A"], d["equ_X"], d["equ_B"])


def test_grid_placement_equals_gather_components(backend):
    d = _two_disks_system()
    _same_as_gather(backend, d["N"], d["A"], d["X"], d["B"])


@pytest.mark.parametrize("kernel", ["p16w8k16", "p16w8k16d", "p16w8k12d", "p16w8k12dp", "sweep1"])
def test_grid_placement_pinned_kernels(backend, kernel):
    d = _two_disks_system()
    s = backend.EquSolver(256)
    s.set_kernel(kernel)
    s.reset(d["N"], d["A"], d["X"], d["B"])
    assert s.kernel == "grid:" + kernel
    s.step(150)
    o = cjacobi.CEqu(d["A"], d["X"], d["B"])
    o.sweep(150)
    np.testing.assert_array_equal(s.state(), o.X)


def test_grid_placement_refuses_non_raster(backend):
    from fpie_gb300 import _abi

    rng = np.random.default_rng(3)
    N = 64
    A = rng.integers(0, N, (N, 4)).astype(np.int32)
    A[0] = 0
    X = rng.uniform(0, 255, (N, 3)).astype(np.float32)
    X[0] = 0
    B = rng.uniform(-20, 20, (N, 3)).astype(np.float32)
    B[0] = 0
    s = backend.EquSolver(256)
    s.reset(N, A, X, B)                 # auto: the gather kernel
    assert s.kernel == "gather"
    p = backend.EquSolver(256)
    p.set_kernel("p16w8k16")
    with pytest.raises(_abi.FpieArgumentError):
        p.reset(N, A, X, B)


def test_grid_placement_from_images(backend):
    """The GPU-side reset places the mask's unknowns directly (no search)."""
    from fpie_gb300 import workloads

    pb = workloads.circle256()
    s = backend.EquSolver(256)
    N, box, idx = s.reset_images(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    assert s.kernel.startswith("grid:")
    A, B = s.inputs()
    X0 = s.state()
    q = backend.EquSolver(256)
    q.set_kernel("gather")
    q.reset(N, A, X0, B)
    xs, es = s.step(300)
    xq, eq = q.step(300)
    np.testing.assert_array_equal(xs, xq)
    np.testing.assert_array_equal(s.state(), q.state())


def test_placed_reset_equals_the_searched_placement(backend, golden):
    """reset with the processor's placement (checked on the device) runs the
    same grid sweeps as reset without it (placement searched on the host)."""
    from fpie_gb300 import prep as pprep

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    a = backend.EquSolver(1024)
    sysm = pprep.equ_inputs(src, mask, tgt, mos, mot, grad, a.partition)
    a.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=sysm.placement())
    b = backend.EquSolver(1024)
    b.reset(sysm.N, sysm.A, sysm.X, sysm.B)
    assert a.kernel.startswith("grid:") and a.kernel == b.kernel
    for k in (5, 70):
        xa, ea = a.step(k)
        xb, eb = b.step(k)
        np.testing.assert_array_equal(a.state(), b.state())
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(ea, eb)


def test_wrong_placement_is_refused(backend):
    from fpie_gb300 import prep as pprep

    d = load_golden("circle256")
    src, mask, tgt, mos, mot, grad = problem_args(d)
    s = backend.EquSolver(1024)
    sysm = pprep.equ_inputs(src, mask, tgt, mos, mot, grad, s.partition)
    pos, n, m = sysm.placement()
    bad = pos.copy()
    bad[1], bad[2] = pos[2], pos[1]  # two unknowns swapped
    with pytest.raises(ValueError):
        s.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=(bad, n, m))
    edge = pos.copy()
    edge[1] = 0  # on the crop's frame
    with pytest.raises(ValueError):
        s.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=(edge, n, m))
    s.reset(sysm.N, sysm.A, sysm.X, sysm.B, placement=(pos, n, m))  # and the right one works
    assert s.kernel.startswith("grid:")
