"""GridSolver on the GPU against the oracle, through the C ABI.

Tolerances: FP32 states are compared bit for bit (the kernels keep the numpy
backend's order of additions); uint8 images exactly; the per-channel error
(a sum over unknowns, reduced in double on the GPU) within rtol 1e-5 of the
oracle's float64 sum.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden
from oracle import cjacobi, np_jacobi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    from fpie_gb300 import backend as b

    return b


def test_golden_cases(backend, golden):
    name, d = golden
    s = backend.GridSolver(8, 8)
    s.reset(int(d["grid_n"]), d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    done = 0
    cps = [int(k) for k in d["checkpoints"]]
    for k in cps:
        img, err = s.step(k - done)
        done = k
        assert img.dtype == np.uint8 and img.shape == d["grid_mask"].shape + (3,)
        assert err.dtype == np.float32 and err.shape == (3,)
        np.testing.assert_array_equal(img, d[f"grid_img_{k}"])
        np.testing.assert_allclose(err, d[f"grid_err_{k}"], rtol=1e-4, atol=1e-3)
    np.testing.assert_array_equal(s.state(), d[f"grid_state_{cps[-1]}"])
    o = np_jacobi.GridJacobi(d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    o.x = d[f"grid_state_{cps[-1]}"].copy()
    np.testing.assert_allclose(err, o.err64(), rtol=1e-5, atol=1e-3)


def test_border_pixels(backend):
    d = load_golden("grid_border")
    s = backend.GridSolver(1, 1)
    s.reset(d["mask"].size, d["mask"], d["tgt"], d["grad"])
    done = 0
    for k in (1, 6, 30):
        img, err = s.step(k - done)
        done = k
        np.testing.assert_array_equal(s.state(), d[f"state_{k}"])
        np.testing.assert_array_equal(img, d[f"img_{k}"])
        np.testing.assert_allclose(err, d[f"err_{k}"], rtol=1e-5, atol=1e-3)


def _square800_grid():
    from fpie_gb300 import prep, workloads

    pb = workloads.square800()
    return prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)


def test_square800_5000_sweeps_bit_exact(backend):
    """640k unknowns, 5000 sweeps: state identical to the C oracle's."""
    mc, t, g, _ = _square800_grid()
    s = backend.GridSolver(8, 8)
    s.reset(mc.size, mc, t, g)
    img, err = s.step(5000)
    o = cjacobi.CGrid(mc, t, g)
    o.sweep(5000)
    np.testing.assert_array_equal(s.state(), o.x)
    np.testing.assert_array_equal(img, o.image())
    np.testing.assert_allclose(err, o.err64(), rtol=1e-5)


def test_flow_depths_square800_bit_exact(backend):
    """The depth-12 flow kernel (104x104 tiles: 8 x 8 of them cover the
    802-pixel grid, where 96x96 tiles need 9 x 9) after 5000 sweeps, then
    both depths alternating on one solver (each switch rebuilds the tile
    tables): states identical to the C oracle's."""
    mc, t, g, _ = _square800_grid()
    s = backend.GridSolver(8, 8)
    s.set_kernel("p16w8k12d")
    s.reset(mc.size, mc, t, g)
    img, err = s.step(5000)
    o = cjacobi.CGrid(mc, t, g)
    o.sweep(5000)
    np.testing.assert_array_equal(s.state(), o.x)
    np.testing.assert_array_equal(img, o.image())
    np.testing.assert_allclose(err, o.err64(), rtol=1e-5)
    for kernel, k in (("p16w8k16d", 37), ("p16w8k12dp", 50), ("p16w8k16dp", 21),
                      ("p16w8k12d", 13)):
        s.set_kernel(kernel)
        s.step(k)
        o.sweep(k)
        assert s.kernel == kernel
        np.testing.assert_array_equal(s.state(), o.x)


@pytest.mark.parametrize("kernel", ["p16w8k16dp", "p16w8k12dp"])
@pytest.mark.parametrize("shift", [0, 1, 2, 3])
def test_flow_pinned_boundary_bodies(backend, kernel, shift):
    """Regions holding unmasked pixels sweep with selects only at pinned
    pixels (unmasked, next to a masked one) and leave the other unmasked
    pixels unstored.  Rectangles shifted by 0..3 columns put their vertical
    edges in every column group of the lanes (single-group bodies), their
    horizontal edges make row-selected bodies, a disk the select-everywhere
    body, and a band on the grid's first columns pins the zero padding next
    to masked pixels: states and images identical to the C oracle's."""
    rng = np.random.default_rng(40 + shift)
    n, m = 300, 430
    mask = np.zeros((n, m), np.int32)
    mask[20:280, 10 + shift:400 + shift] = 1
    mask[0:n, 0:3 + shift] = 1                      # masked pixels on the grid edge
    yy, xx = np.mgrid[0:n, 0:m]
    mask[(yy - 150) ** 2 + (xx - 415) ** 2 < 12 ** 2] = 1
    tgt = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    grad = rng.uniform(-30, 30, (n, m, 3)).astype(np.float32)
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.reset(n * m, mask, tgt, grad)
    o = cjacobi.CGrid(mask, tgt, grad)
    for k in (7, 45):
        img, err = s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.x)
        np.testing.assert_array_equal(img, o.image())
        np.testing.assert_allclose(err, o.err64(), rtol=1e-5)


def test_flow_depth12_is_fp32_only(backend):
    """The depth-12 and pinned-boundary flow kernels run FP32 sweeps only:
    the mixed forms (whose refinement cycles are 64 sweeps of 16-sweep
    levels) refuse them by name."""
    from fpie_gb300 import _abi

    d = load_golden("rand24")
    s = backend.GridSolver(8, 8)
    s.set_precision("fp16")
    s.reset(int(d["grid_n"]), d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    for name in ("p16w8k12d", "p16w8k12dp", "p16w8k16dp"):
        with pytest.raises(_abi.FpieArgumentError):
            s.set_kernel(name)


def test_step_continues_and_reset_restarts(backend):
    d = load_golden("rand24")
    args = (int(d["grid_n"]), d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    a = backend.GridSolver(8, 8)
    a.reset(*args)
    for k in (1, 2, 0, 64, 3, 130):   # mixes graph chunks and single sweeps
        a.step(k)
    b = backend.GridSolver(8, 8)
    b.reset(*args)
    b.step(200)
    np.testing.assert_array_equal(a.state(), b.state())
    a.reset(*args)  # a second reset starts over from the new inputs
    a.step(50)
    np.testing.assert_array_equal(a.state(), d["grid_state_50"])
    img, err = a.step(-3)  # a negative count runs no sweep, like the reference
    np.testing.assert_array_equal(a.state(), d["grid_state_50"])


def test_before_reset_and_bad_args(backend):
    s = backend.GridSolver(8, 8)
    img, err = s.step(10)
    assert img.shape == (0, 0, 3) and np.all(err == 0)
    from fpie_gb300 import _abi

    with pytest.raises(_abi.FpieArgumentError):
        s.reset(4, np.ones((2, 2), np.int32), np.zeros((2, 3, 3), np.float32), np.zeros((2, 2, 3), np.float32))
    with pytest.raises(_abi.FpieArgumentError):
        s.reset(0, np.ones((0, 5), np.int32), np.zeros((0, 5, 3), np.float32), np.zeros((0, 5, 3), np.float32))


def test_tensor_handoff(backend):
    torch = pytest.importorskip("torch")
    d = load_golden("circle256")
    s = backend.GridSolver(8, 8)
    s.set_stream(torch.cuda.current_stream().cuda_stream)
    dev = torch.device("cuda", 0)
    m = torch.from_numpy(d["grid_mask"]).to(dev)
    t = torch.from_numpy(d["grid_tgt"]).to(dev)
    g = torch.from_numpy(d["grid_grad"]).to(dev)
    s.reset_tensors(m, t, g)
    img = torch.empty(d["grid_mask"].shape + (3,), dtype=torch.uint8, device=dev)
    err = torch.empty(3, dtype=torch.float32, device=dev)
    s.step_tensors(100, img, err)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(img.cpu().numpy(), d["grid_img_100"])
    np.testing.assert_allclose(err.cpu().numpy(), d["grid_err_100"], rtol=1e-4, atol=1e-3)
    assert s.launches >= 4  # pack, sweeps, residual/image, finalize


KERNELS = ["sweep1", "p16w8k8", "p16w8k16", "p8w16k16", "p8w8k8", "p16w8k16t", "p16w8k16d",
           "p16w8k12d", "p16w8k16dp", "p16w8k12dp"]


@pytest.mark.parametrize("kernel", KERNELS)
def test_every_kernel_is_bit_exact(backend, kernel):
    """Each sweep kernel, pinned, reproduces the reference's numpy states."""
    d = load_golden("circle256")
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.reset(int(d["grid_n"]), d["grid_mask"], d["grid_tgt"], d["grid_grad"])
    assert s.kernel == kernel
    done = 0
    for k in (1, 100, 5000):  # 1, 99 and 4900 sweeps: partial blocks and chunks
        img, err = s.step(k - done)
        done = k
        np.testing.assert_array_equal(img, d[f"grid_img_{k}"])
        np.testing.assert_allclose(err, d[f"grid_err_{k}"], rtol=1e-4, atol=1e-3)
    np.testing.assert_array_equal(s.state(), d["grid_state_5000"])


@pytest.mark.parametrize("kernel", KERNELS)
def test_sparse_tiles(backend, kernel):
    """A mostly empty grid: tiles without masked pixels are skipped."""
    rng = np.random.default_rng(11)
    n, m = 301, 517
    mask = np.zeros((n, m), np.int32)
    mask[5:40, 7:33] = 1          # top-left corner
    mask[200:290, 400:505] = 1    # bottom-right region
    mask[150, 260] = 1            # a single pixel
    mask[n - 1, 100:120] = 1      # on the last row (neighbours outside read 0)
    tgt = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    grad = rng.uniform(-30, 30, (n, m, 3)).astype(np.float32)
    grad[mask == 0] = 0
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.reset(n * m, mask, tgt, grad)
    o = np_jacobi.GridJacobi(mask, tgt, grad)
    for k in (3, 77, 130):
        img, err = s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.x)
        np.testing.assert_array_equal(img, o.image())
        np.testing.assert_allclose(err, o.err64(), rtol=1e-5)


def test_autotuner_choice_is_reported(backend):
    mc, t, g, _ = _square800_grid()
    s = backend.GridSolver(8, 8)
    s.reset(mc.size, mc, t, g)
    s.step(2000)
    assert s.kernel in KERNELS
    o = cjacobi.CGrid(mc, t, g)
    o.sweep(2000)
    np.testing.assert_array_equal(s.state(), o.x)


def _many_items_case():
    """1500x1700 grid: 288 tiles x 3 channels = 864 (tile, channel) items, so
    every persistent CTA of the TMA kernel sweeps several, prefetching each
    next region during the current one's sweeps.  Empty top rows (inactive
    tiles, skipped), a solid right half (fully masked tiles) and a holed left
    half (tiles with unmasked pixels)."""
    rng = np.random.default_rng(5)
    n, m = 1500, 1700
    mask = np.zeros((n, m), np.int32)
    mask[200:1450, 60:1650] = 1
    holes = rng.random((n, m)) < 0.03
    holes[:, 850:] = False
    mask[holes] = 0
    tgt = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    grad = rng.uniform(-30, 30, (n, m, 3)).astype(np.float32)
    grad[mask == 0] = 0
    return mask, tgt, grad


@pytest.mark.parametrize("kernel", ["p16w8k16t", "p16w8k16d", "p16w8k12d", "p16w8k12dp"])
def test_persistent_kernels_many_items_per_cta(backend, kernel):
    """The persistent kernels (TMA prefetch; dependency flow, whose CTAs run
    ahead into the next level where neighbourhoods are ready) on a grid with
    several items per CTA, against the oracle."""
    mask, tgt, grad = _many_items_case()
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.reset(mask.size, mask, tgt, grad)
    o = cjacobi.CGrid(mask, tgt, grad)
    for k in (1, 15, 130):  # a 1-sweep launch, a partial block, graph chunks
        img, err = s.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(s.state(), o.x)
    np.testing.assert_array_equal(img, o.image())


def test_tma_wait_times_out_without_hanging(backend):
    """A spin limit of 0 makes a region-copy wait give up: the step returns a
    timeout error (after the CTA's copies in flight have landed) instead of
    hanging, and the solver and GPU stay usable."""
    from fpie_gb300 import _abi

    mc, t, g, _ = _square800_grid()
    s = backend.GridSolver(8, 8)
    s.set_kernel("p16w8k16t")
    s.set_spin_limit(0)
    s.reset(mc.size, mc, t, g)
    with pytest.raises(_abi.FpieTimeoutError):
        s.step(64)
    s.set_spin_limit(1 << 26)
    s.reset(mc.size, mc, t, g)
    s.step(100)
    o = cjacobi.CGrid(mc, t, g)
    o.sweep(100)
    np.testing.assert_array_equal(s.state(), o.x)


@pytest.mark.parametrize("kernel", ["p16w8k16d", "p16w8k12d"])
def test_flow_wait_times_out_without_hanging(backend, kernel):
    """Spin limit 0: a neighbourhood wait of the dependency-flow kernel gives
    up at its first unmet check; the launch stops, the next synchronising
    call raises the timeout, and the solver and GPU stay usable."""
    from fpie_gb300 import _abi

    mc, t, g, _ = _square800_grid()
    s = backend.GridSolver(8, 8)
    s.set_kernel(kernel)
    s.set_spin_limit(0)
    s.reset(mc.size, mc, t, g)
    with pytest.raises(_abi.FpieTimeoutError):
        s.step(5000)
    s.set_spin_limit(1 << 26)
    s.reset(mc.size, mc, t, g)
    s.step(100)
    o = cjacobi.CGrid(mc, t, g)
    o.sweep(100)
    np.testing.assert_array_equal(s.state(), o.x)
