"""The allocation-free grid step against the solver object, on the GPU.

``fpie_grid_step_noalloc`` serves callers that cannot allocate device memory
where they need a step (hosts whose device memory belongs to their own pool
allocator, latency-critical loops where cudaMalloc may synchronize the
device): they pass every buffer, and the step's own scratch is a fixed array
inside the library.  This test calls it through the C ABI twice in a row on
the same state and checks each result against ``GridSolver`` (the existing
entry point) after the same total sweeps: state and uint8 image bit for bit,
err within rtol 1e-5 (another fixed summation order in double).  A grid of
exactly the size limit, with masked pixels on its border, fills the whole
scratch array.

The file name sorts last so that a run stopping at the first failure has
already run every other test.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _noalloc_step(lib, torch, mask_t, x_t, grad_t, iteration):
    n, m = mask_t.shape
    img = torch.empty((n, m, 3), dtype=torch.uint8, device=x_t.device)
    err = torch.empty(3, dtype=torch.float32, device=x_t.device)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fpie_grid_step_noalloc(n, m, mask_t.data_ptr(), x_t.data_ptr(), grad_t.data_ptr(),
                                    iteration, img.data_ptr(), err.data_ptr(), ctypes.c_void_p(stream))
    from fpie_gb300 import _abi

    _abi.check(rc)
    torch.cuda.synchronize()
    return img.cpu().numpy(), err.cpu().numpy()


@pytest.mark.parametrize("case", ["circle256", "rand24"])
def test_noalloc_step_matches_grid_solver(case):
    torch = pytest.importorskip("torch")
    from fpie_gb300 import _abi, backend

    lib = _abi.lib()
    d = load_golden(case)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    mask_t = torch.from_numpy(d["grid_mask"]).to(dev)
    x_t = torch.from_numpy(d["grid_tgt"]).to(dev).contiguous()
    grad_t = torch.from_numpy(d["grid_grad"]).to(dev)

    ref = backend.GridSolver(8, 8)
    ref.reset(int(d["grid_n"]), d["grid_mask"], d["grid_tgt"], d["grid_grad"])

    for k in (37, 64):  # two calls in a row; an odd and an even sweep count
        img, err = _noalloc_step(lib, torch, mask_t, x_t, grad_t, k)
        ref_img, ref_err = ref.step(k)
        np.testing.assert_array_equal(x_t.cpu().numpy(), ref.state())
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_allclose(err, ref_err, rtol=1e-5, atol=1e-3)


def test_noalloc_full_size_grid_with_border_pixels():
    """512 x 512 = the limit: the scratch array and its partials table are
    used to their last element; masked pixels on the border read zeros
    outside the grid, as the numpy backend's shifted sums do."""
    torch = pytest.importorskip("torch")
    from fpie_gb300 import _abi, backend
    from oracle import np_jacobi

    lib = _abi.lib()
    rng = np.random.default_rng(5)
    n = m = 512
    mask = (rng.random((n, m)) < 0.7).astype(np.int32)
    mask[0, ::3] = 1
    mask[-1, 1::3] = 1
    mask[::5, 0] = 1
    mask[2::5, -1] = 1
    tgt = rng.uniform(0, 255, (n, m, 3)).astype(np.float32)
    grad = rng.uniform(-60, 60, (n, m, 3)).astype(np.float32)
    grad[mask == 0] = 0
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    mask_t = torch.from_numpy(mask).to(dev)
    x_t = torch.from_numpy(tgt).to(dev).contiguous()
    grad_t = torch.from_numpy(grad).to(dev)
    ref = backend.GridSolver(8, 8)
    ref.reset(n * m, mask, tgt, grad)
    o = np_jacobi.GridJacobi(mask, tgt, grad)
    for k in (51, 30):
        img, err = _noalloc_step(lib, torch, mask_t, x_t, grad_t, k)
        ref_img, ref_err = ref.step(k)
        o.sweep(k)
        np.testing.assert_array_equal(x_t.cpu().numpy(), ref.state())
        np.testing.assert_array_equal(x_t.cpu().numpy(), o.x)
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_allclose(err, ref_err, rtol=1e-5, atol=1e-3)


def test_noalloc_rejects_grids_over_the_limit():
    torch = pytest.importorskip("torch")
    from fpie_gb300 import _abi

    lib = _abi.lib()
    dev = torch.device("cuda", 0)
    n, m = 513, 512  # 262,656 pixels > 262,144
    mask_t = torch.zeros((n, m), dtype=torch.int32, device=dev)
    x_t = torch.zeros((n, m, 3), dtype=torch.float32, device=dev)
    rc = lib.fpie_grid_step_noalloc(n, m, mask_t.data_ptr(), x_t.data_ptr(), x_t.data_ptr(),
                                    1, None, None, None)
    assert rc == _abi.FPIE_ERR_ARG
    assert b"262144" in lib.fpie_last_error()
