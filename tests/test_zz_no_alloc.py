"""The allocation-free grid step against the solver object, on the GPU.

``fpie_grid_step_noalloc`` serves callers that cannot allocate device memory
where they need a step (stream capture, pool-owned device memory,
latency-critical loops): they pass every buffer, and the step's own scratch
is a fixed array inside the library.  This test calls it through the C ABI
twice in a row on the same state and checks each result against
``GridSolver`` (the existing entry point) after the same total sweeps:
state and uint8 image bit for bit, err within rtol 1e-5.

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
