"""GPU-side reset (mask threshold, crop, gradient mixing) against the reference.

The mask, crop box and grad the GPU builds from the uint8 images must equal
the reference processor's bit for bit, and so must every later state.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import problem_args

pytestmark = pytest.mark.gpu


def test_inputs_equal_reference(golden):
    from fpie_gb300 import backend

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    s = backend.GridSolver(8, 8)
    box = s.reset_images(src, mask, tgt, mos, mot, grad)
    assert box == tuple(int(v) for v in d["grid_box"])
    m, g = s.inputs()
    np.testing.assert_array_equal(m, d["grid_mask"])
    np.testing.assert_array_equal(g, d["grid_grad"])
    np.testing.assert_array_equal(s.state(), d["grid_tgt"])
    k = int(d["checkpoints"][0])
    img, err = s.step(k)
    np.testing.assert_array_equal(img, d[f"grid_img_{k}"])


@pytest.mark.parametrize("gradient", ["src", "avg", "max"])
def test_square800_inputs_equal_host_prep(gradient):
    from fpie_gb300 import backend, prep, workloads

    pb = workloads.square800()
    mc, t, g, crop = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, gradient)
    s = backend.GridSolver(8, 8)
    box = s.reset_images(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, gradient)
    assert box == (crop.x0, crop.x1, crop.y0, crop.y1)
    m, gg = s.inputs()
    np.testing.assert_array_equal(m, mc)
    np.testing.assert_array_equal(gg, g)


def test_device_tensors_and_three_channel_mask():
    torch = pytest.importorskip("torch")
    from fpie_gb300 import backend, prep

    rng = np.random.default_rng(4)
    src = rng.integers(0, 256, (70, 90, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, (80, 100, 3), dtype=np.uint8)
    mask3 = np.zeros((50, 60, 3), np.uint8)
    mask3[5:40, 6:50] = (200, 100, 90)   # sum 390 >= 384: on
    mask3[10:20, 10:20] = (128, 128, 127)  # 383: off
    mc, t, g, crop = prep.grid_inputs(src, mask3, tgt, (7, 11), (9, 13), "max")
    dev = torch.device("cuda", 0)
    s = backend.GridSolver(8, 8)
    box = s.reset_images(torch.from_numpy(src).to(dev), torch.from_numpy(mask3).to(dev),
                         torch.from_numpy(tgt).to(dev), (7, 11), (9, 13), "max")
    torch.cuda.synchronize()
    assert box == (crop.x0, crop.x1, crop.y0, crop.y1)
    m, gg = s.inputs()
    np.testing.assert_array_equal(m, mc)
    np.testing.assert_array_equal(gg, g)


def test_bad_inputs_raise():
    from fpie_gb300 import _abi, backend

    img = np.zeros((20, 20, 3), np.uint8)
    s = backend.GridSolver(8, 8)
    with pytest.raises(_abi.FpieArgumentError):
        s.reset_images(img, np.zeros((20, 20), np.uint8), img, (0, 0), (0, 0), "max")
    mask = np.zeros((20, 20), np.uint8)
    mask[2:18, 2:18] = 255
    with pytest.raises(_abi.FpieArgumentError):
        s.reset_images(img, mask, img, (0, 5), (0, 0), "max")
    with pytest.raises(_abi.FpieArgumentError):
        s.reset_images(img, mask, img, (0, 0), (0, 0), "median")


def test_processor_with_device_prep(golden):
    from fpie_gb300.process import GridProcessor

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    proc = GridProcessor(gradient=grad, backend="gb300", device_prep=True)
    proc.reset(src, mask, tgt.copy(), mos, mot)
    k = int(d["checkpoints"][-1])
    out, err = proc.step(k)
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    np.testing.assert_array_equal(out[x0:x1, y0:y1], d[f"grid_img_{k}"])


def test_equ_inputs_equal_reference(golden):
    from fpie_gb300 import backend

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    s = backend.EquSolver(256)
    N, box, (rows, cols) = s.reset_images(src, mask, tgt, mos, mot, grad)
    assert N == int(d["equ_N"])
    assert box == tuple(int(v) for v in d["grid_box"])
    A, B = s.inputs()
    np.testing.assert_array_equal(A, d["equ_A"])
    np.testing.assert_array_equal(B, d["equ_B"])
    np.testing.assert_array_equal(s.state(), d["equ_X"])
    np.testing.assert_array_equal(np.stack([rows, cols]), d["equ_tgt_index"])


@pytest.mark.parametrize("gradient", ["src", "avg", "max"])
def test_equ_square800_equals_host_prep(gradient):
    from fpie_gb300 import backend, prep, workloads

    pb = workloads.square800()
    s = backend.EquSolver(256)
    N, box, idx = s.reset_images(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, gradient)
    host = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, gradient,
                           lambda m: np.cumsum((m > 0).reshape(-1)).reshape(m.shape))
    assert N == host.N == 640001
    A, B = s.inputs()
    np.testing.assert_array_equal(A, host.A)
    np.testing.assert_array_equal(B, host.B)
    np.testing.assert_array_equal(s.state(), host.X)
    np.testing.assert_array_equal(np.stack(idx), np.stack(host.tgt_index))


def test_equ_processor_with_device_prep(golden):
    from fpie_gb300.process import EquProcessor

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    proc = EquProcessor(gradient=grad, backend="gb300", device_prep=True)
    proc.reset(src, mask, tgt.copy(), mos, mot)
    k = int(d["checkpoints"][-1])
    out, err = proc.step(k)
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    np.testing.assert_array_equal(out[x0:x1, y0:y1], d[f"equ_img_{k}"])
