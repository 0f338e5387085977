"""Host-side pieces that need no GPU: input construction, routing, the ABI."""

from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import ROOT, problem_args
from fpie_gb300 import _abi, build, prep, process, workloads


def _numpy_partition(m):
    return np.cumsum((m > 0).reshape(-1)).reshape(m.shape)


def test_grid_inputs_match_reference(golden):
    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    mc, t, g, crop = prep.grid_inputs(src, mask, tgt, mos, mot, grad)
    np.testing.assert_array_equal(mc, d["grid_mask"])
    np.testing.assert_array_equal(t, d["grid_tgt"])
    np.testing.assert_array_equal(g, d["grid_grad"])
    assert (crop.x0, crop.x1, crop.y0, crop.y1) == tuple(int(v) for v in d["grid_box"])


def test_equ_inputs_match_reference(golden):
    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    s = prep.equ_inputs(src, mask, tgt, mos, mot, grad, _numpy_partition)
    assert s.N == int(d["equ_N"])
    np.testing.assert_array_equal(s.A, d["equ_A"])
    np.testing.assert_array_equal(s.X, d["equ_X"])
    np.testing.assert_array_equal(s.B, d["equ_B"])
    np.testing.assert_array_equal(np.stack(s.tgt_index), d["equ_tgt_index"])


def test_inputs_match_oracle_at_640k_unknowns():
    from oracle import prep as oprep

    pb = workloads.square800()
    a = oprep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    b = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    e0 = oprep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    e1 = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                         _numpy_partition)
    assert e0["N"] == e1.N == 640001
    for k in ("A", "X", "B"):
        np.testing.assert_array_equal(e0[k], getattr(e1, k))


def test_empty_mask_and_bad_offsets_raise():
    src = np.zeros((8, 8, 3), np.uint8)
    with pytest.raises(ValueError):
        prep.grid_inputs(src, np.zeros((8, 8), np.uint8), src, (0, 0), (0, 0), "max")
    mask = np.zeros((8, 8), np.uint8)
    mask[2:5, 2:5] = 255
    with pytest.raises(ValueError):
        prep.grid_inputs(src, mask, src, (5, 0), (0, 0), "max")
    with pytest.raises(ValueError):
        prep.mix(np.zeros(1), np.zeros(1), "median")


def test_backend_list_and_invalid_backend(capsys):
    assert process.ALL_BACKEND == ["gb300", "gb300-rb", "gb300-fp16", "gb300-bf16"]
    assert process.DEFAULT_BACKEND == "gb300"
    with pytest.raises(AssertionError):
        process.GridProcessor(backend="numpy")
    assert "available" in capsys.readouterr().out


def _declared_symbols() -> list[str]:
    text = (ROOT / "include" / "fpie_gb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(fpie_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    build.build()
    lib = ctypes.CDLL(str(_abi.library_path()))
    names = _declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_abi._PROTOS)
    assert _abi.lib().fpie_version() >= 100


def test_no_gpu_means_a_loud_error():
    """Without a device the backend refuses to run; there is no CPU path."""
    build.build()
    if _abi.device_count() > 0:
        pytest.skip("a GPU is visible")
    from fpie_gb300 import backend

    with pytest.raises(_abi.FpieError):
        backend.GridSolver(8, 8)
    with pytest.raises(_abi.FpieError):
        backend.EquSolver(256)


def test_equ_placement_follows_the_target_index(golden):
    from fpie_gb300 import prep as pprep
    from oracle import np_jacobi

    name, d = golden
    src, mask, tgt, mos, mot, grad = problem_args(d)
    for part in (lambda mc: np.cumsum((mc > 0).reshape(-1)).reshape(mc.shape),
                 lambda mc: np_jacobi.red_black_ids(mc)[0]):
        sysm = pprep.equ_inputs(src, mask, tgt, mos, mot, grad, part)
        pos, n, m = sysm.placement()
        assert (n, m) == tuple(d["grid_mask"].shape)
        r, c = pos[1:] // m, pos[1:] % m
        np.testing.assert_array_equal(r + sysm.crop.x0, sysm.tgt_index[0])
        np.testing.assert_array_equal(c + sysm.crop.y0, sysm.tgt_index[1])
        assert (d["grid_mask"][r, c] != 0).all()


def test_fp32_probe_rejects_bad_arguments_without_a_gpu_call():
    """Argument checks come before any CUDA call (kind and iteration count)."""
    from fpie_gb300 import _abi

    import ctypes

    out = ctypes.c_double(0)
    lib = _abi.lib()
    assert lib.fpie_probe_fp32_rate(None, 7, 100, ctypes.byref(out)) == _abi.FPIE_ERR_ARG
    assert lib.fpie_probe_fp32_rate(None, 0, 0, ctypes.byref(out)) == _abi.FPIE_ERR_ARG
    assert lib.fpie_probe_fp32_rate(None, 0, 100, None) == _abi.FPIE_ERR_ARG
