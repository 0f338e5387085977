"""The processors with the gb300 backend, as the reference's tests use them."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import problem_args

pytestmark = pytest.mark.gpu


def test_smoke_like_reference():
    """The reference smoke test's checks (tests/test_smoke.py:26-46)."""
    from fpie_gb300.process import EquProcessor, GridProcessor

    src = np.zeros((6, 6, 3), np.uint8)
    mask = np.zeros((6, 6), np.uint8)
    mask[2:4, 2:4] = 255
    tgt = np.ones((6, 6, 3), np.uint8) * 10
    for cls in (EquProcessor, GridProcessor):
        proc = cls(backend="gb300")
        n = proc.reset(src, mask, tgt, (0, 0), (0, 0))
        out, err = proc.step(2)
        assert n > 0 and out.shape == tgt.shape and out.dtype == np.uint8 and err.shape == (3,)


def test_processors_match_reference_output(golden):
    from fpie_gb300.process import EquProcessor, GridProcessor

    name, d = golden
    args = problem_args(d)
    src, mask, tgt, mos, mot, grad = args
    x0, x1, y0, y1 = (int(v) for v in d["grid_box"])
    for cls, key in ((GridProcessor, "grid"), (EquProcessor, "equ")):
        proc = cls(gradient=grad, backend="gb300", grid_x=1, grid_y=1) if cls is GridProcessor \
            else cls(gradient=grad, backend="gb300")
        proc.reset(src, mask, tgt.copy(), mos, mot)
        done = 0
        for k in (int(v) for v in d["checkpoints"]):
            out, err = proc.step(k - done)
            done = k
            np.testing.assert_array_equal(out[x0:x1, y0:y1], d[f"{key}_img_{k}"])
            outside = np.ones(tgt.shape[:2], bool)
            outside[x0:x1, y0:y1] = False
            np.testing.assert_array_equal(out[outside], tgt[outside])
            np.testing.assert_allclose(err, d[f"{key}_err_{k}"], rtol=1e-4, atol=1e-3)
