"""Property checks of the host-side input construction on random masks
(no GPU): the package's prep against the oracle's restatement, and the
red-black numbering's invariants."""

from __future__ import annotations

import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

from fpie_gb300 import prep  # noqa: E402
from oracle import np_jacobi  # noqa: E402
from oracle import prep as oprep  # noqa: E402


@st.composite
def problems(draw):
    h = draw(st.integers(6, 24))
    w = draw(st.integers(6, 24))
    seed = draw(st.integers(0, 2**31 - 1))
    rng = np.random.default_rng(seed)
    mask = (rng.random((h, w)) > draw(st.floats(0.1, 0.9))).astype(np.uint8) * 255
    mask[h // 2, w // 2] = 255  # at least one pixel off the frame
    src = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
    tgt = rng.integers(0, 256, size=(h, w, 3), dtype=np.uint8)
    mode = draw(st.sampled_from(["src", "avg", "max"]))
    return src, mask, tgt, mode


@settings(max_examples=40, deadline=None)
@given(problems())
def test_grid_inputs_match_the_oracle(p):
    src, mask, tgt, mode = p
    mc, t, g, _ = prep.grid_inputs(src, mask, tgt, (0, 0), (0, 0), mode)
    omc, ot, og, _ = oprep.grid_inputs(src, mask, tgt, (0, 0), (0, 0), mode)
    np.testing.assert_array_equal(mc, omc)
    np.testing.assert_array_equal(t, ot)
    np.testing.assert_array_equal(g, og)


@settings(max_examples=40, deadline=None)
@given(problems())
def test_red_black_numbering(p):
    src, mask, tgt, mode = p
    e = oprep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), mode, order="red_black")
    ids, n_mid = e["ids"], e["n_mid"]
    mc = e["mask"]
    on = ids[mc > 0]
    # a permutation of 1..U, odd cells first, each colour in row-major order
    np.testing.assert_array_equal(np.sort(on), np.arange(1, on.size + 1))
    ii, jj = np.nonzero(mc)
    odd = (ii + jj) % 2 == 1
    assert (ids[ii[odd], jj[odd]] < n_mid).all() and (ids[ii[~odd], jj[~odd]] >= n_mid).all()
    assert (np.diff(ids[ii[odd], jj[odd]]) > 0).all() and (np.diff(ids[ii[~odd], jj[~odd]]) > 0).all()
    # every neighbour in A has the other colour (or is the constant row 0)
    A = e["A"]
    red = np.arange(e["N"]) < n_mid
    nb = A[1:]
    assert not ((nb != 0) & (red[nb] == red[1:, None])).any()
    # the same system as the row-major one, relabelled
    r = oprep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), mode)
    perm = np.zeros(e["N"], np.int64)  # red-black id -> row-major id
    perm[ids[mc > 0]] = r["ids"][mc > 0]
    np.testing.assert_array_equal(r["X"][perm[1:]], e["X"][1:])
    np.testing.assert_array_equal(r["B"][perm[1:]], e["B"][1:])
    np.testing.assert_array_equal(perm[A[1:]], r["A"][perm[1:]])


@settings(max_examples=20, deadline=None)
@given(problems())
def test_red_black_sweep_is_a_gauss_seidel_sweep(p):
    """One red-black sweep equals updating the odd cells, then the even
    cells, one at a time in any order (the colours do not read themselves)."""
    src, mask, tgt, mode = p
    e = oprep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), mode, order="red_black")
    o = np_jacobi.EquRedBlack(e["A"], e["X"], e["B"], e["n_mid"])
    o.sweep(1)
    X = e["X"].copy()
    rng = np.random.default_rng(0)
    for lo, hi in ((1, e["n_mid"]), (e["n_mid"], e["N"])):
        for i in rng.permutation(np.arange(lo, hi)):
            a = e["A"][i]
            s = e["B"][i] + X[a[0]]
            s = s + X[a[1]]
            s = s + X[a[2]]
            s = s + X[a[3]]
            X[i] = s / np.float32(4.0)
    np.testing.assert_array_equal(o.X, X)


@settings(max_examples=40, deadline=None)
@given(problems(), st.sampled_from(["row", "red_black"]))
def test_equ_inputs_match_the_oracle(p, order):
    """The package's slab-based construction of A / X / B equals the oracle's
    unknown-by-unknown restatement, for either numbering."""
    src, mask, tgt, mode = p
    part = ((lambda mc: np.cumsum((mc > 0).reshape(-1)).reshape(mc.shape)) if order == "row"
            else (lambda mc: np_jacobi.red_black_ids(mc)[0]))
    e = oprep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), mode, order=order)
    s = prep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), mode, part)
    for k in ("A", "X", "B"):
        np.testing.assert_array_equal(e[k], getattr(s, k))
    np.testing.assert_array_equal(np.stack(e["tgt_index"]), np.stack(s.tgt_index))


@settings(max_examples=25, deadline=None)
@given(problems(), st.integers(0, 2**31 - 1))
def test_float_images_take_the_float_arithmetic(p, seed):
    """Images that are not uint8 (fractional values) go through the
    reference's float32 arithmetic, not the exact-integer shortcut."""
    src, mask, tgt, mode = p
    rng = np.random.default_rng(seed)
    fsrc = src.astype(np.float32) + rng.random(src.shape).astype(np.float32)
    ftgt = tgt.astype(np.float32) * np.float32(0.77)
    a = oprep.grid_inputs(fsrc, mask, ftgt, (0, 0), (0, 0), mode)
    b = prep.grid_inputs(fsrc, mask, ftgt, (0, 0), (0, 0), mode)
    for x, y in zip(a[:3], b[:3]):
        np.testing.assert_array_equal(x, y)
    e = oprep.equ_inputs(fsrc, mask, ftgt, (0, 0), (0, 0), mode)
    s = prep.equ_inputs(fsrc, mask, ftgt, (0, 0), (0, 0), mode,
                        lambda mc: np.cumsum((mc > 0).reshape(-1)).reshape(mc.shape))
    for k in ("A", "X", "B"):
        np.testing.assert_array_equal(e[k], getattr(s, k))
