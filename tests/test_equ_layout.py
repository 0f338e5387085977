"""Placement of equation systems on a grid (host code, no GPU).

An EquSolver system whose index table A is a 4-neighbour raster stencil --
what EquProcessor builds from a mask (fpie/process.py:252-266) -- is swept
by the grid kernels; these tests pin the placement the library computes
(fpie_equ_raster_layout) against the oracle's systems, and its refusals.
"""

from __future__ import annotations

import numpy as np
import pytest

from fpie_gb300 import backend, workloads
from oracle import prep

DIRS = [(-1, 0), (1, 0), (0, -1), (0, 1)]  # A columns: up, down, left, right


def _check_layout(A, pos, n, m):
    """Every unknown's grid neighbours are exactly its A entries."""
    occ = np.zeros(n * m, np.int64)
    assert (pos[1:] >= 0).all() and (pos[1:] < n * m).all()
    assert np.unique(pos[1:]).size == pos.size - 1
    occ[pos[1:]] = np.arange(1, pos.size)
    r, c = pos[1:] // m, pos[1:] % m
    for k, (dr, dc) in enumerate(DIRS):
        rr, cc = r + dr, c + dc
        assert ((rr >= 0) & (rr < n) & (cc >= 0) & (cc < m)).all()
        np.testing.assert_array_equal(occ[rr * m + cc], A[1:, k])


def test_single_component_is_the_crop():
    """circle256: one component, placed exactly where the crop has it."""
    pb = workloads.circle256()
    d = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)
    A = d["A"]
    res = backend.raster_layout(A)
    assert res is not None
    pos, (n, m) = res
    assert (n, m) == d["ids"].shape
    ids = d["ids"]
    rows, cols = np.nonzero(ids)
    order = np.argsort(ids[rows, cols])
    np.testing.assert_array_equal(pos[1:], rows[order] * m + cols[order])
    _check_layout(A, pos, n, m)


def test_components_are_stacked():
    """Two disks, a square and a lone pixel: each component keeps its shape,
    components sit one below the other, a row apart."""
    n0, m0 = 120, 150
    mask = np.zeros((n0, m0), np.uint8)
    yy, xx = np.mgrid[:n0, :m0]
    mask[(yy - 30) ** 2 + (xx - 30) ** 2 < 20 ** 2] = 255
    mask[(yy - 80) ** 2 + (xx - 100) ** 2 < 25 ** 2] = 255
    mask[60:70, 10:40] = 255
    mask[20, 120] = 255
    src = workloads.smooth_image(3, n0 + 10, m0 + 10, 8)
    tgt = workloads.smooth_image(4, n0 + 10, m0 + 10, 8)
    d = prep.equ_inputs(src, mask, tgt, (0, 0), (0, 0), "max")
    res = backend.raster_layout(d["A"])
    assert res is not None
    pos, (n, m) = res
    _check_layout(d["A"], pos, n, m)


def test_non_raster_systems_are_refused():
    rng = np.random.default_rng(5)
    pb = workloads.circle256()
    A = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient)["A"]
    assert backend.raster_layout(rng.integers(0, 40, (40, 4)).astype(np.int32)) is None
    # (Exchanging the up and down columns everywhere is a mirrored image,
    # still a raster stencil; one link pointing elsewhere is not.)
    assert backend.raster_layout(A[:, [1, 0, 2, 3]].copy()) is not None
    far = A.copy()
    i = int(np.nonzero(A[:, 3])[0][10])
    far[i, 3] = A.shape[0] - 1                     # a right link to a far unknown
    assert backend.raster_layout(far) is None
    row0 = A.copy()
    row0[0, 2] = 5                                 # row 0 is not the constant
    assert backend.raster_layout(row0) is None
    one = A.copy()
    one[7, 3] = 0                                  # a missing right link
    assert backend.raster_layout(one) is None
    assert backend.raster_layout(np.zeros((1, 4), np.int32)) is None   # no unknown


def test_isolated_unknowns():
    """Unknowns with no unknown neighbour: one pixel each, a row apart."""
    A = np.zeros((4, 4), np.int32)
    res = backend.raster_layout(A)
    assert res is not None
    pos, (n, m) = res
    assert (n, m) == (7, 3)
    np.testing.assert_array_equal(pos[1:], [1 * 3 + 1, 3 * 3 + 1, 5 * 3 + 1])
    _check_layout(A, pos, n, m)
