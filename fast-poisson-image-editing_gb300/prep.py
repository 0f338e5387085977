"""Host-side construction of solver inputs (the producer of the hot path).

Same semantics as the reference processors' ``reset`` (fpie/process.py),
bit for bit:

* mask: a 3-channel mask is averaged over channels and compared with 128
  (for integer masks this is ``channel sum >= 384``), the 1-pixel frame is
  cleared, and the problem is cropped to the set pixels' bounding box grown
  by one pixel (fpie/process.py:209-224, :338-351);
* gradient mixing 'src' / 'avg' / 'max' (BaseProcessor.mixgrad,
  fpie/process.py:113-122), with ties in 'max' keeping the source term;
* grid inputs: grad = mixed(C-U) + mixed(C-D) + mixed(C-L) + mixed(C-R)
  summed in that order, zero outside the mask (fpie/process.py:362-378);
* equation inputs: ids from the solver's partition (row-major, or odd
  cells first in red-black order), A = ids of (up, down, left, right),
  grad summed (L, R, U, D), B = grad + target values of unmasked
  neighbours added (U, L, R, D), row 0 the constant 0 (fpie/process.py:
  180-190, 225-266).
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Crop:
    x0: int
    x1: int
    y0: int
    y1: int


def binary_mask(mask: np.ndarray) -> np.ndarray:
    """int32 0/1 mask with the outer frame cleared."""
    if mask.ndim == 3:
        if np.issubdtype(mask.dtype, np.integer):
            sel = mask.sum(axis=-1, dtype=np.int64) >= 384
        else:
            sel = mask.mean(axis=-1) >= 128
    else:
        sel = mask >= 128
    out = np.zeros(sel.shape, np.int32)
    out[1:-1, 1:-1] = sel[1:-1, 1:-1]
    return out


def bounding_crop(m01: np.ndarray) -> Crop:
    rows = np.any(m01, axis=1)
    cols = np.any(m01, axis=0)
    if not rows.any():
        raise ValueError("the mask selects no pixel (after clearing its 1-pixel frame)")
    r = np.nonzero(rows)[0]
    c = np.nonzero(cols)[0]
    return Crop(int(r[0]) - 1, int(r[-1]) + 2, int(c[0]) - 1, int(c[-1]) + 2)


def mix(a: np.ndarray, b: np.ndarray, gradient: str) -> np.ndarray:
    """Mixed gradient term of source difference a and target difference b."""
    if gradient == "src":
        return a
    if gradient == "avg":
        return (a + b) / 2
    if gradient == "max":  # b where |a| < |b|, else a (a select: no arithmetic)
        return np.where(np.abs(a) < np.abs(b), b, a)
    raise ValueError(f"unknown gradient mode {gradient!r}")


def _mixed_int(a: np.ndarray, b: np.ndarray, gradient: str) -> np.ndarray:
    """mix() of integer differences of uint8 pixels, times _scale(gradient):
    every mixed term is then an integer (|term| <= 510), so sums of up to
    eight of them are exact in int16 -- and equal, after the division by the
    scale, to the float32 results of mix(), whose partial sums (integers or
    halves below 2^11) are exact as well."""
    if gradient == "src":
        return a
    if gradient == "avg":
        return a + b
    if gradient == "max":
        return np.where(np.abs(a) < np.abs(b), b, a)
    raise ValueError(f"unknown gradient mode {gradient!r}")


def _scale(gradient: str) -> int:
    return 2 if gradient == "avg" else 1


def _arithmetic(src, tgt, gradient):
    """(working dtype, mixer, scale): exact int16 terms for uint8 images
    (the reference's inputs), else the reference's float32 arithmetic."""
    if src.dtype == np.uint8 and tgt.dtype == np.uint8:
        return np.int16, _mixed_int, _scale(gradient)
    return np.float32, mix, 1


def _check_offsets(shape, img_shape, off, crop: Crop, name: str) -> None:
    if (off[0] + crop.x0 < 0 or off[1] + crop.y0 < 0
            or off[0] + crop.x1 > img_shape[0] or off[1] + crop.y1 > img_shape[1]):
        raise ValueError(
            f"mask of shape {shape} at offset {tuple(off)} does not fit the {name} "
            f"image of shape {img_shape[:2]}")


def grid_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, gradient):
    """Return (mask int32[n,m], tgt f32[n,m,3], grad f32[n,m,3], Crop on target)."""
    m01 = binary_mask(mask)
    cr = bounding_crop(m01)
    _check_offsets(mask.shape[:2], src.shape, mask_on_src, cr, "source")
    _check_offsets(mask.shape[:2], tgt.shape, mask_on_tgt, cr, "target")
    mc = m01[cr.x0:cr.x1, cr.y0:cr.y1]
    # uint8 images: exact integer terms (see _mixed_int), the same values as
    # the reference's float32 arithmetic; other dtypes: that arithmetic.
    work, mixer, k = _arithmetic(src, tgt, gradient)
    s = src[mask_on_src[0] + cr.x0:mask_on_src[0] + cr.x1,
            mask_on_src[1] + cr.y0:mask_on_src[1] + cr.y1].astype(work)
    ti = tgt[mask_on_tgt[0] + cr.x0:mask_on_tgt[0] + cr.x1,
             mask_on_tgt[1] + cr.y0:mask_on_tgt[1] + cr.y1].astype(work)
    t = ti.astype(np.float32)
    acc = np.zeros(t.shape, work)
    # Vertical differences between rows i and i+1, then horizontal ones.
    dv_s, dv_t = s[1:] - s[:-1], ti[1:] - ti[:-1]
    acc[1:] += mixer(dv_s, dv_t, gradient)          # centre minus up
    acc[:-1] += mixer(-dv_s, -dv_t, gradient)       # centre minus down
    dh_s, dh_t = s[:, 1:] - s[:, :-1], ti[:, 1:] - ti[:, :-1]
    acc[:, 1:] += mixer(dh_s, dh_t, gradient)       # centre minus left
    acc[:, :-1] += mixer(-dh_s, -dh_t, gradient)    # centre minus right
    acc[mc == 0] = 0
    grad = acc.astype(np.float32)
    if k != 1:
        grad *= np.float32(1.0 / k)
    on_tgt = Crop(mask_on_tgt[0] + cr.x0, mask_on_tgt[0] + cr.x1,
                  mask_on_tgt[1] + cr.y0, mask_on_tgt[1] + cr.y1)
    return mc, t, grad, on_tgt


@dataclasses.dataclass
class EquSystem:
    N: int
    A: np.ndarray
    X: np.ndarray
    B: np.ndarray
    tgt_index: tuple[np.ndarray, np.ndarray]
    crop: Crop | None = None  # the crop on the target

    def placement(self) -> tuple[np.ndarray, int, int] | None:
        """(pos int32[N], n, m): unknown i at row * m + col of the crop
        (pos[0] = 0, unused), for EquSolver.reset(..., placement=...)."""
        if self.crop is None:
            return None
        n, m = self.crop.x1 - self.crop.x0, self.crop.y1 - self.crop.y0
        pos = np.zeros(self.N, np.int32)
        pos[1:] = (self.tgt_index[0] - self.crop.x0) * m + (self.tgt_index[1] - self.crop.y0)
        return pos, n, m


def equ_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, gradient, partition) -> EquSystem:
    """Build A/X/B; ``partition`` is the solver's id assignment (mask -> ids).

    The arithmetic is the reference's, per unknown and in its order
    (fpie/process.py:225-266): the gradient sums the mixed L, R, U, D terms,
    B then adds the target value of each unmasked neighbour in U, L, R, D
    order.  It runs on whole slabs of the crop (every unknown lies inside
    the crop's 1-pixel frame) and gathers the unknowns' rows once, instead
    of gathering neighbour by neighbour.
    """
    m01 = binary_mask(mask)
    cr = bounding_crop(m01)
    _check_offsets(mask.shape[:2], src.shape, mask_on_src, cr, "source")
    _check_offsets(mask.shape[:2], tgt.shape, mask_on_tgt, cr, "target")
    mc = m01[cr.x0:cr.x1, cr.y0:cr.y1]
    ids = np.asarray(partition(mc)).astype(np.int64)
    ids[mc == 0] = 0
    px, py = np.nonzero(mc)
    key = ids[px, py]
    if key.size and not (np.diff(key) > 0).all():  # row-major ids are already in order
        order = np.argsort(key, kind="stable")
        px, py = px[order], py[order]
    N = px.size + 1
    sr, sc_ = mask_on_src[0] + cr.x0, mask_on_src[1] + cr.y0
    tr, tc_ = mask_on_tgt[0] + cr.x0, mask_on_tgt[1] + cr.y0
    n, m = mc.shape
    work, mixer, k = _arithmetic(src, tgt, gradient)
    s = src[sr:sr + n, sc_:sc_ + m].astype(work)
    t = tgt[tr:tr + n, tc_:tc_ + m].astype(work)
    # Interior [1:-1, 1:-1] of the crop and its four shifted neighbours.
    inner = (slice(1, n - 1), slice(1, m - 1))
    shifts = {"L": (slice(1, n - 1), slice(0, m - 2)), "R": (slice(1, n - 1), slice(2, m)),
              "U": (slice(0, n - 2), slice(1, m - 1)), "D": (slice(2, n), slice(1, m - 1))}
    s0, t0 = s[inner], t[inner]
    # uint8 images: integer terms, times k (see _mixed_int), exact, so the
    # sums equal the reference's float32 sums in its order (L, R, U, D, then
    # the unmasked neighbours' target values U, L, R, D); other dtypes: the
    # reference's float32 arithmetic in that order.
    acc = None
    for d in ("L", "R", "U", "D"):
        term = mixer(s0 - s[shifts[d]], t0 - t[shifts[d]], gradient)
        acc = term if acc is None else acc + term
    for d in ("U", "L", "R", "D"):
        outside = np.broadcast_to((mc[shifts[d]] == 0)[..., None], acc.shape)
        np.add(acc, t[shifts[d]] * work(k), out=acc, where=outside)
    q = (px - 1) * (m - 2) + (py - 1)  # unknowns as flat indices of the interior
    A = np.zeros((N, 4), np.int32)
    X = np.zeros((N, 3), np.float32)
    B = np.zeros((N, 3), np.float32)
    X[1:] = np.ascontiguousarray(t0).reshape(-1, 3)[q]
    for j, d in enumerate(("U", "D", "L", "R")):
        A[1:, j] = np.ascontiguousarray(ids[shifts[d]]).reshape(-1)[q]
    B[1:] = acc.reshape(-1, 3)[q]
    if k != 1:
        B[1:] *= np.float32(1.0 / k)
    crop = Crop(mask_on_tgt[0] + cr.x0, mask_on_tgt[0] + cr.x1, mask_on_tgt[1] + cr.y0,
                mask_on_tgt[1] + cr.y1)
    return EquSystem(N, A, X, B, (px + tr, py + tc_), crop)
