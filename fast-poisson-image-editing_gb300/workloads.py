"""Seeded synthetic paste problems shaped like the benchmark workloads.

No image files are read: every problem is generated from a seed so the same
inputs can be rebuilt on any machine.  An image is a coarse uniform[0,255]
field bilinearly upsampled to full size, plus Gaussian noise (sigma 8), rounded
and clipped to uint8.

Workloads (sizes are those of the fpie benchmark tables, docs/benchmark.md,
scaled to the configurations this backend is measured on):

* ``circle256``  -- 256x256 source and target, 16x16 base field, filled circle
  of radius 96 at the centre, zero offsets, 'src' gradient, 5000 sweeps.
* ``square800``  -- 1024x1024 target, 900x900 source, 32x32 base field, an
  802x802 mask whose inner 800x800 square is set (640,000 unknowns), mask
  placed at (49,49) on the source and (99,99) on the target, 'max' gradient,
  5000 sweeps.
* ``circle1800`` -- 4096x4096 source and target, 16x16 base field, circle of
  radius 1800 (about 10.2 M unknowns), 'max' gradient.
* ``circle450``  -- the same construction at 1024x1024, radius 450 (636,121
  unknowns, 903x903 crop): the smallest circle paste on which plain FP32
  Jacobi stalls above 0.5 intensity units of the converged solution (at
  0.566), so the precision comparison runs on it in seconds.
* ``jobs``       -- a seeded mix of uneven paste jobs (circles, squares and
  Gaussian-smoothed noise blobs) for the batched and serving forms.
"""

from __future__ import annotations

import dataclasses

import numpy as np


@dataclasses.dataclass
class Problem:
    """One paste job: the arguments of ``Processor.reset`` plus its sweeps."""

    name: str
    src: np.ndarray
    mask: np.ndarray
    tgt: np.ndarray
    mask_on_src: tuple[int, int]
    mask_on_tgt: tuple[int, int]
    gradient: str
    iterations: int


def smooth_image(seed: int, h: int, w: int, base: int, sigma: float = 8.0) -> np.ndarray:
    """Return an HxWx3 uint8 image: upsampled uniform field plus noise."""
    rng = np.random.default_rng(seed)
    field = rng.uniform(0.0, 255.0, size=(base, base, 3))
    ys = np.linspace(0.0, base - 1.0, h)
    xs = np.linspace(0.0, base - 1.0, w)
    iy = np.minimum(np.floor(ys).astype(np.int64), base - 2)
    ix = np.minimum(np.floor(xs).astype(np.int64), base - 2)
    fy = (ys - iy)[:, None, None]
    fx = (xs - ix)[None, :, None]
    f00 = field[iy][:, ix]
    f01 = field[iy][:, ix + 1]
    f10 = field[iy + 1][:, ix]
    f11 = field[iy + 1][:, ix + 1]
    img = (1 - fy) * ((1 - fx) * f00 + fx * f01) + fy * ((1 - fx) * f10 + fx * f11)
    img = img + rng.normal(0.0, sigma, size=img.shape)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def disk_mask(h: int, w: int, radius: float, centre: tuple[float, float] | None = None) -> np.ndarray:
    """Return an HxW uint8 mask (0/255) holding a filled circle."""
    cy, cx = centre if centre is not None else (h // 2, w // 2)
    yy, xx = np.ogrid[:h, :w]
    inside = (yy - cy) ** 2 + (xx - cx) ** 2 <= radius * radius
    return inside.astype(np.uint8) * 255


def circle256(iterations: int = 5000) -> Problem:
    """256x256 circle paste, 'src' gradient."""
    src = smooth_image(1, 256, 256, 16)
    tgt = smooth_image(2, 256, 256, 16)
    return Problem("circle256", src, disk_mask(256, 256, 96), tgt, (0, 0), (0, 0), "src", iterations)


def square800(iterations: int = 5000) -> Problem:
    """800x800 square (640k unknowns) from a 900^2 source into a 1024^2 target."""
    src = smooth_image(3, 900, 900, 32)
    tgt = smooth_image(4, 1024, 1024, 32)
    mask = np.zeros((802, 802), np.uint8)
    mask[1:801, 1:801] = 255
    return Problem("square800", src, mask, tgt, (49, 49), (99, 99), "max", iterations)


def circle1800(iterations: int = 0) -> Problem:
    """4096x4096 paste with a radius-1800 circle (about 10.2 M unknowns)."""
    src = smooth_image(5, 4096, 4096, 16)
    tgt = smooth_image(6, 4096, 4096, 16)
    return Problem("circle1800", src, disk_mask(4096, 4096, 1800), tgt, (0, 0), (0, 0), "max", iterations)


def circle450(iterations: int = 0) -> Problem:
    """1024x1024 paste with a radius-450 circle (636,121 unknowns)."""
    src = smooth_image(5, 1024, 1024, 16)
    tgt = smooth_image(6, 1024, 1024, 16)
    return Problem("circle450", src, disk_mask(1024, 1024, 450), tgt, (0, 0), (0, 0), "max", iterations)


def blob_mask(rng: np.random.Generator, h: int, w: int, sigma: float = 6.0) -> np.ndarray:
    """Gaussian-smoothed uniform noise thresholded at 0.5, as a 0/255 mask.

    The smoothing is a separable FFT-free Gaussian (explicit 1-D kernels); the
    smoothed field is renormalised to [0,1] before thresholding so the blob
    covers a sizeable part of the box.
    """
    noise = rng.uniform(0.0, 1.0, size=(h, w))
    rad = int(3 * sigma)
    t = np.arange(-rad, rad + 1, dtype=np.float64)
    k = np.exp(-0.5 * (t / sigma) ** 2)
    k /= k.sum()
    pad = np.pad(noise, rad, mode="reflect")
    rows = sum(k[i] * pad[i : i + h, :] for i in range(2 * rad + 1))
    sm = sum(k[i] * rows[:, i : i + w] for i in range(2 * rad + 1))
    sm = (sm - sm.min()) / max(sm.max() - sm.min(), 1e-12)
    m = (sm > 0.5).astype(np.uint8) * 255
    m[0, :] = m[-1, :] = 0
    m[:, 0] = m[:, -1] = 0
    return m


def job_mix(n_jobs: int = 256, seed: int = 7, min_box: int = 32, max_box: int = 1024,
            it_lo: int = 2000, it_hi: int = 10000) -> list[Problem]:
    """Uneven paste jobs: log-uniform boxes, mixed shapes, random gradient.

    Each job's images are box+margin in size; the mask has the box's size and
    is placed at a fixed margin offset on both images.
    """
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        side = int(round(np.exp(rng.uniform(np.log(min_box), np.log(max_box)))))
        h = w = max(side, 8)
        kind = rng.integers(0, 3)
        if kind == 0:
            mask = disk_mask(h, w, (min(h, w) - 2) / 2.0, ((h - 1) / 2.0, (w - 1) / 2.0))
        elif kind == 1:
            mask = np.zeros((h, w), np.uint8)
            mask[1:-1, 1:-1] = 255
        else:
            mask = blob_mask(rng, h, w)
            if not mask.any():
                mask[1:-1, 1:-1] = 255
        margin = 4
        base = int(rng.integers(8, 33))
        src = smooth_image(int(rng.integers(1 << 30)), h + 2 * margin, w + 2 * margin, base)
        tgt = smooth_image(int(rng.integers(1 << 30)), h + 2 * margin, w + 2 * margin, base)
        grad = "src" if rng.integers(0, 2) == 0 else "max"
        iters = int(rng.integers(it_lo, it_hi + 1))
        jobs.append(Problem(f"job{j}", src, mask, tgt, (margin, margin), (margin, margin), grad, iters))
    return jobs


WORKLOADS = {"circle256": circle256, "square800": square800, "circle450": circle450,
             "circle1800": circle1800}
