"""Processors and backend routing, mirroring ``fpie.process``.

``EquProcessor`` / ``GridProcessor`` take the same constructor arguments as
the reference's (fpie/process.py:149-178, :286-319), build the solver inputs
on the host (``prep``), hand them to the backend solver through the plugin
surface (``partition`` / ``reset`` / ``sync`` / ``step``) and merge the
solver's uint8 result into a copy of the target (fpie/process.py:273-280,
:388-395).

Backends (``ALL_BACKEND``, printed by ``--check-backend``):

* ``gb300``      -- plain FP32 Jacobi on the GB300 kernels (the numpy
                    backend's iteration);
* ``gb300-rb``   -- the OpenMP backend's iterations: red-black Gauss-Seidel
                    for the equation method (fpie/core/openmp/equ.cc), Jacobi
                    for the grid method;
* ``gb300-fp16`` -- iterative refinement, FP16 correction sweeps;
* ``gb300-bf16`` -- iterative refinement, BF16 correction sweeps.

An unknown or unavailable backend prints a hint and raises AssertionError,
as the reference does (fpie/process.py:94-105).
"""

from __future__ import annotations

import os
from abc import ABC, abstractmethod
from typing import Any

import numpy as np

from . import prep

DEFAULT_CPU_CAP = 8


def _default_cpu_count() -> int:
    counts = [c for c in (os.cpu_count(),) if c]
    try:
        counts.append(len(os.sched_getaffinity(0)))
    except (AttributeError, OSError):
        pass
    return max(1, min(min(counts), DEFAULT_CPU_CAP)) if counts else 1


CPU_COUNT = _default_cpu_count()
_PRECISION_OF = {"gb300": "fp32", "gb300-rb": "fp32", "gb300-fp16": "fp16", "gb300-bf16": "bf16"}
ALL_BACKEND = list(_PRECISION_OF)
# When to pick which backend (printed by --check-backend after the list).
BACKEND_NOTES = {
    "gb300": "strict FP32 Jacobi, bit-identical to the reference's numpy solver (default)",
    "gb300-rb": "the reference OpenMP EquSolver's red-black order for --method equ (grid: "
                "Jacobi); reaches a given residual ~20x sooner than Jacobi on an 800x800 paste",
    "gb300-fp16": "--method grid; FP16 correction sweeps refined in FP32: keeps converging where "
                  "FP32 Jacobi stalls (~0.6 LSB from the converged image on large pastes)",
    "gb300-bf16": "--method grid; as gb300-fp16 with BF16 corrections",
}
DEFAULT_BACKEND = "gb300"

_HINTS = {
    "gb300": "The gb300 backend needs its CUDA library (fpie_gb300.build.build()) "
             "and a visible GPU.",
}


def _make_core(kind: str, backend: str, block_size: int, grid_x: int, grid_y: int):
    if backend not in _PRECISION_OF:
        return None
    if kind == "equ" and _PRECISION_OF[backend] != "fp32":
        print(f"{backend} is a grid-only backend: use the grid method (GridProcessor).")
        return None
    from . import backend as _backend  # the native library loads here

    if kind == "equ":
        core = _backend.EquSolver(block_size, order="red_black" if backend == "gb300-rb" else "jacobi")
    else:
        core = _backend.GridSolver(grid_x, grid_y)
    if _PRECISION_OF[backend] != "fp32":
        core.set_precision(_PRECISION_OF[backend])
    return core


class BaseProcessor(ABC):
    """State shared by both processors: gradient mode, rank and the core."""

    def __init__(self, gradient: str, rank: int, backend: str, core: Any | None):
        if core is None:
            print(_HINTS.get(backend.split("-")[0], f"Unknown backend {backend!r}; "
                             f"available: {ALL_BACKEND}"))
            raise AssertionError(f"Invalid backend {backend}.")
        self.gradient = gradient
        self.rank = rank
        self.backend = backend
        self.core = core
        self.root = rank == 0

    def mixgrad(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        return prep.mix(a, b, self.gradient)

    @abstractmethod
    def reset(self, src: np.ndarray, mask: np.ndarray, tgt: np.ndarray,
              mask_on_src: tuple[int, int], mask_on_tgt: tuple[int, int]) -> int:
        ...

    def sync(self) -> None:
        self.core.sync()

    @abstractmethod
    def step(self, iteration: int) -> tuple[np.ndarray, np.ndarray] | None:
        ...


class EquProcessor(BaseProcessor):
    """Equation-form processor: unknowns relabelled, neighbour table A."""

    def __init__(self, gradient: str = "max", backend: str = DEFAULT_BACKEND,
                 n_cpu: int = CPU_COUNT, min_interval: int = 100, block_size: int = 1024,
                 device_prep: bool = False):
        """device_prep: build ids/A/X/B on the GPU from the uint8 images
        (fpie_equ_reset_images) instead of with numpy on the host."""
        super().__init__(gradient, 0, backend, _make_core("equ", backend, block_size, 8, 8))
        self.device_prep = device_prep

    def mask2index(self, mask: np.ndarray):
        """ids, N, and the unknowns' (row, col) in id order (fpie/process.py:180-190)."""
        ids = np.asarray(self.core.partition(mask)).astype(np.int64)
        ids[mask == 0] = 0
        x, y = np.nonzero(mask)
        order = np.argsort(ids[x, y], kind="stable")
        return ids, x.size + 1, x[order], y[order]

    def reset(self, src, mask, tgt, mask_on_src, mask_on_tgt) -> int:
        if self.device_prep:
            N, _, self.tgt_index = self.core.reset_images(src, mask, tgt, mask_on_src, mask_on_tgt,
                                                          self.gradient)
            self.tgt = tgt.copy()
            return N
        system = prep.equ_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, self.gradient,
                                 self.core.partition)
        self.tgt = tgt.copy()
        self.tgt_index = system.tgt_index
        # The mask gives every unknown's pixel: the solver checks that
        # placement on the device instead of searching for one.
        self.core.reset(system.N, system.A, system.X, system.B, placement=system.placement())
        return system.N

    def step(self, iteration: int):
        x, err = self.core.step(iteration)
        self.tgt[self.tgt_index] = x[1:]
        return self.tgt, err


class GridProcessor(BaseProcessor):
    """Grid-form processor: the cropped image with its mask."""

    def __init__(self, gradient: str = "max", backend: str = DEFAULT_BACKEND,
                 n_cpu: int = CPU_COUNT, min_interval: int = 100, block_size: int = 1024,
                 grid_x: int = 8, grid_y: int = 8, device_prep: bool = False):
        """device_prep: build mask/crop/grad on the GPU from the uint8 images
        (fpie_grid_reset_images) instead of with numpy on the host."""
        super().__init__(gradient, 0, backend, _make_core("grid", backend, block_size, grid_x, grid_y))
        self.device_prep = device_prep

    def reset(self, src, mask, tgt, mask_on_src, mask_on_tgt) -> int:
        if self.device_prep:
            x0, x1, y0, y1 = self.core.reset_images(src, mask, tgt, mask_on_src, mask_on_tgt,
                                                    self.gradient)
            self.x0, self.x1, self.y0, self.y1 = x0, x1, y0, y1
            self.tgt = tgt.copy()
            return (x1 - x0) * (y1 - y0)
        mc, t, grad, crop = prep.grid_inputs(src, mask, tgt, mask_on_src, mask_on_tgt, self.gradient)
        self.x0, self.x1, self.y0, self.y1 = crop.x0, crop.x1, crop.y0, crop.y1
        self.tgt = tgt.copy()
        n = int(mc.shape[0] * mc.shape[1])
        self.core.reset(n, mc, t, grad)
        return n

    def step(self, iteration: int):
        img, err = self.core.step(iteration)
        self.tgt[self.x0:self.x1, self.y0:self.y1] = img
        return self.tgt, err
