"""Batched paste jobs: many uneven grid problems in one persistent launch.

``BatchSolver`` holds jobs (each a GridSolver problem: int32 mask, float32
target and grad crops, plus a sweep count) in device memory under an HBM
budget and advances all of them with one persistent kernel launch per
``run`` (see include/fpie_gb300.h, ``fpie_batch_*``).  Results are
bit-identical to ``GridSolver`` runs of the same sweeps.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from .backend import _as, _ptr


class BatchSolver:
    def __init__(self, budget_bytes: float = 40e9, precision: str = "fp32") -> None:
        from .backend import PRECISIONS

        self._lib = _abi.lib()
        self._h = ctypes.c_void_p()
        _abi.call("fpie_batch_create", float(budget_bytes), ctypes.byref(self._h))
        if precision not in PRECISIONS:
            raise _abi.FpieArgumentError(f"unknown precision {precision!r}")
        _abi.call("fpie_batch_set_precision", self._h, PRECISIONS[precision])
        self.precision = precision
        self._shape: dict[int, tuple[int, int]] = {}

    def job_bytes_for(self, n: int, m: int) -> int:
        """Device bytes a job of an n x m grid takes in this batch's precision."""
        b = ctypes.c_double(0)
        _abi.call("fpie_batch_job_bytes_for", self._h, int(n), int(m), ctypes.byref(b))
        return int(b.value)

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.fpie_batch_destroy(h)
            except Exception:
                pass
            h.value = None

    close = __del__

    @staticmethod
    def job_bytes(n: int, m: int) -> int:
        b = ctypes.c_double(0)
        _abi.call("fpie_batch_job_bytes", int(n), int(m), ctypes.byref(b))
        return int(b.value)

    def add(self, mask: np.ndarray, tgt: np.ndarray, grad: np.ndarray, iterations: int) -> int:
        m = _as(mask, np.int32, (None, None), "mask")
        n_, m_ = m.shape
        t = _as(tgt, np.float32, (n_, m_, 3), "tgt")
        g = _as(grad, np.float32, (n_, m_, 3), "grad")
        jid = ctypes.c_int(-1)
        _abi.call("fpie_batch_add", self._h, n_, m_, _ptr(m), _ptr(t), _ptr(g), int(iterations),
                  ctypes.byref(jid))
        self._shape[jid.value] = (n_, m_)
        return jid.value

    def add_images(self, src, mask, tgt, mask_on_src: tuple[int, int],
                   mask_on_tgt: tuple[int, int], gradient: str, iterations: int):
        """A job from uint8 images (host arrays), built as GridProcessor.reset
        builds the grid inputs, on the GPU.  Returns (job id, crop box on the
        target: row0, row1, col0, col1)."""
        from .backend import _image_args

        keep, args, mode, on_dev = _image_args(src, mask, tgt, gradient)
        if on_dev:
            raise _abi.FpieArgumentError("add_images takes host (numpy) images")
        jid = ctypes.c_int(-1)
        box = (ctypes.c_int * 4)()
        _abi.call("fpie_batch_add_images", self._h, *args, int(mask_on_src[0]), int(mask_on_src[1]),
                  int(mask_on_tgt[0]), int(mask_on_tgt[1]), mode, int(iterations), ctypes.byref(jid),
                  box)
        del keep
        self._shape[jid.value] = (box[1] - box[0], box[3] - box[2])
        return jid.value, tuple(box)

    def run(self, max_sweeps: int = -1) -> None:
        """Advance every job by min(max_sweeps, its remaining sweeps); -1 = to completion."""
        _abi.call("fpie_batch_run", self._h, int(max_sweeps))

    def run_async(self, max_sweeps: int = -1) -> None:
        """``run`` without waiting for the launch; ``wait`` joins it."""
        _abi.call("fpie_batch_run_async", self._h, int(max_sweeps))

    def wait(self) -> None:
        _abi.call("fpie_batch_wait", self._h)

    def norms_async(self, jobs: list[int]) -> None:
        """Queue the norms of `jobs` (after the queued work); ``norms_wait`` returns them."""
        self._norm_ids = np.ascontiguousarray(jobs, dtype=np.int32)
        _abi.call("fpie_batch_norms_async", self._h,
                  _ptr(self._norm_ids) if len(self._norm_ids) else None, len(self._norm_ids))

    def norms_wait(self) -> np.ndarray:
        """[count, 6] float64 of the last ``norms_async``, as ``norms``."""
        out = np.empty((len(self._norm_ids), 6), np.float64)
        _abi.call("fpie_batch_norms_wait", self._h, _ptr(out) if len(out) else None)
        return out

    def progress(self, job: int) -> tuple[int, int]:
        d, t = ctypes.c_int(0), ctypes.c_int(0)
        _abi.call("fpie_batch_progress", self._h, int(job), ctypes.byref(d), ctypes.byref(t))
        return d.value, t.value

    def result(self, job: int) -> tuple[np.ndarray, np.ndarray]:
        n_, m_ = self._shape[job]
        img = np.empty((n_, m_, 3), np.uint8)
        err = np.empty(3, np.float32)
        _abi.call("fpie_batch_result", self._h, int(job), _ptr(img), _ptr(err))
        return img, err

    def state(self, job: int) -> np.ndarray:
        n_, m_ = self._shape[job]
        out = np.empty((n_, m_, 3), np.float32)
        _abi.call("fpie_batch_state", self._h, int(job), _ptr(out))
        return out

    def norms(self, jobs: list[int]) -> np.ndarray:
        """[len(jobs), 6] float64: max |r| per channel, then sum |r| per channel."""
        ids = np.ascontiguousarray(jobs, dtype=np.int32)
        out = np.empty((len(ids), 6), np.float64)
        if len(ids):
            _abi.call("fpie_batch_norms", self._h, _ptr(ids), len(ids), _ptr(out))
        return out

    def remove(self, job: int) -> None:
        _abi.call("fpie_batch_remove", self._h, int(job))
        self._shape.pop(job, None)

    def memory(self) -> tuple[float, float]:
        u, b = ctypes.c_double(0), ctypes.c_double(0)
        _abi.call("fpie_batch_memory", self._h, ctypes.byref(u), ctypes.byref(b))
        return u.value, b.value

    def set_kernel(self, name: str) -> None:
        _abi.call("fpie_batch_set_kernel", self._h, name.encode())

    @property
    def kernel(self) -> str:
        buf = ctypes.create_string_buffer(64)
        _abi.call("fpie_batch_kernel", self._h, buf, 64)
        return buf.value.decode()

    def set_spin_limit(self, spins: int) -> None:
        _abi.call("fpie_batch_set_spin_limit", self._h, ctypes.c_longlong(int(spins)))

    @property
    def launches(self) -> int:
        c = ctypes.c_longlong(0)
        _abi.call("fpie_batch_launch_count", self._h, ctypes.byref(c))
        return c.value
