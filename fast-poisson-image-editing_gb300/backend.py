"""fpie solver plugin classes backed by the GB300 CUDA library.

``EquSolver`` and ``GridSolver`` have the methods, arguments, dtypes and
return shapes of the reference's native solver classes (pybind11 exports in
fpie/core/cuda/solver.cc:3-15 over fpie/core/base_solver.h), so
``EquProcessor`` / ``GridProcessor`` drive them unchanged:

* ``EquSolver(block_size)``: ``partition(mask) -> int32[n,m]``,
  ``reset(N, A int32[N,4], X f32[N,3], B f32[N,3])``, ``sync()``,
  ``step(iteration) -> (uint8[N,3], float32[3])``.
* ``GridSolver(grid_x, grid_y)``: ``reset(N, mask int32[n,m], tgt f32[n,m,3],
  grad f32[n,m,3])``, ``sync()``, ``step(iteration) -> (uint8[n,m,3],
  float32[3])``.

Inputs are copied at ``reset`` (the caller may reuse its arrays); ``step``
continues from the previous state and returns fresh arrays.  Extra methods
hand device buffers over without host copies (``reset_tensors`` /
``step_tensors``, torch CUDA tensors) and expose the unclipped FP32 state
(``state()``).
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import FPIE_FP32, FPIE_MIXED_BF16, FPIE_MIXED_FP16

PRECISIONS = {"fp32": FPIE_FP32, "fp16": FPIE_MIXED_FP16, "bf16": FPIE_MIXED_BF16}


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _as(a, dtype, shape=None, name="array") -> np.ndarray:
    out = np.ascontiguousarray(np.asarray(a), dtype=dtype)
    if shape is not None:
        if out.ndim != len(shape) or any(s is not None and d != s for d, s in zip(out.shape, shape)):
            raise _abi.FpieArgumentError(f"{name} has shape {out.shape}, expected {shape}")
    return out


def _image_args(src, mask, tgt, gradient):
    """Pointers, shapes and codes for the *_reset_images calls (numpy or CUDA tensors)."""
    mode = {"src": 0, "avg": 1, "max": 2}.get(gradient)
    if mode is None:
        raise _abi.FpieArgumentError(f"unknown gradient mode {gradient!r}")
    on_dev = bool(getattr(src, "is_cuda", False))
    if on_dev:
        keep = (src, mask, tgt)
        ptrs = [_tensor_ptr(a, "uint8", n) for a, n in zip(keep, ("src", "mask", "tgt"))]
        shapes = [tuple(a.shape) for a in keep]
    else:
        keep = tuple(np.ascontiguousarray(a, dtype=np.uint8) for a in (src, mask, tgt))
        ptrs = [_ptr(a) for a in keep]
        shapes = [a.shape for a in keep]
    (sh, sw, sc), msh, (th, tw, tc) = shapes
    if sc != 3 or tc != 3 or len(msh) not in (2, 3):
        raise _abi.FpieArgumentError("src/tgt must be HxWx3 and the mask HxW or HxWx3")
    mch = 1 if len(msh) == 2 else msh[2]
    args = (ptrs[0], sh, sw, ptrs[1], msh[0], msh[1], mch, ptrs[2], th, tw)
    return keep, args, mode, on_dev


def _tensor_ptr(t, dtype_name: str, name: str) -> int:
    if not t.is_cuda:
        raise _abi.FpieArgumentError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise _abi.FpieArgumentError(f"{name} must be contiguous")
    if str(t.dtype) != f"torch.{dtype_name}":
        raise _abi.FpieArgumentError(f"{name} must be {dtype_name}, got {t.dtype}")
    return t.data_ptr()


class _Solver:
    _kind = ""

    def __init__(self) -> None:
        self._h = ctypes.c_void_p()
        self._lib = _abi.lib()

    def _create(self, fn: str, *args) -> None:
        _abi.call(fn, *args, ctypes.byref(self._h))

    def __del__(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._lib.fpie_destroy(h)
            except Exception:
                pass
            h.value = None

    def close(self) -> None:
        """Free device memory now instead of at garbage collection."""
        self.__del__()

    def sync(self) -> None:
        """Wait for the solver's queued device work (a no-op in the reference)."""
        _abi.call("fpie_sync", self._h)

    def set_stream(self, stream: int) -> None:
        """Enqueue later work on a cudaStream_t, e.g. torch's ``.cuda_stream``
        (0 is the legacy default stream, torch's default)."""
        _abi.call("fpie_set_stream", self._h, ctypes.c_void_p(int(stream)))

    def set_precision(self, precision: str) -> None:
        """'fp32' (default), or the mixed forms 'fp16' / 'bf16'."""
        if precision not in PRECISIONS:
            raise _abi.FpieArgumentError(f"unknown precision {precision!r}")
        _abi.call("fpie_set_precision", self._h, PRECISIONS[precision])

    def sweeps(self, iteration: int) -> None:
        """Enqueue sweeps only (no residual, no image)."""
        _abi.call("fpie_sweeps", self._h, int(iteration))

    @property
    def launches(self) -> int:
        c = ctypes.c_longlong(0)
        _abi.call("fpie_launch_count", self._h, ctypes.byref(c))
        return c.value


def raster_layout(A: np.ndarray):
    """Placement of a 4-neighbour raster equation system on a grid (host only).

    Returns (pos int32[N], (n, m)) -- pos[i] = row * m + col of unknown i,
    pos[0] = -1 -- or None when A is not a raster stencil."""
    A = _as(A, np.int32, (None, 4), "A")
    pos = np.empty(A.shape[0], np.int32)
    n, m = ctypes.c_int(0), ctypes.c_int(0)
    rc = _abi.lib().fpie_equ_raster_layout(A.shape[0], _ptr(A), _ptr(pos), ctypes.byref(n),
                                           ctypes.byref(m))
    if rc != 0:
        return None
    return pos, (n.value, m.value)


class EquSolver(_Solver):
    """Jacobi on relabelled unknowns (fpie/core/base_solver.h:12-75).

    order "jacobi" (default): the numpy EquSolver's iteration and row-major
    partition.  order "red_black": the reference's OpenMP EquSolver
    (fpie/core/openmp/equ.cc): partition numbers odd row+col cells first,
    then even ones, and each sweep updates the two colours in turn, in place.
    """

    ORDERS = {"jacobi": 0, "red_black": 1}

    def __init__(self, block_size: int = 1024, order: str = "jacobi") -> None:
        super().__init__()
        self._create("fpie_equ_create", int(block_size))
        self.N = 0
        if order != "jacobi":
            self.set_order(order)

    def set_order(self, order: str) -> None:
        """Iteration order; a change discards the loaded system."""
        if order not in self.ORDERS:
            raise ValueError(f"order must be one of {sorted(self.ORDERS)}")
        _abi.call("fpie_equ_set_order", self._h, self.ORDERS[order])

    @property
    def order(self) -> str:
        o, mid = ctypes.c_int(0), ctypes.c_int(0)
        _abi.call("fpie_equ_order", self._h, ctypes.byref(o), ctypes.byref(mid))
        return {v: k for k, v in self.ORDERS.items()}[o.value]

    @property
    def n_mid(self) -> int:
        """First even id of the last red-black partition (0 if none)."""
        o, mid = ctypes.c_int(0), ctypes.c_int(0)
        _abi.call("fpie_equ_order", self._h, ctypes.byref(o), ctypes.byref(mid))
        return mid.value

    def partition(self, mask: np.ndarray) -> np.ndarray:
        m = _as(mask, np.int32, (None, None), "mask")
        ids = np.empty(m.shape, np.int32)
        _abi.call("fpie_equ_partition", self._h, _ptr(m), m.shape[0], m.shape[1], _ptr(ids))
        return ids

    def reset(self, N: int, A: np.ndarray, X: np.ndarray, B: np.ndarray,
              placement: tuple[np.ndarray, int, int] | None = None) -> None:
        """placement: optional (pos int32[N], n, m), unknown i at crop pixel
        pos[i] = row * m + col -- checked on the device instead of searched
        for on the host (fpie_equ_reset_placed)."""
        N = int(N)
        A = _as(A, np.int32, (N, 4), "A")
        X = _as(X, np.float32, (N, 3), "X")
        B = _as(B, np.float32, (N, 3), "B")
        if placement is None:
            _abi.call("fpie_equ_reset", self._h, N, _ptr(A), _ptr(X), _ptr(B))
        else:
            pos, n, m = placement
            pos = _as(pos, np.int32, (N,), "pos")
            _abi.call("fpie_equ_reset_placed", self._h, N, _ptr(A), _ptr(X), _ptr(B), _ptr(pos),
                      int(n), int(m))
        self.N = N

    def step(self, iteration: int) -> tuple[np.ndarray, np.ndarray]:
        x = np.empty((self.N, 3), np.uint8)
        err = np.empty(3, np.float32)
        _abi.call("fpie_equ_step", self._h, int(iteration), _ptr(x), _ptr(err))
        return x, err

    def reset_images(self, src, mask, tgt, mask_on_src: tuple[int, int],
                     mask_on_tgt: tuple[int, int], gradient: str = "max"):
        """Build ids/A/X/B on the GPU from uint8 images (EquProcessor.reset semantics).

        Returns (N, crop box on the target, (rows, cols) target index of unknowns 1..N-1).
        """
        keep, args, mode, on_dev = _image_args(src, mask, tgt, gradient)
        box = (ctypes.c_int * 4)()
        n_out = ctypes.c_int(0)
        _abi.call("fpie_equ_reset_images", self._h, *args, int(mask_on_src[0]), int(mask_on_src[1]),
                  int(mask_on_tgt[0]), int(mask_on_tgt[1]), mode, 1 if on_dev else 0, box,
                  ctypes.byref(n_out))
        del keep
        self.N = n_out.value
        rows = np.empty(self.N - 1, np.int32)
        cols = np.empty(self.N - 1, np.int32)
        if self.N > 1:
            _abi.call("fpie_equ_get_index", self._h, _ptr(rows), _ptr(cols))
        return self.N, tuple(box), (rows.astype(np.int64), cols.astype(np.int64))

    def set_kernel(self, name: str) -> None:
        """"auto" (grid kernels for 4-neighbour raster systems, else gather),
        "gather", or a grid kernel name; applies from the next reset."""
        _abi.call("fpie_equ_set_kernel", self._h, name.encode())

    @property
    def kernel(self) -> str:
        """"gather" or "grid:<grid kernel>"."""
        buf = ctypes.create_string_buffer(64)
        _abi.call("fpie_equ_kernel", self._h, buf, 64)
        return buf.value.decode()

    def set_spin_limit(self, spins: int) -> None:
        """Bounded-wait limit of the grid kernels used in grid placement."""
        _abi.call("fpie_equ_set_spin_limit", self._h, ctypes.c_longlong(int(spins)))

    def inputs(self) -> tuple[np.ndarray, np.ndarray]:
        """(A int32[N,4], B float32[N,3]) as the solver holds them."""
        A = np.empty((self.N, 4), np.int32)
        B = np.empty((self.N, 3), np.float32)
        _abi.call("fpie_equ_get_inputs", self._h, _ptr(A), _ptr(B))
        return A, B

    def state(self) -> np.ndarray:
        out = np.empty((self.N, 3), np.float32)
        _abi.call("fpie_get_state", self._h, _ptr(out))
        return out

    def reset_tensors(self, N: int, A, X, B) -> None:
        """reset() from torch CUDA tensors (int32[N,4], float32[N,3] x2)."""
        _abi.call("fpie_equ_reset_device", self._h, int(N), _tensor_ptr(A, "int32", "A"),
                  _tensor_ptr(X, "float32", "X"), _tensor_ptr(B, "float32", "B"))
        self.N = int(N)

    def step_tensors(self, iteration: int, x=None, err=None) -> None:
        """Enqueue step(); results into torch CUDA tensors uint8[N,3] / float32[3]."""
        _abi.call("fpie_equ_step_device", self._h, int(iteration),
                  _tensor_ptr(x, "uint8", "x") if x is not None else None,
                  _tensor_ptr(err, "float32", "err") if err is not None else None)


class GridSolver(_Solver):
    """Jacobi on the cropped image grid (fpie/core/base_solver.h:77-152)."""

    def __init__(self, grid_x: int = 8, grid_y: int = 8) -> None:
        super().__init__()
        self._create("fpie_grid_create", int(grid_x), int(grid_y))
        self.grid_x, self.grid_y = int(grid_x), int(grid_y)
        self.N = 0
        self.shape = (0, 0)

    def reset(self, N: int, mask: np.ndarray, tgt: np.ndarray, grad: np.ndarray) -> None:
        m = _as(mask, np.int32, (None, None), "mask")
        n_, m_ = m.shape
        t = _as(tgt, np.float32, (n_, m_, 3), "tgt")
        g = _as(grad, np.float32, (n_, m_, 3), "grad")
        _abi.call("fpie_grid_reset", self._h, int(N), n_, m_, _ptr(m), _ptr(t), _ptr(g))
        self.N = int(N)
        self.shape = (n_, m_)

    def step(self, iteration: int) -> tuple[np.ndarray, np.ndarray]:
        img = np.empty((*self.shape, 3), np.uint8)
        err = np.empty(3, np.float32)
        _abi.call("fpie_grid_step", self._h, int(iteration), _ptr(img), _ptr(err))
        return img, err

    def set_kernel(self, name: str) -> None:
        """Pin the sweep kernel ("auto", "sweep1", or a variant like "p16w8k16")."""
        _abi.call("fpie_grid_set_kernel", self._h, name.encode())

    def set_spin_limit(self, spins: int) -> None:
        """Polls a flow-kernel neighbourhood wait, or a TMA-kernel copy wait,
        may take before the step fails with FpieTimeoutError."""
        _abi.call("fpie_grid_set_spin_limit", self._h, ctypes.c_longlong(int(spins)))

    @property
    def kernel(self) -> str:
        buf = ctypes.create_string_buffer(64)
        _abi.call("fpie_grid_kernel", self._h, buf, 64)
        return buf.value.decode()

    def reset_images(self, src, mask, tgt, mask_on_src: tuple[int, int],
                     mask_on_tgt: tuple[int, int], gradient: str = "max") -> tuple[int, int, int, int]:
        """Build the inputs on the GPU from uint8 images (GridProcessor.reset semantics).

        Arrays may be numpy (copied to the device) or torch CUDA uint8 tensors.
        Returns the crop on the target (row0, row1, col0, col1).
        """
        keep, args, mode, on_dev = _image_args(src, mask, tgt, gradient)
        box = (ctypes.c_int * 4)()
        _abi.call("fpie_grid_reset_images", self._h, *args, int(mask_on_src[0]), int(mask_on_src[1]),
                  int(mask_on_tgt[0]), int(mask_on_tgt[1]), mode, 1 if on_dev else 0, box)
        del keep
        self.shape = (box[1] - box[0], box[3] - box[2])
        self.N = self.shape[0] * self.shape[1]
        return tuple(box)

    def inputs(self) -> tuple[np.ndarray, np.ndarray]:
        """(mask int32[n,m], grad float32[n,m,3]) as the solver holds them."""
        mask = np.empty(self.shape, np.int32)
        grad = np.empty((*self.shape, 3), np.float32)
        _abi.call("fpie_grid_get_inputs", self._h, _ptr(mask), _ptr(grad))
        return mask, grad

    def residual_norms(self) -> tuple[np.ndarray, np.ndarray]:
        """(max |r| per channel, sum |r| per channel) of the current state, FP64."""
        out = np.empty(6, np.float64)
        _abi.call("fpie_residual_norms", self._h, _ptr(out))
        return out[:3].copy(), out[3:].copy()

    def solve(self, tol: float, max_sweeps: int, check_every: int = 256) -> int:
        """Sweep until every channel's max |residual| <= tol (or max_sweeps); return sweeps run."""
        done = ctypes.c_int(0)
        _abi.call("fpie_grid_solve", self._h, float(tol), int(max_sweeps), int(check_every),
                  ctypes.byref(done))
        return done.value

    def state(self) -> np.ndarray:
        out = np.empty((*self.shape, 3), np.float32)
        _abi.call("fpie_get_state", self._h, _ptr(out))
        return out

    def reset_tensors(self, mask, tgt, grad) -> None:
        """reset() from torch CUDA tensors int32[n,m], float32[n,m,3] x2."""
        n_, m_ = mask.shape
        _abi.call("fpie_grid_reset_device", self._h, int(n_), int(m_),
                  _tensor_ptr(mask, "int32", "mask"), _tensor_ptr(tgt, "float32", "tgt"),
                  _tensor_ptr(grad, "float32", "grad"))
        self.N = int(n_ * m_)
        self.shape = (int(n_), int(m_))

    def step_tensors(self, iteration: int, img=None, err=None) -> None:
        """Enqueue step(); results into torch CUDA tensors uint8[n,m,3] / float32[3]."""
        _abi.call("fpie_grid_step_device", self._h, int(iteration),
                  _tensor_ptr(img, "uint8", "img") if img is not None else None,
                  _tensor_ptr(err, "float32", "err") if err is not None else None)
