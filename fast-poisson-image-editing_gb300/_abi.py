"""ctypes binding of the C ABI declared in include/fpie_gb300.h.

The library is loaded from the package's ``_lib`` directory.  There is no
fallback: if it is missing or cannot be loaded, every solver constructor
raises, naming the build step to run.
"""

from __future__ import annotations

import ctypes
import pathlib
import threading

_LIB_PATH = pathlib.Path(__file__).resolve().parent / "_lib" / "libfpie_gb300.so"
_lock = threading.Lock()
_lib: ctypes.CDLL | None = None

FPIE_OK, FPIE_ERR_ARG, FPIE_ERR_CUDA, FPIE_ERR_STATE, FPIE_ERR_TIMEOUT = range(5)
FPIE_FP32, FPIE_MIXED_FP16, FPIE_MIXED_BF16 = range(3)


class FpieError(RuntimeError):
    """A call into the native backend failed."""


class FpieArgumentError(FpieError, ValueError):
    """The native backend rejected an argument."""


class FpieTimeoutError(FpieError, TimeoutError):
    """A bounded device-side wait gave up."""


_P = ctypes.c_void_p
_I = ctypes.c_int
_PROTOS: dict[str, tuple] = {
    "fpie_version": ([], _I),
    "fpie_last_error": ([], ctypes.c_char_p),
    "fpie_device_count": ([ctypes.POINTER(_I)], _I),
    "fpie_equ_create": ([_I, ctypes.POINTER(_P)], _I),
    "fpie_equ_partition": ([_P, _P, _I, _I, _P], _I),
    "fpie_equ_set_order": ([_P, _I], _I),
    "fpie_equ_reset_placed": ([_P, _I, _P, _P, _P, _P, _I, _I], _I),
    "fpie_equ_order": ([_P, _P, _P], _I),
    "fpie_equ_reset": ([_P, _I, _P, _P, _P], _I),
    "fpie_equ_step": ([_P, _I, _P, _P], _I),
    "fpie_grid_create": ([_I, _I, ctypes.POINTER(_P)], _I),
    "fpie_grid_reset": ([_P, _I, _I, _I, _P, _P, _P], _I),
    "fpie_grid_step": ([_P, _I, _P, _P], _I),
    "fpie_sync": ([_P], _I),
    "fpie_destroy": ([_P], _I),
    "fpie_set_stream": ([_P, _P], _I),
    "fpie_set_precision": ([_P, _I], _I),
    "fpie_grid_reset_device": ([_P, _I, _I, _P, _P, _P], _I),
    "fpie_grid_step_device": ([_P, _I, _P, _P], _I),
    "fpie_equ_reset_device": ([_P, _I, _P, _P, _P], _I),
    "fpie_equ_step_device": ([_P, _I, _P, _P], _I),
    "fpie_sweeps": ([_P, _I], _I),
    "fpie_get_state": ([_P, _P], _I),
    "fpie_launch_count": ([_P, ctypes.POINTER(ctypes.c_longlong)], _I),
    "fpie_grid_set_kernel": ([_P, ctypes.c_char_p], _I),
    "fpie_grid_kernel": ([_P, ctypes.c_char_p, _I], _I),
    "fpie_grid_set_spin_limit": ([_P, ctypes.c_longlong], _I),
    "fpie_grid_step_noalloc": ([_I, _I, _P, _P, _P, _I, _P, _P, _P], _I),
    "fpie_residual_norms": ([_P, _P], _I),
    "fpie_grid_solve": ([_P, ctypes.c_double, _I, _I, ctypes.POINTER(_I)], _I),
    "fpie_grid_reset_images": ([_P, _P, _I, _I, _P, _I, _I, _I, _P, _I, _I, _I, _I, _I, _I, _I,
                                _I, _P], _I),
    "fpie_grid_get_inputs": ([_P, _P, _P], _I),
    "fpie_equ_reset_images": ([_P, _P, _I, _I, _P, _I, _I, _I, _P, _I, _I, _I, _I, _I, _I, _I,
                               _I, _P, ctypes.POINTER(_I)], _I),
    "fpie_equ_get_index": ([_P, _P, _P], _I),
    "fpie_equ_get_inputs": ([_P, _P, _P], _I),
    "fpie_equ_set_kernel": ([_P, ctypes.c_char_p], _I),
    "fpie_equ_kernel": ([_P, ctypes.c_char_p, _I], _I),
    "fpie_equ_set_spin_limit": ([_P, ctypes.c_longlong], _I),
    "fpie_equ_raster_layout": ([_I, _P, _P, _P, _P], _I),
    "fpie_batch_create": ([ctypes.c_double, ctypes.POINTER(_P)], _I),
    "fpie_batch_destroy": ([_P], _I),
    "fpie_batch_job_bytes": ([_I, _I, ctypes.POINTER(ctypes.c_double)], _I),
    "fpie_batch_job_bytes_for": ([_P, _I, _I, ctypes.POINTER(ctypes.c_double)], _I),
    "fpie_batch_set_precision": ([_P, _I], _I),
    "fpie_batch_add": ([_P, _I, _I, _P, _P, _P, _I, ctypes.POINTER(_I)], _I),
    "fpie_batch_run": ([_P, _I], _I),
    "fpie_batch_progress": ([_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "fpie_batch_result": ([_P, _I, _P, _P], _I),
    "fpie_batch_state": ([_P, _I, _P], _I),
    "fpie_batch_remove": ([_P, _I], _I),
    "fpie_batch_norms": ([_P, _P, _I, _P], _I),
    "fpie_batch_memory": ([_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)], _I),
    "fpie_batch_set_kernel": ([_P, ctypes.c_char_p], _I),
    "fpie_batch_kernel": ([_P, ctypes.c_char_p, _I], _I),
    "fpie_batch_set_spin_limit": ([_P, ctypes.c_longlong], _I),
    "fpie_batch_launch_count": ([_P, ctypes.POINTER(ctypes.c_longlong)], _I),
    "fpie_batch_add_images": ([_P, _P, _I, _I, _P, _I, _I, _I, _P, _I, _I, _I, _I, _I, _I, _I,
                               _I, ctypes.POINTER(_I), _P], _I),
    "fpie_batch_run_async": ([_P, _I], _I),
    "fpie_batch_wait": ([_P], _I),
    "fpie_batch_norms_async": ([_P, _P, _I], _I),
    "fpie_batch_norms_wait": ([_P, _P], _I),
    "fpie_probe_fp32_rate": ([_P, _I, _I, ctypes.POINTER(ctypes.c_double)], _I),
}


PROBE_KINDS = {"fadd2": 0, "fmul2": 1, "ffma2": 2, "fadd": 3}


def fp32_rate(kind: str = "fadd2", iters: int = 20000, stream: int = 0) -> float:
    """FP32 operations per second of one kind of instruction on the current
    device (one operation per value; see fpie_probe_fp32_rate)."""
    out = ctypes.c_double(0)
    call("fpie_probe_fp32_rate", _P(stream), PROBE_KINDS[kind], int(iters), ctypes.byref(out))
    return out.value


def library_path() -> pathlib.Path:
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    """Load the native library once (raises if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                raise FpieError(
                    f"native library {_LIB_PATH} is missing; build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` "
                    "(or fpie_gb300.build.build())")
            handle = ctypes.CDLL(str(_LIB_PATH))
            for name, (args, res) in _PROTOS.items():
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = res
            _lib = handle
    return _lib


def check(rc: int) -> None:
    """Raise the matching exception for a non-zero status."""
    if rc == FPIE_OK:
        return
    msg = (lib().fpie_last_error() or b"").decode(errors="replace") or f"status {rc}"
    if rc == FPIE_ERR_ARG:
        raise FpieArgumentError(msg)
    if rc == FPIE_ERR_TIMEOUT:
        raise FpieTimeoutError(msg)
    raise FpieError(msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def device_count() -> int:
    n = _I(0)
    call("fpie_device_count", ctypes.byref(n))
    return n.value
