"""ORACLE (benchmark/test infrastructure only): the reference's own CUDA
solvers run on this GPU, as the comparison arm beside the GB300 backend.

The kernels are the reference's, unchanged: ``oracle/build_ref.sh`` compiles
its ``fpie/core/cuda/grid.cu`` and ``fpie/core/cuda/equ.cu`` (device code
only, ``nvcc -cubin`` for sm_103a) into ``oracle/_ref/cuda/`` where the
reference tree is present, and the cubins travel with the repository.  The
host side is ``oracle/ref_cuda_host.c``, a restatement of the reference's
``step`` loops (``fpie/core/cuda/grid.cu:133-153``, ``fpie/core/cuda/equ.cu:189-211``) over
the CUDA driver API, compiled here with gcc on first use.

The reference's CUDA kernels update in place (each sweep reads neighbours
that other threads of the same launch may already have updated), so they
are not Jacobi: results differ from run to run and converge faster per
sweep than Jacobi.  They are compared with the GB300 backend on time to the
same error against the converged solution and to the same residual sum,
never bit for bit.

Only tests, bench.py's baseline legs and the profiling entry point at the
end of this file (python -m oracle.ref_cuda) use this module.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

_HERE = pathlib.Path(__file__).resolve().parent
_SRC = _HERE / "ref_cuda_host.c"
_LIB = _HERE / "_build" / "libref_cuda_host.so"
CUBIN_DIR = _HERE / "_ref" / "cuda"
GRID_CUBIN = CUBIN_DIR / "grid.sm_103a.cubin"
EQU_CUBIN = CUBIN_DIR / "equ.sm_103a.cubin"
_lib = None


def cuda_home() -> pathlib.Path:
    return pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def unavailable_reason() -> str | None:
    """None when the reference's kernels can run here, else why not."""
    for p in (GRID_CUBIN, EQU_CUBIN):
        if not p.is_file():
            return (f"{p.relative_to(_HERE.parent)} missing: the reference's CUDA sources are "
                    "compiled by oracle/build_ref.sh where the reference tree is present")
    if not (cuda_home() / "include" / "cuda.h").is_file():
        return "cuda.h not found under CUDA_HOME"
    return None


def build(force: bool = False) -> pathlib.Path:
    if force or not _LIB.exists() or _LIB.stat().st_mtime < _SRC.stat().st_mtime:
        _LIB.parent.mkdir(parents=True, exist_ok=True)
        tmp = _LIB.with_suffix(f".{os.getpid()}.tmp")
        home = cuda_home()
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", f"-I{home / 'include'}", str(_SRC),
                        "-o", str(tmp), f"-L{home / 'lib64' / 'stubs'}", f"-L{home / 'lib64'}",
                        "-lcuda"], check=True)
        os.replace(tmp, _LIB)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        why = unavailable_reason()
        if why:
            raise RuntimeError(why)
        L = ctypes.CDLL(str(build()))
        i, p, u64 = ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64
        L.refcuda_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.refcuda_grid_sweeps.argtypes = [i, i, u64, u64, u64, i, i, i, p]
        L.refcuda_grid_step.argtypes = [i, i, u64, u64, u64, u64, u64, u64, i, i, i, p, p, p]
        L.refcuda_equ_sweeps.argtypes = [i, u64, u64, u64, i, i, p]
        L.refcuda_equ_step.argtypes = [i, u64, u64, u64, u64, u64, u64, i, i, p, p, p]
        _lib = L
    return _lib


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"reference CUDA {what} failed: CUresult {rc}")


def _load() -> None:
    import torch

    torch.cuda.init()
    torch.zeros(1, device="cuda")  # makes the primary context current on this thread
    _check(lib().refcuda_load(str(GRID_CUBIN).encode(), str(EQU_CUBIN).encode()), "module load")


class RefCudaGrid:
    """The reference's CudaGridSolver (fpie/core/cuda/grid.cu) on the current
    CUDA device: reset copies mask / tgt / grad in (post_reset, fpie/core/cuda/grid.cu:33-52),
    step(n) is the reference's step."""

    def __init__(self, grid_x: int = 8, grid_y: int = 8):
        self.grid_x, self.grid_y = int(grid_x), int(grid_y)
        _load()

    def reset(self, mask, tgt, grad) -> None:
        import torch

        mask = np.ascontiguousarray(mask, dtype=np.int32)
        n, m = mask.shape
        # The in-place kernel reads the four neighbours of every masked pixel
        # without bounds checks; the processor's frame clear keeps the crop's
        # outer ring unmasked, which this restates as a precondition.
        if mask[0].any() or mask[-1].any() or mask[:, 0].any() or mask[:, -1].any():
            raise ValueError("masked pixel on the crop's outer ring")
        self.n, self.m = n, m
        dev = torch.device("cuda", torch.cuda.current_device())
        self.mask = torch.from_numpy(mask).to(dev)
        self.tgt = torch.from_numpy(np.ascontiguousarray(tgt, dtype=np.float32)).to(dev)
        self.grad = torch.from_numpy(np.ascontiguousarray(grad, dtype=np.float32)).to(dev)
        assert self.tgt.shape == (n, m, 3) and self.grad.shape == (n, m, 3)
        self.tmp = torch.zeros((n, m, 3), dtype=torch.float32, device=dev)
        self.img = torch.empty((n, m, 3), dtype=torch.uint8, device=dev)
        self.err = torch.zeros(4, dtype=torch.float32, device=dev)
        self.img_host = np.empty((n, m, 3), np.uint8)
        self.err_host = np.zeros(3, np.float32)
        torch.cuda.synchronize()

    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def sweeps(self, iters: int) -> None:
        """Sweep launches only (no synchronize), on torch's current stream."""
        _check(lib().refcuda_grid_sweeps(self.n, self.m, self.mask.data_ptr(), self.tgt.data_ptr(),
                                         self.grad.data_ptr(), self.grid_x, self.grid_y, int(iters),
                                         self._stream()), "grid sweeps")

    def step(self, iters: int):
        _check(lib().refcuda_grid_step(
            self.n, self.m, self.mask.data_ptr(), self.tgt.data_ptr(), self.grad.data_ptr(),
            self.tmp.data_ptr(), self.img.data_ptr(), self.err.data_ptr(), self.grid_x, self.grid_y,
            int(iters), self._stream(), self.err_host.ctypes.data, self.img_host.ctypes.data),
            "grid step")
        return self.img_host.copy(), self.err_host.copy()

    def state(self) -> np.ndarray:
        return self.tgt.cpu().numpy()


class RefCudaEqu:
    """The reference's CudaEquSolver (fpie/core/cuda/equ.cu): reset copies
    A / X / B in (post_reset, fpie/core/cuda/equ.cu:56-74), step(n) is the reference's step."""

    def __init__(self, block_size: int = 1024):
        self.block_size = int(block_size)
        _load()

    def reset(self, N: int, A, X, B) -> None:
        import torch

        A = np.ascontiguousarray(A, dtype=np.int32)
        if A.shape != (N, 4) or A.min() < 0 or A.max() >= N:
            raise ValueError("A must be N x 4 with entries in [0, N)")
        self.N = int(N)
        dev = torch.device("cuda", torch.cuda.current_device())
        self.A = torch.from_numpy(A).to(dev)
        self.X = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
        self.B = torch.from_numpy(np.ascontiguousarray(B, dtype=np.float32)).to(dev)
        self.tmp = torch.zeros((N, 3), dtype=torch.float32, device=dev)
        self.img = torch.empty((N, 3), dtype=torch.uint8, device=dev)
        self.err = torch.zeros(4, dtype=torch.float32, device=dev)
        self.img_host = np.empty((N, 3), np.uint8)
        self.err_host = np.zeros(3, np.float32)
        torch.cuda.synchronize()

    def _stream(self):
        import torch

        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def sweeps(self, iters: int) -> None:
        _check(lib().refcuda_equ_sweeps(self.N, self.A.data_ptr(), self.B.data_ptr(), self.X.data_ptr(),
                                        self.block_size, int(iters), self._stream()), "equ sweeps")

    def step(self, iters: int):
        _check(lib().refcuda_equ_step(
            self.N, self.A.data_ptr(), self.B.data_ptr(), self.X.data_ptr(), self.tmp.data_ptr(),
            self.img.data_ptr(), self.err.data_ptr(), self.block_size, int(iters), self._stream(),
            self.err_host.ctypes.data, self.img_host.ctypes.data), "equ step")
        return self.img_host.copy(), self.err_host.copy()

    def state(self) -> np.ndarray:
        return self.X.cpu().numpy()


def _main() -> None:
    """Runs the reference's CUDA GridSolver (and EquSolver) steps on the
    square800 workload, for timing and profiling the reference's kernels:
    python -m oracle.ref_cuda --sweeps N [--equ]."""
    import argparse
    import sys
    import time

    root = pathlib.Path(__file__).resolve().parent.parent
    sys.path.insert(0, str(root))
    from fpie_gb300 import backend, prep, workloads

    ap = argparse.ArgumentParser()
    ap.add_argument("--sweeps", type=int, default=50)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--equ", action="store_true", help="the EquSolver instead of the GridSolver")
    a = ap.parse_args()
    pb = workloads.square800(a.sweeps)
    if a.equ:
        sysm = prep.equ_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt, pb.gradient,
                               backend.EquSolver(1024).partition)
        s = RefCudaEqu(1024)
        reset = lambda: s.reset(sysm.N, sysm.A, sysm.X, sysm.B)  # noqa: E731
    else:
        mc, t, g, _ = prep.grid_inputs(pb.src, pb.mask, pb.tgt, pb.mask_on_src, pb.mask_on_tgt,
                                       pb.gradient)
        s = RefCudaGrid(8, 8)
        reset = lambda: s.reset(mc, t, g)  # noqa: E731
    for k in range(a.steps):
        reset()
        t0 = time.perf_counter()
        _, err = s.step(a.sweeps)
        dt = time.perf_counter() - t0
        print(f"step {k}: {a.sweeps} sweeps in {dt * 1e3:.2f} ms ({dt / a.sweeps * 1e6:.2f} us/sweep), "
              f"err {err.tolist()}")


if __name__ == "__main__":
    _main()
