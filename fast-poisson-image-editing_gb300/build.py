"""Builds the backend's shared library ``_lib/libfpie_gb300.so`` with nvcc.

Every ``csrc/*.cu`` is compiled for sm_103a only (one ``-gencode``), in
parallel, then linked into one C-ABI library (CUDA runtime linked
statically).  A rebuild happens only when a source or header is newer than
the library.  ``ptxas -v`` output (registers, spills, shared memory) is kept
in ``_build/ptxas.log`` beside the objects.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
LIB_DIR = PKG / "_lib"
LIB = LIB_DIR / "libfpie_gb300.so"
OBJ_DIR = PKG / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
              "-Xptxas", "-v", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = pathlib.Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fpie_gb300")


def _sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[pathlib.Path]:
    return _sources() + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def needs_build() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    return any(p.stat().st_mtime > t for p in _deps())


def _compile(src: pathlib.Path) -> tuple[pathlib.Path, str]:
    obj = OBJ_DIR / (src.stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC),
           "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose: bool = False) -> pathlib.Path:
    """Compile and link the library if it is missing or stale; return its path."""
    if not force and not needs_build():
        return LIB
    OBJ_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=max(1, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    (OBJ_DIR / "ptxas.log").write_text("".join(log for _, log in results))
    tmp = LIB.with_suffix(f".so.{os.getpid()}.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *[str(o) for o, _ in results]]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
