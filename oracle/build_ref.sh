#!/usr/bin/env bash
# Builds the reference fpie's own CPU solver modules (core_gcc, core_openmp)
# and the device code of its CUDA solvers (cubins) from their sources under
# the reference tree ($FPIE_REFERENCE; by default the read-only copy this
# recipe was written against) into oracle/_ref/, for use as a checker and
# comparison arm only.  Needs pybind11 headers (pip package) and the reference tree;
# exits 0 without doing anything when either is missing (e.g. on a box that
# only carries this repository).
set -euo pipefail
REF=${FPIE_REFERENCE:-/root/reference}
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/fpie/core" ]; then
  echo "build_ref: no reference tree at $REF; skipping"
  exit 0
fi
PYBIND_INC=$(python3 -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || true)
if [ -z "$PYBIND_INC" ]; then
  echo "build_ref: pybind11 not importable; skipping"
  exit 0
fi
PY_INC=$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
SUFFIX=$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
mkdir -p "$OUT/fpie"
CXXFLAGS="-O3 -shared -fPIC -std=c++17 -I$PYBIND_INC -I$PY_INC -I$REF/fpie/core"
g++ $CXXFLAGS "$REF"/fpie/core/gcc/*.cc -o "$OUT/fpie/core_gcc$SUFFIX" &
g++ $CXXFLAGS -fopenmp "$REF"/fpie/core/openmp/*.cc -o "$OUT/fpie/core_openmp$SUFFIX" &
# The reference's CUDA solvers: device code only, one cubin per source file,
# for sm_103a (the reference's CMake build uses -O3 and no arch flags of its
# own).  oracle/ref_cuda.py loads them with the driver API on the GPU.
NVCC=${CUDA_HOME:-/usr/local/cuda}/bin/nvcc
if [ -x "$NVCC" ]; then
  mkdir -p "$OUT/cuda"
  for f in grid equ; do
    "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 \
      -I"$PYBIND_INC" -I"$PY_INC" -I"$REF/fpie/core" -I"$REF/fpie/core/cuda" \
      "$REF/fpie/core/cuda/$f.cu" -o "$OUT/cuda/$f.sm_103a.cubin" &
  done
fi
wait
# The reference's pure-Python modules are not copied: the checker imports them
# from the reference tree and finds the compiled modules through fpie.__path__.
echo "build_ref: built $(ls "$OUT/fpie") $(ls "$OUT/cuda" 2>/dev/null)"
