#!/usr/bin/env bash
# Builds the reference fpie's own CPU solver modules (core_gcc, core_openmp)
# from their sources under /root/reference into oracle/_ref/, for use as a
# checker only.  Needs pybind11 headers (pip package) and the reference tree;
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
wait
# The reference's pure-Python modules are not copied: the checker imports them
# from the reference tree and finds the compiled modules through fpie.__path__.
echo "build_ref: built $(ls "$OUT/fpie")"
