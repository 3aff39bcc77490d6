#!/usr/bin/env bash
# Builds the reference implementation (ssciwr/hammingdist 1.4.0) from its own
# sources, where they lie, into oracle/_ref/ as a Python extension module named
# `hammingdist`. Test infrastructure only: the result is the oracle that pins
# the C restatement (oracle/hd_oracle.c) and generates tests/golden/ fixtures.
#
# Missing third-party pieces of the reference (empty git submodules) are
# replaced by: pybind11 from pip, fmt's header-only build shipped inside the
# torch wheel, and oracle/shim/cpuinfo_x86.h for cpu_features.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF=${1:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -d "$REF/src" ]; then
  echo "reference sources not found at $REF" >&2
  exit 1
fi
PY=${PYTHON:-python3}
PYINC=$($PY -c 'import sysconfig; print(sysconfig.get_paths()["include"])')
PYBIND=$($PY -c 'import pybind11; print(pybind11.get_include())')
TORCHINC=$($PY -c 'import os, torch; print(os.path.join(os.path.dirname(torch.__file__), "include"))')
SUFFIX=$($PY -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')
ARCH=$(uname -m)

CXX=${CXX:-g++}
DEFS="-DHAMMING_WITH_OPENMP -DFMT_HEADER_ONLY"
SIMD_SRCS=()
if [ "$ARCH" = "x86_64" ]; then
  DEFS="$DEFS -DHAMMING_WITH_SSE2 -DHAMMING_WITH_AVX2 -DHAMMING_WITH_AVX512"
else
  DEFS="$DEFS -DHAMMING_WITH_NEON"
fi
# fmt is taken from torch's include dir only (pybind11 from pip comes first).
INCS="-I$REF/include -I$HERE/shim -I$PYBIND -I$PYINC -isystem $TORCHINC"
CXXFLAGS="-O3 -std=c++17 -fPIC -fopenmp $DEFS $INCS"

OBJ="$OUT/obj"
mkdir -p "$OBJ"
$CXX $CXXFLAGS -c "$REF/src/hamming.cc" -o "$OBJ/hamming.o" &
$CXX $CXXFLAGS -c "$REF/src/hamming_impl.cc" -o "$OBJ/hamming_impl.o" &
$CXX $CXXFLAGS -c "$REF/python/hammingdist.cc" -o "$OBJ/hammingdist.o" &
if [ "$ARCH" = "x86_64" ]; then
  $CXX $CXXFLAGS -msse2 -c "$REF/src/distance_sse2.cc" -o "$OBJ/distance_sse2.o" &
  $CXX $CXXFLAGS -mavx2 -c "$REF/src/distance_avx2.cc" -o "$OBJ/distance_avx2.o" &
  $CXX $CXXFLAGS -mavx512bw -c "$REF/src/distance_avx512.cc" -o "$OBJ/distance_avx512.o" &
else
  $CXX $CXXFLAGS -c "$REF/src/distance_neon.cc" -o "$OBJ/distance_neon.o" &
fi
wait
$CXX -shared -fopenmp "$OBJ"/*.o -o "$OUT/hammingdist$SUFFIX"
echo "built $OUT/hammingdist$SUFFIX"
