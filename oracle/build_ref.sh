#!/bin/sh
# Build the reference's native library (common/math/wrapper/a.so) from the reference's own
# sources into oracle/_ref/a.so, with the recipe of the reference README (g++, C++17, the
# vendored Eigen 3.3.7).  VECTOR.h uses AVX intrinsics, so this builds on x86-64 only; the
# output is a checker used to pin the oracle and to generate golden fixtures, never product.
set -e
REF=${FASTIPC_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
W=$REF/common/math/wrapper
[ -f "$W/wrapper.cpp" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -mavx2 -mfma -fPIC -shared -w -I "$W" "$W/wrapper.cpp" "$W/EVCTCD/CTCD.cpp" -o "$HERE/_ref/a.so"
echo "built $HERE/_ref/a.so"
