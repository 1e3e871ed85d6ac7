#!/bin/sh
# Builds oracle/_ref/libref.so: the reference's header-only tricubic spline evaluator
# compiled in place from the reference's source tree (and libref_delayed.so, libref_bspline.so
# for its delayed-update engine and its spline coefficient solve) (first argument, else
# $QMCPACK_REFERENCE_DIR, else /root/reference), with a minimal config.h shim.
# Test infrastructure only; skipped when the reference sources are absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-${QMCPACK_REFERENCE_DIR:-/root/reference}}
[ -d "$REF/src/spline2" ] || { echo "reference sources not found at $REF; skipping oracle/_ref"; exit 0; }
mkdir -p "$HERE/_ref"
${CXX:-g++} -O2 -std=c++17 -fPIC -shared -Drestrict=__restrict__ \
  -I "$HERE/ref_shim" -I "$REF/src" -I "$REF/src/einspline" -I "$REF/src/Platforms" \
  "$HERE/ref_spline.cpp" -o "$HERE/_ref/libref.so"
# the reference's CPU delayed-update engine, its BLAS calls forwarded to scipy's OpenBLAS
BLASDIR=$(${PYTHON:-python3} -c "import scipy, os; print(os.path.realpath(os.path.join(os.path.dirname(scipy.__file__), '..', 'scipy.libs')))" 2>/dev/null || true)
BLAS=$(ls "$BLASDIR"/libscipy_openblas*.so 2>/dev/null | head -1)
if [ -n "$BLAS" ]; then
  ${CXX:-g++} -O2 -std=c++17 -fPIC -shared -fopenmp -Drestrict=__restrict__ \
    -I "$HERE/ref_shim" -I "$REF/src" -I "$REF/src/Platforms" -I "$REF/src/Containers" -I "$REF/src/einspline" \
    -I "$REF/src/Utilities" -I "$REF/src/Concurrency" \
    "$HERE/ref_delayed.cpp" -o "$HERE/_ref/libref_delayed.so" "$BLAS" -Wl,-rpath,"$BLASDIR" -Wl,--no-undefined
fi
# the reference's einspline coefficient solve (periodic cubic B-spline interpolation)
${CC:-gcc} -O2 -std=gnu99 -fPIC -shared -Drestrict=__restrict__ -w \
  -I "$HERE/ref_shim" -I "$REF/src/einspline" -I "$REF/src" \
  "$HERE/ref_bspline.c" "$REF/src/einspline/bspline_create.c" "$REF/src/einspline/multi_bspline_create.c" \
  -o "$HERE/_ref/libref_bspline.so"
echo "built $HERE/_ref"
