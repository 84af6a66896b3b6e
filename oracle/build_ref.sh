#!/usr/bin/env bash
# Builds the reference's own CPU DMRG (block2, header-only) with ref_harness.cpp
# into oracle/_ref/ref_harness.  TEST INFRASTRUCTURE ONLY: the binary is the
# oracle that generates golden fixtures; it is never part of the product.
# Usage: oracle/build_ref.sh [REFERENCE_SRC_DIR]   (default: /root/reference/src)
# BLAS/LAPACK: scipy's bundled LP64 OpenBLAS (symbols prefixed scipy_).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${1:-/root/reference/src}"
[ -f "$ref/block2_core.hpp" ] || { echo "reference sources not found at $ref" >&2; exit 3; }
blasdir="$(python3 -c 'import scipy, os; print(os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs"))')"
blas="$(ls "$blasdir"/libscipy_openblas*.so | head -1)"
defs=""
for s in caxpy ccopy cdotc cgeev cgelqf cgels cgemm cgemv cgeqp3 cgeqrf cgesv cgesvd cgetrf cgetri cheev chegv clacpy cscal csscal cunglq cungqr \
         daxpy dcopy ddot dgeev dgelqf dgels dgemm dgemv dgeqp3 dgeqrf dgesv dgesvd dgetrf dgetri dlacpy dnrm2 dorglq dorgqr dscal dsyev dsygv dznrm2 \
         saxpy scnrm2 scopy sdot sgeev sgegv sgelqf sgels sgemm sgemv sgeqp3 sgeqrf sgesv sgesvd sgetrf sgetri slacpy snrm2 sorglq sorgqr sscal ssyev ssygv \
         zaxpy zcopy zdotc zdscal zgeev zgelqf zgels zgemm zgemv zgeqp3 zgeqrf zgesv zgesvd zgetrf zgetri zheev zhegv zlacpy zscal zunglq zungqr; do
  defs="$defs -D${s}_=scipy_${s}_"
done
mkdir -p "$here/_ref"
g++ -std=c++17 -O2 -fopenmp -D_F77UNDERSCORE $defs -I"$ref" "$here/ref_harness.cpp" \
    -o "$here/_ref/ref_harness" "$blas" -Wl,-rpath,"$(dirname "$blas")" -lpthread
echo "built $here/_ref/ref_harness"
