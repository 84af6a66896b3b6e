#!/usr/bin/env bash
# Builds block2's own CPU DMRG (header-only) from a block2 source tree into
# oracle/_ref/.  TEST INFRASTRUCTURE ONLY: these binaries are the reference
# that generates golden fixtures and the CPU baseline; nothing of the product
# links or runs them.
#   oracle/build_ref.sh BLOCK2_SRC            dmrg_sweep_ref: block2's DMRG::solve on the
#                                             host cores (the sweep program built with
#                                             -DB2G_REFERENCE_ONLY: no GPU code at all)
#   oracle/build_ref.sh BLOCK2_SRC harness    also ref_harness (fixture dumps)
# BLOCK2_SRC defaults to $BLOCK2_SRC, then to the staged copy
# block2-preview_gb300/shim/_block2/src (see shim/stage_block2.py).
# BLAS/LAPACK: scipy's bundled LP64 OpenBLAS (shim/blas_defs.sh).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
root="$(dirname "$here")"
shim="$root/block2-preview_gb300/shim"
ref="${1:-${BLOCK2_SRC:-$shim/_block2/src}}"
[ -f "$ref/block2_core.hpp" ] || { echo "block2 sources not found at $ref" >&2; exit 3; }
mkdir -p "$here/_ref"
bash "$shim/build.sh" "$ref" cpu "$here/_ref/dmrg_sweep_ref"
if [ "${2:-}" = harness ]; then
  . "$shim/blas_defs.sh"
  g++ -std=c++17 -O2 -fopenmp $B2G_BLAS_DEFS -I"$ref" "$here/ref_harness.cpp" \
      -o "$here/_ref/ref_harness" "$B2G_BLAS" -Wl,-rpath,"$(dirname "$B2G_BLAS")" -lpthread
  echo "built $here/_ref/ref_harness"
fi
