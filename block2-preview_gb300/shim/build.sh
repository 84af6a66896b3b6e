#!/usr/bin/env bash
# Builds the DMRG sweep program (dmrg_sweep.cpp) against block2's headers.
#   build.sh BLOCK2_SRC gpu OUT   block2 + the GB300 drop-in, links lib/libb2g.so
#   build.sh BLOCK2_SRC cpu OUT   block2's own CPU path only (-DB2G_REFERENCE_ONLY)
# BLOCK2_SRC is a block2 source tree's src/ directory (block2 is header-only).
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
pkg="$(dirname "$here")"
root="$(dirname "$pkg")"
src="$1"; mode="$2"; out="$3"
[ -f "$src/block2_core.hpp" ] || { echo "block2 headers not found at $src" >&2; exit 3; }
. "$here/blas_defs.sh"
mkdir -p "$(dirname "$out")"
flags="-std=c++17 -O2 -fopenmp $B2G_BLAS_DEFS -I$src"
if [ "$mode" = gpu ]; then
  g++ $flags -I"$root/include" -I"$here" "$here/dmrg_sweep.cpp" -o "$out.tmp" \
      "$B2G_BLAS" -L"$pkg/lib" -lb2g -Wl,-rpath,"$(dirname "$B2G_BLAS")" -Wl,-rpath,"$pkg/lib" -lpthread
else
  g++ $flags -DB2G_REFERENCE_ONLY "$here/dmrg_sweep.cpp" -o "$out.tmp" \
      "$B2G_BLAS" -Wl,-rpath,"$(dirname "$B2G_BLAS")" -lpthread
fi
mv "$out.tmp" "$out"
echo "built $out"
