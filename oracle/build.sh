#!/usr/bin/env bash
# Builds the C restatement (test infrastructure) into oracle/lib/libb2g_oracle.so.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/lib"
gcc -O2 -std=c11 -fopenmp -fPIC -shared -Wall -Wno-unused-variable \
    "$here/b2g_oracle.c" -o "$here/lib/libb2g_oracle.so" -ldl -lm
