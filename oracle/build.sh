#!/bin/sh
# Builds the oracle (test infrastructure) into oracle/_build/libether_oracle.so.
# -ffp-contract=off keeps every FP32 operation rounded separately, as the GPU kernels
# (compiled with --fmad=false, explicit fmaf) do.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-cc} -O2 -std=c11 -D_GNU_SOURCE -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared \
    -Wall -Wno-unused-function -o "$here/_build/libether_oracle.so" "$here/ether_oracle.c" "$here/learn_oracle.c" -lm
