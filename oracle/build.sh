#!/bin/sh
# Builds the oracle (test infrastructure) into oracle/_build/:
#   libether_oracle.so        the checker: -ffp-contract=off keeps every FP32 operation
#                             rounded separately, as the GPU kernels (compiled with
#                             --fmad=false, explicit fmaf) do;
#   libether_oracle_timed.so  the CPU baseline that bench.py times: the same source with the
#                             reference's own optimisation flags (make.sys: -O3 -fopenmp
#                             -funroll-loops -finline-functions -fno-math-errno
#                             -fno-trapping-math), without -march=native so that one build
#                             recipe serves x86-64 and aarch64 hosts alike.
set -e
here=$(cd "$(dirname "$0")" && pwd)
mkdir -p "$here/_build"
${CC:-cc} -O2 -std=c11 -D_GNU_SOURCE -fopenmp -ffp-contract=off -fno-fast-math -fPIC -shared \
    -Wall -Wno-unused-function -o "$here/_build/libether_oracle.so" "$here/ether_oracle.c" "$here/learn_oracle.c" -lm
${CC:-cc} -O3 -std=c11 -D_GNU_SOURCE -fopenmp -funroll-loops -finline-functions -fno-math-errno \
    -fno-trapping-math -fPIC -shared -Wall -Wno-unused-function \
    -o "$here/_build/libether_oracle_timed.so" "$here/ether_oracle.c" -lm
