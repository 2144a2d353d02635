#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.
# -ffp-contract=off keeps a*b+c as two roundings, the order the engine's
# FP64 kernels use (they are compiled with --fmad=false).
set -e
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
${CXX:-g++} -O2 -std=c++17 -fPIC -shared -ffp-contract=off -fno-fast-math \
    -Wall -Wno-unused-function \
    -o "$here/_build/liboracle.so" "$here/neci_oracle.cpp"
