#!/usr/bin/env bash
# Builds the CPU restatement (the oracle) as oracle/_build/liboracle.so.
# Test infrastructure only.  -ffp-contract=off keeps FP64 results identical
# on x86-64 and AArch64 (no fused multiply-add contraction).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$HERE/_build"
"${CXX:-g++}" -std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -shared \
  -o "$HERE/_build/liboracle.so" "$HERE/prender_oracle.cpp" ${ORACLE_EXTRA_SOURCES:-}
echo "built $HERE/_build/liboracle.so"
