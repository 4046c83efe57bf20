#!/usr/bin/env bash
# Builds the CPU checkers (test infrastructure, never shipped in libgba):
#   oracle/_build/liboracle.so   — the C restatement (oracle.c), always;
#   oracle/_ref/libslamplay_ref.so — the reference's own residual functor,
#       rotation and BALProblem.cpp compiled from where they lie in the
#       reference tree, with declaration shims for Ceres/Eigen; only when the
#       reference tree is present (REF_ROOT, default /root/reference).
# Usage: oracle/build_ref.sh [oracle|ref|all|root]   (root: prints the
# reference tree's path when it is present, nothing otherwise)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
WHAT="${1:-all}"
if [[ "$WHAT" == "root" ]]; then
  if [[ -f "$REF_ROOT/utils/datasets/BALProblem.cpp" ]]; then echo "$REF_ROOT"; fi
  exit 0
fi
CFLAGS="-O2 -fPIC -ffp-contract=off -fopenmp"

if [[ "$WHAT" == "oracle" || "$WHAT" == "all" ]]; then
  mkdir -p "$HERE/_build"
  gcc -std=c11 $CFLAGS -shared "$HERE/oracle.c" "$HERE/synth.c" -o "$HERE/_build/liboracle.so.tmp" -lm
  mv -f "$HERE/_build/liboracle.so.tmp" "$HERE/_build/liboracle.so"
fi

if [[ "$WHAT" == "ref" || "$WHAT" == "all" ]]; then
  if [[ -f "$REF_ROOT/utils/datasets/BALProblem.cpp" ]]; then
    mkdir -p "$HERE/_ref"
    g++ -std=c++17 -O2 -fPIC -ffp-contract=off -shared -w \
      -I "$HERE/ref_shim" -I "$REF_ROOT/utils" -I "$REF_ROOT/utils/datasets" \
      "$REF_ROOT/utils/datasets/BALProblem.cpp" "$HERE/ref_driver.cpp" \
      -o "$HERE/_ref/libslamplay_ref.so.tmp"
    mv -f "$HERE/_ref/libslamplay_ref.so.tmp" "$HERE/_ref/libslamplay_ref.so"
  else
    echo "build_ref.sh: reference tree not found at $REF_ROOT; skipping oracle/_ref" >&2
  fi
fi
