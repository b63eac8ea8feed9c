#!/usr/bin/env bash
# Build recipe for oracle/_build/libmpm_oracle.so, the FP64 C restatement.
# TEST INFRASTRUCTURE ONLY.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
gcc -O2 -fopenmp -fPIC -shared -std=c11 "$here/mpm_oracle.c" -o "$here/_build/libmpm_oracle.so" -lm
echo "built $here/_build/libmpm_oracle.so"
