#!/usr/bin/env bash
# Build recipe for oracle/_build/libmpm_oracle.so, the FP64 C restatement.
# TEST INFRASTRUCTURE ONLY.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
mkdir -p "$here/_build"
# no multiply-add contraction: the FP32 renderer restatement follows the
# reference's unfused arithmetic on every host architecture
gcc -O2 -fopenmp -fPIC -shared -std=gnu11 -ffp-contract=off "$here/mpm_oracle.c" "$here/render_oracle.c" \
    -o "$here/_build/libmpm_oracle.so" -lm
echo "built $here/_build/libmpm_oracle.so"
