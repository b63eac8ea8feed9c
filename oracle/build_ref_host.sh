#!/usr/bin/env bash
# Build recipe for oracle/_ref/libref_host.so: DexDeform's mpm/csrc/integrator.cu
# compiled unmodified, from the reference tree, as host C++ (see ref_host/ref_host.cpp).
# TEST INFRASTRUCTURE ONLY.  Needs the reference tree (REF_ROOT, default
# /root/reference); exits 0 without building when it is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
REF_ROOT="${REF_ROOT:-/root/reference}"
CUDA_HOME="${CUDA_HOME:-/usr/local/cuda}"
if [ ! -f "$REF_ROOT/mpm/csrc/integrator.cu" ]; then
  echo "reference tree not found at $REF_ROOT: oracle/_ref not built"; exit 0
fi
mkdir -p "$here/_ref"
g++ -O2 -fPIC -shared -w -I "$here/ref_host/shim" -I "$CUDA_HOME/include" \
    -DREF_CSRC="$REF_ROOT/mpm/csrc" "$here/ref_host/ref_host.cpp" \
    -o "$here/_ref/libref_host.so" -L "$CUDA_HOME/lib64" -lcudart
echo "built $here/_ref/libref_host.so"
