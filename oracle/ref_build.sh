#!/bin/bash
# Build the reference harness (test infrastructure) into oracle/_ref/ from the
# reference's own CUDA headers where they lie.  The reference checkout is the
# first argument, else $SFD_REFERENCE_DIR, else /root/reference; nothing is
# copied from it.  Without a checkout (the GPU machines have none) it builds
# nothing and exits 0.
#   oracle/ref_build.sh [/path/to/reference]
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${SFD_REFERENCE_DIR:-/root/reference}}"
if [ ! -d "$REF/CuSuperHelium/CuSuperHelium" ]; then
  echo "no reference checkout at $REF: oracle/_ref not built"
  exit 0
fi
mkdir -p "$HERE/_ref"
nvcc -std=c++20 -O2 -gencode arch=compute_103a,code=sm_103a \
  -I "$HERE/ref_stub" -I "$REF/CuSuperHelium/CuSuperHelium" \
  "$HERE/ref_harness.cu" -o "$HERE/_ref/ref_harness" -lcusolver -lcublas -lcufft
echo "$HERE/_ref/ref_harness"
