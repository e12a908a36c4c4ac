#!/bin/bash
# Build the reference harness (test infrastructure) into oracle/_ref/ from the
# reference's own CUDA headers where they lie.  The reference checkout is the
# first argument or $SFD_REFERENCE_DIR; nothing is copied from it.
#   oracle/ref_build.sh [/path/to/reference]
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${SFD_REFERENCE_DIR:-}}"
if [ -z "$REF" ] || [ ! -d "$REF/CuSuperHelium/CuSuperHelium" ]; then
  echo "give the reference checkout as the argument or in SFD_REFERENCE_DIR" >&2
  exit 1
fi
mkdir -p "$HERE/_ref"
nvcc -std=c++20 -O2 -gencode arch=compute_103a,code=sm_103a \
  -I "$HERE/ref_stub" -I "$REF/CuSuperHelium/CuSuperHelium" \
  "$HERE/ref_harness.cu" -o "$HERE/_ref/ref_harness" -lcusolver -lcublas -lcufft
echo "$HERE/_ref/ref_harness"
