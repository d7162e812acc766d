#!/bin/sh
# Compile the reference's device code, unmodified and from its own source files
# (lib/contract_kernels_*.cu with the lib/calculate_*_core.h bodies), into
# sm_103a cubins under oracle/_ref/.  Runs only where the reference tree is
# mounted, given as $1 or in $CTR_REFERENCE_ROOT (no default: without either it
# stops with a message).  The cubins are test infrastructure:
# oracle/refkernels.py launches them to record the reference's own outputs as
# golden vectors.
set -e
REF=${1:-$CTR_REFERENCE_ROOT}
[ -n "$REF" ] || { echo "usage: build_ref.sh <reference tree> (or set CTR_REFERENCE_ROOT)" >&2; exit 1; }
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/lib" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
for k in rho rhopi pipi loop_unity sigma sigmapi; do
  nvcc -cubin -gencode arch=compute_103a,code=sm_103a -O3 -I"$REF/include" -I"$REF/lib" \
       "$REF/lib/contract_kernels_$k.cu" -o "$OUT/contract_kernels_$k.cubin" &
done
wait
ls "$OUT"
