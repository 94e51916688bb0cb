#!/bin/sh
# Compiles the reference's own cuda/poc_gpu.cu, unchanged and read where it lies in the
# reference checkout, into device-only cubins for sm_103a under oracle/_ref/:
#   ref_l{3,8,16,32}.cubin  -DNLIGHTS=3, 8, 16, 32 (8 x 4 x 4 grid),
#   ref_l3_g16x8x6.cubin  -DNLIGHTS=3 with the transit grid 16 x 8 x 6
# with the transit grid of the reference's build script (cuda/build.sh: -DGX=8 -DGY=4
# -DGZ=4) and its optimisation flags (-O3 -lineinfo -std=c++17).  Only the device code is
# compiled (the host side of poc_gpu.cu is driven by oracle/refrun.cpp).
# Usage: oracle/build_ref.sh [reference checkout]; default $RC_REFERENCE_DIR, else the
# directory "reference" beside this repository
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${RC_REFERENCE_DIR:-$HERE/../../reference}}"
SRC="$REF/cuda/poc_gpu.cu"
[ -f "$SRC" ] || { echo "reference source not found: $SRC" >&2; exit 1; }
mkdir -p "$HERE/_ref"
for L in 3 8 16 32; do
  nvcc -cubin -O3 -lineinfo -std=c++17 -gencode arch=compute_103a,code=sm_103a \
       -DGX=8 -DGY=4 -DGZ=4 -DNLIGHTS=$L -w "$SRC" -o "$HERE/_ref/ref_l$L.cubin.tmp"
  mv "$HERE/_ref/ref_l$L.cubin.tmp" "$HERE/_ref/ref_l$L.cubin"
done
# a finer transit grid (768 voxels, 24 mask words), the grid being a compile-time constant there
nvcc -cubin -O3 -lineinfo -std=c++17 -gencode arch=compute_103a,code=sm_103a \
     -DGX=16 -DGY=8 -DGZ=6 -DNLIGHTS=3 -w "$SRC" -o "$HERE/_ref/ref_l3_g16x8x6.cubin.tmp"
mv "$HERE/_ref/ref_l3_g16x8x6.cubin.tmp" "$HERE/_ref/ref_l3_g16x8x6.cubin"
