#!/bin/sh
# Builds the reference's own command-line program (cuda/poc_gpu.cu of a reference checkout,
# unmodified, with the flags of its cuda/build.sh) on a GPU machine and writes under
# tests/golden/ref_main/ what it prints for the modes whose outputs the reference does not
# publish: quality, recon and taa on scene_main, and run_cuda.sh's scenf lines on scene_main and
# scene_holdout.  tests/test_ref_main_outputs.py and tests/test_gpu_ref_main_outputs.py compare
# this repository's drop-in binaries with them.
# Usage, from the repository root:  sh tests/golden/make_ref_main_fixtures.sh <reference checkout>
# CUDA_ARCH (default sm_103a) stands for build.sh's -arch.  As run_cuda.sh does, a file that is
# already there (and not empty) is skipped: delete it to make it again.
set -e
REF=$1
G=tests/golden
O=$G/ref_main
T=$(mktemp -d)
mkdir -p $O
nvcc -O3 -lineinfo -arch=${CUDA_ARCH:-sm_103a} -std=c++17 -DGX=8 -DGY=4 -DGZ=4 -DNLIGHTS=3 $REF/cuda/poc_gpu.cu -o $T/poc_gpu_l3
for s in scene_main scene_holdout; do
    gzip -dc $G/$s.bin.gz > $T/$s.bin
done
R() {   # output file, command...
    out=$1
    shift
    if [ -s $O/$out ]; then
        echo "already there: $out"
        return
    fi
    echo "$out"
    "$@" > $O/$out.tmp
    mv $O/$out.tmp $O/$out
}
R quality_main.jsonl $T/poc_gpu_l3 quality $T/scene_main.bin 4 1,1.5
R recon_main.jsonl $T/poc_gpu_l3 recon $T/scene_main.bin 4
R taa_main.jsonl $T/poc_gpu_l3 taa $T/scene_main.bin 10 $G/scenarios_main.txt
R scenf_main.jsonl $T/poc_gpu_l3 scenf $T/scene_main.bin 10 $G/scenarios_main.txt
R scenf_holdout.jsonl $T/poc_gpu_l3 scenf $T/scene_holdout.bin 10 $G/scenarios_main.txt
rm -rf $T
