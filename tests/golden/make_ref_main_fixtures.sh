#!/bin/sh
# Builds the reference's own command-line program (cuda/poc_gpu.cu of a reference checkout,
# unmodified, with the flags of its cuda/build.sh) on a GPU machine and writes under
# tests/golden/ref_main/ what it prints for the modes whose outputs the reference does not
# publish: quality, recon and taa on scene_main (poc_gpu_l3) and on the 8-light scene_stress
# (poc_gpu_l8), and run_cuda.sh's scenf lines on scene_main and scene_holdout.
# tests/test_ref_main_outputs.py and tests/test_gpu_ref_main_outputs.py compare this
# repository's drop-in binaries with them.
# Usage, from the repository root:  sh tests/golden/make_ref_main_fixtures.sh <reference checkout>
# CUDA_ARCH (default sm_103a) stands for build.sh's -arch.  As run_cuda.sh does, a file that is
# already there (and not empty) is skipped: delete it to make it again.
set -e
REF=$1
G=tests/golden
O=$G/ref_main
T=$(mktemp -d)
mkdir -p $O
for s in scene_main scene_holdout scene_stress; do
    gzip -dc $G/$s.bin.gz > $T/$s.bin
done
ref() {   # light count, arguments: the reference's poc_gpu_l<n>, built on first use
    nl=$1
    shift
    if [ ! -x $T/poc_gpu_l$nl ]; then
        nvcc -O3 -lineinfo -arch=${CUDA_ARCH:-sm_103a} -std=c++17 -DGX=8 -DGY=4 -DGZ=4 -DNLIGHTS=$nl $REF/cuda/poc_gpu.cu \
            -o $T/poc_gpu_l$nl 1>&2
    fi
    $T/poc_gpu_l$nl "$@"
}
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
R quality_main.jsonl ref 3 quality $T/scene_main.bin 4 1,1.5
R recon_main.jsonl ref 3 recon $T/scene_main.bin 4
R taa_main.jsonl ref 3 taa $T/scene_main.bin 10 $G/scenarios_main.txt
R scenf_main.jsonl ref 3 scenf $T/scene_main.bin 10 $G/scenarios_main.txt
R scenf_holdout.jsonl ref 3 scenf $T/scene_holdout.bin 10 $G/scenarios_main.txt
R quality_stress.jsonl ref 8 quality $T/scene_stress.bin 4 1,1.5
R recon_stress.jsonl ref 8 recon $T/scene_stress.bin 4
R taa_stress.jsonl ref 8 taa $T/scene_stress.bin 10 $G/scenarios_stress.txt
rm -rf $T
