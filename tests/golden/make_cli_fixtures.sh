#!/bin/sh
# Runs this repository's drop-in binaries (render_engine_gb300/_build/poc_gpu_l3, poc_gpu_l8) on a
# GPU the way the reference's cuda/run_cuda.sh runs its own, and writes their JSONL under
# tests/golden/cli/ with run_cuda.sh's file names; tests/test_dropin_scripts.py feeds them to the
# reference's unmodified analyse_cuda.py and budget.py.  Run from the repository root after the
# build:  sh tests/golden/make_cli_fixtures.sh
# As run_cuda.sh does, a file that is already there (and not empty) is skipped: delete it to make
# it again.
set -e
B=render_engine_gb300/_build
G=tests/golden
O=$G/cli
T=$(mktemp -d)
mkdir -p $O
for s in scene_main scene_stress scene_holdout scene_scale_43k scene_scale_1M; do
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
# the published curves' commands (reference/cuda_rtx4060/scen_main.jsonl, scen_stress.jsonl,
# scen_holdout.jsonl: the built-in scenarios and the 18 methods of `scen` on both box scenes)
R scen_main.jsonl $B/poc_gpu_l3 scen $T/scene_main.bin 10
R scen_stress.jsonl $B/poc_gpu_l8 scenf $T/scene_stress.bin 10 $G/scenarios_stress.txt
R scen_holdout.jsonl $B/poc_gpu_l3 scen $T/scene_holdout.bin 10
# run_cuda.sh's own lines for the box scenes (scenarios_main.txt, the 14 methods of `scenf`) and
# the timing scenes
R scenf_main.jsonl $B/poc_gpu_l3 scenf $T/scene_main.bin 10 $G/scenarios_main.txt
R scenf_holdout.jsonl $B/poc_gpu_l3 scenf $T/scene_holdout.bin 10 $G/scenarios_main.txt
# the modes the reference publishes nothing for, with the commands of
# tests/golden/make_ref_main_fixtures.sh (which runs the reference's own binary)
R quality_main.jsonl $B/poc_gpu_l3 quality $T/scene_main.bin 4 1,1.5
R recon_main.jsonl $B/poc_gpu_l3 recon $T/scene_main.bin 4
R taa_main.jsonl $B/poc_gpu_l3 taa $T/scene_main.bin 10 $G/scenarios_main.txt
R quality_stress.jsonl $B/poc_gpu_l8 quality $T/scene_stress.bin 4 1,1.5
R recon_stress.jsonl $B/poc_gpu_l8 recon $T/scene_stress.bin 4
R taa_stress.jsonl $B/poc_gpu_l8 taa $T/scene_stress.bin 10 $G/scenarios_stress.txt
R timing_43k.jsonl $B/poc_gpu_l3 timing $T/scene_scale_43k.bin
R timing_1M.jsonl $B/poc_gpu_l3 timing $T/scene_scale_1M.bin
R res_1M.jsonl $B/poc_gpu_l3 res $T/scene_scale_1M.bin
rm -rf $T
