#!/bin/sh
# Runs this repository's drop-in binaries (render_engine_gb300/_build/poc_gpu_l3, poc_gpu_l8) on a
# GPU the way the reference's cuda/run_cuda.sh runs its own, and writes their JSONL under
# tests/golden/cli/ with run_cuda.sh's file names; tests/test_dropin_scripts.py feeds them to the
# reference's unmodified analyse_cuda.py and budget.py.  Run from the repository root after the
# build:  sh tests/golden/make_cli_fixtures.sh
set -e
B=render_engine_gb300/_build
G=tests/golden
O=$G/cli
T=$(mktemp -d)
mkdir -p $O
gzip -dc $G/scene_main.bin.gz > $T/scene_main.bin
gzip -dc $G/scene_stress.bin.gz > $T/scene_stress.bin
gzip -dc $G/scene_scale_1M.bin.gz > $T/scene_scale_1M.bin
# the published curves' commands (reference/cuda_rtx4060/scen_main.jsonl, scen_stress.jsonl)
$B/poc_gpu_l3 scen $T/scene_main.bin 10 > $O/scen_main.jsonl
$B/poc_gpu_l8 scenf $T/scene_stress.bin 10 $G/scenarios_stress.txt > $O/scen_stress.jsonl
# run_cuda.sh's own lines for the box scenes and the 1 M-point scale scene
$B/poc_gpu_l3 scenf $T/scene_main.bin 10 $G/scenarios_main.txt > $O/scenf_main.jsonl
$B/poc_gpu_l3 timing $T/scene_scale_1M.bin > $O/timing_1M.jsonl
$B/poc_gpu_l3 res $T/scene_scale_1M.bin > $O/res_1M.jsonl
rm -rf $T
