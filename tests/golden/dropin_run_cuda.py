"""Runs the reference's own `cuda/run_cuda.sh --test` on a GPU with this repository's drop-in
binaries in place of its poc_gpu_l3 / poc_gpu_l8.

The checkout's run_cuda.sh, analyse_cuda.py and budget.py are copied, unmodified, into a
temporary cuda/ folder beside render_engine_gb300/_build/poc_gpu_l3, poc_gpu_l8 and the library
they load from their own folder, librc_gb300.so (with no poc_gpu.cu there, run_cuda.sh does not
rebuild) and the scenes it reads: scene_main, scene_holdout, scene_stress, scene_scale_43k and
the scenario files, from tests/golden/.
Its --test mode also reads scenes/scene_scale_170k.bin, which the checkout does not hold; a
stand-in takes its place: render_engine_gb300.scene.box_room at 170,000 points (the box-room
layout of the reference's scale scenes), its references converged on the GPU.  run_cuda.sh must
exit 0; its results folder (results/cuda_test/: the JSONL of every run, systeme_cuda.txt and
RESULTATS_CUDA.md written by analyse_cuda.py) is copied to the output folder.

Usage, from the repository root after the build:
    python tests/golden/dropin_run_cuda.py <reference checkout> <output folder>
"""
import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

SCRIPTS = ("run_cuda.sh", "analyse_cuda.py", "budget.py")
SCENES = ("scene_main.bin", "scene_holdout.bin", "scene_stress.bin", "scene_scale_43k.bin")


def stand_in_170k(path):
    from render_engine_gb300 import native as N
    from render_engine_gb300 import scene as S
    sc = S.box_room(points=170_000)
    ctx = N.Context()
    ctx.load_bytes(S.write(sc))
    ctx.build_reference()
    S.with_references(sc, ctx)
    ctx.close()
    with open(path, "wb") as f:
        f.write(S.write(sc))


def main(ref, out):
    build = os.path.join(ROOT, "render_engine_gb300", "_build")
    with tempfile.TemporaryDirectory() as t:
        cuda = os.path.join(t, "cuda")
        scenes = os.path.join(cuda, "scenes")
        os.makedirs(scenes)
        for s in SCRIPTS:
            shutil.copy(os.path.join(ref, "cuda", s), os.path.join(cuda, s))
        for b in ("poc_gpu_l3", "poc_gpu_l8", "librc_gb300.so"):
            shutil.copy(os.path.join(build, b), os.path.join(cuda, b))
        for s in SCENES:
            with gzip.open(os.path.join(HERE, s + ".gz"), "rb") as f, open(os.path.join(scenes, s), "wb") as g:
                shutil.copyfileobj(f, g)
        for s in ("scenarios_main.txt", "scenarios_stress.txt"):
            shutil.copy(os.path.join(HERE, s), os.path.join(scenes, s))
        stand_in_170k(os.path.join(scenes, "scene_scale_170k.bin"))
        r = subprocess.run(["bash", os.path.join(cuda, "run_cuda.sh"), "--test"], timeout=1200)
        res = os.path.join(t, "results", "cuda_test")
        if os.path.isdir(res):
            shutil.copytree(res, out, dirs_exist_ok=True)
        print("run_cuda.sh --test exit code", r.returncode)
        return r.returncode


if __name__ == "__main__":
    sys.exit(main(sys.argv[1], sys.argv[2]))
