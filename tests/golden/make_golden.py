"""Regenerates the committed golden fixtures from a reference checkout.

Reads, from the reference (falcon123212/render_engine):
  cuda/scenes/scene_main.bin, cuda/scenes/scene_stress.bin     (its box-scene fixtures)
  cuda/scenes/scene_holdout.bin                                (its validation box scene)
  cuda/scenes/scene_scale_43k.bin                              (its smallest timing scene)
  cuda/scenes/scene_scale_1M.bin.gz                            (its 1,082,802-point timing scene)
  reference/cuda_rtx4060/scen_main.jsonl, scen_stress.jsonl,
      scen_holdout.jsonl                                       (its published RTX 4060
      per-frame error curves: `poc_gpu_l3 scen scene_main.bin 10`,
      `poc_gpu_l8 scenf scene_stress.bin 10 scenarios_stress.txt` and
      `poc_gpu_l3 scen scene_holdout.bin 10`)
  cuda/scenes/scenarios_stress.txt, cuda/scenes/scenarios_main.txt
and writes gzip copies of the scenes and the curves as JSON next to this script.

Usage: python tests/golden/make_golden.py [reference checkout]
(default $RC_REFERENCE_DIR, else the directory "reference" beside this repository)
"""
import gzip
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = (sys.argv[1] if len(sys.argv) > 1 else
       os.environ.get("RC_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))


def curves(path):
    out = []
    for line in open(path):
        if not line.startswith("{"):
            continue
        r = json.loads(line)
        if r.get("type") == "scen":
            out.append({k: r[k] for k in ("scen", "name", "pre", "post", "last", "curve")})
    return out


for name in ("scene_main.bin", "scene_stress.bin", "scene_holdout.bin", "scene_scale_43k.bin"):
    with open(os.path.join(REF, "cuda", "scenes", name), "rb") as f, gzip.open(os.path.join(HERE, name + ".gz"), "wb", 9) as g:
        shutil.copyfileobj(f, g)
shutil.copy(os.path.join(REF, "cuda", "scenes", "scenarios_stress.txt"), os.path.join(HERE, "scenarios_stress.txt"))
shutil.copy(os.path.join(REF, "cuda", "scenes", "scenarios_main.txt"), os.path.join(HERE, "scenarios_main.txt"))
# the reference's 1,082,802-point timing scene (its throughput case, cuda/run_cuda.sh), already gzip
shutil.copy(os.path.join(REF, "cuda", "scenes", "scene_scale_1M.bin.gz"), os.path.join(HERE, "scene_scale_1M.bin.gz"))
json.dump({"mode": "scen", "seed0": 2000, "nseeds": 10, "rows": curves(os.path.join(REF, "reference", "cuda_rtx4060", "scen_main.jsonl"))},
          open(os.path.join(HERE, "golden_scen_main.json"), "w"))
json.dump({"mode": "scenf", "seed0": 3000, "nseeds": 10, "rows": curves(os.path.join(REF, "reference", "cuda_rtx4060", "scen_stress.jsonl"))},
          open(os.path.join(HERE, "golden_scen_stress.json"), "w"))
json.dump({"mode": "scen", "seed0": 2000, "nseeds": 10, "rows": curves(os.path.join(REF, "reference", "cuda_rtx4060", "scen_holdout.jsonl"))},
          open(os.path.join(HERE, "golden_scen_holdout.json"), "w"))
print("golden fixtures written to", HERE)
