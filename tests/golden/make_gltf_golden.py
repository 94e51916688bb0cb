"""Regenerates the glTF -> MSH1 fixtures under tests/golden/gltf/ from a reference checkout.

Writes the synthetic scenes of gltf_scenes.py into tests/golden/gltf/, runs the reference's own
converter (scenes_publiques/convertir.py, unmodified, as run_cuda.sh runs it) on each, and keeps
its output mesh (<scene>.mesh) and its summary line (<scene>.json).  tests/test_gltf.py converts the
same scenes with render_engine_gb300/gltf.py and compares.

Usage: python tests/golden/make_gltf_golden.py [reference checkout]
(default $RC_REFERENCE_DIR, else the directory "reference" beside this repository)
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import gltf_scenes  # noqa: E402

REF = (sys.argv[1] if len(sys.argv) > 1 else
       os.environ.get("RC_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(HERE))), "reference"))
CONVERTER = os.path.join(REF, "scenes_publiques", "convertir.py")
OUT = os.path.join(HERE, "gltf")

for name in gltf_scenes.write_all(OUT):
    stem = os.path.splitext(name)[0]
    r = subprocess.run([sys.executable, CONVERTER, os.path.join(OUT, name), os.path.join(OUT, stem + ".mesh")],
                       capture_output=True, text=True, check=True)
    with open(os.path.join(OUT, stem + ".json"), "w") as f:
        f.write(r.stdout)
    print(stem, r.stdout.strip())
