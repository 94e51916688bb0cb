"""Build recipe for the native parts: the C-ABI library and the drop-in command-line binaries.

Everything is compiled for sm_103a only, in-tree, into ``render_engine_gb300/_build``:

* ``librc_gb300.so`` -- kernels (one translation unit per light count, compiled in parallel)
  and the host runtime behind ``include/rc_api.h``, plus the hash-grid cache with dependency
  masks behind ``include/rc_hashgrid.h``;
* ``poc_gpu_l3`` / ``poc_gpu_l8`` -- the command-line front end, a client of the library,
  with the names and argument conventions of the reference's binaries (cuda/build.sh).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "librc_gb300.so")
NL_VALUES = (1, 2, 3, 4, 8, 16, 32)
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources() -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))] + \
        [os.path.join(ROOT, "include", h) for h in ("rc_api.h", "rc_hashgrid.h", "rc_mlp.h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile what is out of date; return the library path."""
    os.makedirs(OUT, exist_ok=True)
    deps = _sources()
    nv = nvcc()
    jobs = []
    objs = []
    for nl in NL_VALUES:
        o = os.path.join(OUT, "rc_kernels_nl%d.o" % nl)
        objs.append(o)
        if force or _stale(o, deps):
            jobs.append([nv, *ARCH, *FLAGS, "-DRC_NL_ONE=%d" % nl, "-c", os.path.join(CSRC, "rc_kernels.cu"), "-o", o])
    for name in ("rc_runtime", "rc_adjoint", "rc_taa", "rc_prep", "rc_noalloc", "rc_hashgrid", "rc_mlp"):
        o = os.path.join(OUT, name + ".o")
        objs.append(o)
        # the scene preparation's host arithmetic rounds every operation (no contraction), the
        # same on every host architecture
        extra = ["-Xcompiler", "-ffp-contract=off"] if name == "rc_prep" else []
        if force or _stale(o, deps):
            jobs.append([nv, *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, name + ".cu"), "-o", o])
    cli_obj = {}
    for nl in (3, 8):
        oc = os.path.join(OUT, "poc_gpu_main_l%d.o" % nl)
        cli_obj[nl] = oc
        if force or _stale(oc, deps):
            jobs.append(["g++", "-O2", "-std=c++17", "-DRC_CLI_NLIGHTS=%d" % nl, "-I", os.path.join(ROOT, "include"),
                         "-c", os.path.join(CSRC, "poc_gpu_main.cpp"), "-o", oc])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    if force or _stale(LIB, objs):
        tmp = LIB + ".%d.tmp" % os.getpid()
        _run([nv, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
        os.replace(tmp, LIB)
    for nl in (3, 8):
        exe = os.path.join(OUT, "poc_gpu_l%d" % nl)
        if force or _stale(exe, [cli_obj[nl], LIB]):
            _run(["g++", "-o", exe, cli_obj[nl], "-L", OUT, "-lrc_gb300", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print("built", LIB, file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
