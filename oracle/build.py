"""Build recipe of the test infrastructure under oracle/ — TEST INFRASTRUCTURE ONLY.

* ``_build/liboracle.so``  -- the CPU restatement (rc_oracle.c), gcc -O3 -fopenmp;
* ``_build/librefrun.so``  -- the driver of the reference's own kernels (refrun.cpp);
* ``_ref/ref_l{3,8,16,32}.cubin`` -- the reference's cuda/poc_gpu.cu compiled for sm_103a by
  build_ref.sh, only where the reference checkout is present (the cubins are device code,
  so the copies built here are used unchanged on the GPU machine);
* ``_ref/libpatch_ref.so`` -- pieces of the reference's bench patch (the dependency-marking
  shader functions, the host function of an object's event zones) compiled as C++ by
  build_patch_ref.sh, where the reference checkout is present (CPU tests only).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $RC_REFERENCE_DIR, else a directory named "reference" beside this repository
REFERENCE = os.environ.get("RC_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
CUDA = "/usr/local/cuda"


def _stale(t, deps):
    return not os.path.exists(t) or any(os.path.getmtime(d) > os.path.getmtime(t) for d in deps)


def build_refrun(force: bool = False) -> str:
    out = os.path.join(HERE, "_build", "librefrun.so")
    src = os.path.join(HERE, "refrun.cpp")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if force or _stale(out, [src]):
        libdir = os.path.join(CUDA, "lib64")
        stubs = os.path.join(libdir, "stubs")
        tmp = out + ".%d.tmp" % os.getpid()
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", src, "-I", os.path.join(CUDA, "include"),
                               "-L", stubs, "-L", libdir, "-lcuda", "-o", tmp])
        os.replace(tmp, out)
    return out


def build_reference_cubins(force: bool = False) -> bool:
    """Compile the reference kernels when the reference checkout is present."""
    src = os.path.join(REFERENCE, "cuda", "poc_gpu.cu")
    outs = [os.path.join(HERE, "_ref", n) for n in ("ref_l3.cubin", "ref_l8.cubin", "ref_l16.cubin", "ref_l32.cubin",
                                                     "ref_l3_g16x8x6.cubin")]
    if not os.path.exists(src):
        return all(os.path.exists(o) for o in outs)
    if force or any(_stale(o, [src, os.path.join(HERE, "build_ref.sh")]) for o in outs):
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), REFERENCE])
    return True


def build_patch_ref(force: bool = False) -> bool:
    """Compile pieces of the reference's bench patch as C++ (build_patch_ref.sh) when the
    reference checkout is present."""
    src = os.path.join(REFERENCE, "windows", "patch", "rtxgi_bench.patch")
    out = os.path.join(HERE, "_ref", "libpatch_ref.so")
    if not os.path.exists(src):
        return os.path.exists(out)
    deps = [src, os.path.join(HERE, "build_patch_ref.sh"), os.path.join(HERE, "hlsl_compat.h"), os.path.join(HERE, "patch_ref.cpp")]
    if force or _stale(out, deps):
        subprocess.check_call(["sh", os.path.join(HERE, "build_patch_ref.sh"), REFERENCE])
    return True


def build(force: bool = False) -> None:
    from oracle import pyoracle
    pyoracle.build(force)
    build_refrun(force)
    build_reference_cubins(force)
    build_patch_ref(force)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(HERE))
    build(force="--force" in sys.argv)
