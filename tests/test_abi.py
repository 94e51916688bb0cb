"""The C-ABI library builds, loads and exports every entry point of include/rc_api.h (no GPU
needed: nothing here launches a kernel)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header="rc_api.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(rc_[a-z_]+)\s*\(", src)))


HEADERS = sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h"))


@pytest.fixture(scope="module")
def lib():
    from render_engine_gb300 import build
    path = build.build()
    return path


def test_header_declares_entry_points():
    names = declared_functions()
    assert "rc_create" in names and "rc_frame" in names and len(names) >= 20


@pytest.mark.parametrize("header", HEADERS)
def test_library_exports_every_declared_symbol(lib, header):
    L = ctypes.CDLL(lib)
    missing = [n for n in declared_functions(header) if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (rc_[a-z_]+)$", out, flags=re.M))
    assert set(declared_functions(header)) <= exported


def test_python_binding_lists_every_symbol():
    from render_engine_gb300 import hashgrid, mlp, native
    assert sorted(native.EXPORTS) == declared_functions("rc_api.h")
    assert sorted(hashgrid.EXPORTS) == declared_functions("rc_hashgrid.h")
    assert sorted(mlp.EXPORTS) == declared_functions("rc_mlp.h")


def test_status_strings_and_version(lib):
    L = ctypes.CDLL(lib)
    L.rc_status_string.restype = ctypes.c_char_p
    assert L.rc_abi_version() == 1
    assert L.rc_status_string(0) == b"ok"
    assert b"CUDA" in L.rc_status_string(4)


def test_binaries_built(lib):
    d = os.path.dirname(lib)
    for n in ("poc_gpu_l3", "poc_gpu_l8"):
        assert os.access(os.path.join(d, n), os.X_OK)


def test_cli_prep_needs_a_gpu(lib):
    d = os.path.dirname(lib)
    for exe in ("poc_gpu_l3", "poc_gpu_l8"):   # three lamps as the reference, or eight
        r = subprocess.run([os.path.join(d, exe), "prep", "x.mesh", "x.bin"], capture_output=True, text=True)
        assert r.returncode == 2                # no GPU here: rc_create fails, nothing falls back


def test_missing_library_fails_loudly(tmp_path, monkeypatch):
    from render_engine_gb300 import native
    monkeypatch.setattr(native, "LIB_PATH", str(tmp_path / "absent.so"))
    monkeypatch.setattr(native, "_lib", None)
    with pytest.raises(RuntimeError):
        native.load_library()
