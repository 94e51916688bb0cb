"""ctypes front end of oracle/refrun.cpp (the reference's own kernels on the GPU) — TEST AND
BASELINE INFRASTRUCTURE ONLY.  Array and scalar ids are those of include/rc_api.h."""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "librefrun.so")


def cubin_path(nl: int, grid=(8, 4, 4)) -> str:
    if tuple(grid) == (8, 4, 4):
        return os.path.join(HERE, "_ref", "ref_l%d.cubin" % nl)
    return os.path.join(HERE, "_ref", "ref_l%d_g%dx%dx%d.cubin" % (nl, *grid))


def available(nl: int = 3, grid=(8, 4, 4)) -> bool:
    return os.path.exists(cubin_path(nl, grid))


_lib = None


def lib():
    global _lib
    if _lib is None:
        from oracle import build as obuild
        obuild.build_refrun()
        L = ctypes.CDLL(LIB)
        vp, i, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_size_t
        L.ref_create.restype = vp
        L.ref_create.argtypes = [ctypes.c_char_p, i, ctypes.c_char_p, i]
        L.ref_create_grid.restype = vp
        L.ref_create_grid.argtypes = [ctypes.c_char_p, i, i, i, i, ctypes.c_char_p, i]
        L.ref_destroy.argtypes = [vp]
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_last_error.argtypes = [vp]
        L.ref_load.restype = i
        L.ref_load.argtypes = [vp, vp, sz]
        L.ref_begin.restype = i
        L.ref_begin.argtypes = [vp, vp, i, ctypes.c_uint32]
        L.ref_frame.restype = i
        L.ref_frame.argtypes = [vp, i, i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)]
        L.ref_sync.restype = i
        L.ref_sync.argtypes = [vp]
        L.ref_array.restype = i
        L.ref_array.argtypes = [vp, i, vp, sz, i]
        L.ref_scalar.restype = i
        L.ref_scalar.argtypes = [vp, i, i, i]
        L.ref_state_array.restype = i
        L.ref_state_array.argtypes = [vp, i, i, vp, sz]
        L.ref_taa_begin.restype = i
        L.ref_taa_begin.argtypes = [vp, ctypes.c_float, ctypes.c_float, i, i, ctypes.c_uint32]
        L.ref_taa_frame.restype = i
        L.ref_taa_frame.argtypes = [vp, i, ctypes.POINTER(ctypes.c_float)]
        L.ref_taa_array.restype = i
        L.ref_taa_array.argtypes = [vp, i, vp, sz, i]
        _lib = L
    return _lib


_DT = {0: np.float32, 1: np.float32, 2: np.float32, 3: np.float32, 4: np.float32, 5: np.int32, 6: np.uint8,
       7: np.uint32, 8: np.uint32, 9: np.uint8, 10: np.float32, 11: np.float32, 12: np.float32, 13: np.float32,
       14: np.float32, 15: np.float32, 16: np.float32, 17: np.int32}


class RefRunner:
    """The reference's kernels on the GPU with the reference's frame driver logic."""

    def __init__(self, nl: int, data: bytes, grid=(8, 4, 4)):
        L = lib()
        err = ctypes.create_string_buffer(256)
        p = L.ref_create_grid(cubin_path(nl, grid).encode(), nl, grid[0], grid[1], grid[2], err, 256)
        if not p:
            raise RuntimeError("reference kernels: " + err.value.decode())
        self.p = p
        self.L = L
        self._data = np.frombuffer(data, np.uint8).copy()
        if L.ref_load(p, self._data.ctypes.data_as(ctypes.c_void_p), self._data.nbytes) != 0:
            raise RuntimeError("reference load: " + L.ref_last_error(p).decode())
        h = np.frombuffer(data[:32], np.int32)
        self.Np, self.NS, self.NL, self.NW = int(h[0]), int(h[3]), int(h[4]), grid[0] * grid[1] * grid[2] // 32

    def begin(self, method, s0: int, seed: int):
        from render_engine_gb300.methods import to_c
        self._cm = to_c(method)
        if self.L.ref_begin(self.p, ctypes.byref(self._cm), s0, seed & 0xFFFFFFFF) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())

    def frame(self, state: int, want_err: bool = False, timers: np.ndarray | None = None):
        e = ctypes.c_float()
        ms = timers.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if timers is not None else None
        rc = self.L.ref_frame(self.p, state, 1 if want_err else 0, ctypes.byref(e), ms)
        if rc < 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())
        return float(e.value) if rc == 1 else None

    def sync(self):
        self.L.ref_sync(self.p)

    def array(self, which: int) -> np.ndarray:
        n = self._nbytes(which)
        a = np.empty(n // np.dtype(_DT[which]).itemsize, _DT[which])
        if self.L.ref_array(self.p, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 0) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())
        return a

    def set_array(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, _DT[which])
        if self.L.ref_array(self.p, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())

    def _nbytes(self, which: int) -> int:
        Np, NL, NW = self.Np, self.NL, self.NW
        NR = int(np.frombuffer(self._data[:32].tobytes(), np.int32)[5])
        return {0: 4 * NL * Np, 1: 4 * NL * Np, 2: 4 * NL * Np, 3: 4 * Np, 4: 4 * Np, 5: 4 * Np, 6: Np, 7: 4 * NW * Np,
                8: 4 * NW * Np, 9: Np, 10: 4 * Np, 11: 4 * 6 * Np * NL, 12: 4 * NR * 28, 13: 4 * NR * 6, 14: 16 * NR,
                15: 12 * NR, 16: 8, 17: 8}[which]

    def scalar(self, which: int) -> int:
        return self.L.ref_scalar(self.p, which, 0, 0)

    def set_scalar(self, which: int, value: int):
        self.L.ref_scalar(self.p, which, 1, int(value))

    def state_array(self, state: int, which: int) -> np.ndarray:
        n = self.NL * self.Np if which == 0 else self.NW * self.Np
        a = np.empty(n, np.float32 if which == 0 else np.uint32)
        if self.L.ref_state_array(self.p, state, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes) != 0:
            raise RuntimeError("state array")
        return a

    # taa mode (run_taa_mode, poc_gpu.cu:1175-1282)
    _TAA_DT = {0: np.float32, 1: np.float32, 2: np.float32, 3: np.float32, 4: np.int32, 5: np.uint8, 6: np.uint32, 7: np.uint32}

    def taa_begin(self, alpha: float, gamma: float, mask: int, s0: int, seed: int):
        if self.L.ref_taa_begin(self.p, alpha, gamma, mask, s0, seed & 0xFFFFFFFF) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())

    def taa_frame(self, state: int) -> float:
        e = ctypes.c_float()
        if self.L.ref_taa_frame(self.p, state, ctypes.byref(e)) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())
        return float(e.value)

    def taa_array(self, which: int, value: np.ndarray | None = None) -> np.ndarray:
        n = self.Np * (self.NW if which in (6, 7) else 1)
        dt = self._TAA_DT[which]
        a = np.empty(n, dt) if value is None else np.ascontiguousarray(value, dt).reshape(-1)
        if self.L.ref_taa_array(self.p, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 0 if value is None else 1) != 0:
            raise RuntimeError(self.L.ref_last_error(self.p).decode())
        return a

    def close(self):
        if getattr(self, "p", None):
            self.L.ref_destroy(self.p)
            self.p = None

    def __del__(self):
        self.close()
