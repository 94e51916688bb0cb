"""ctypes front end of the hash-grid oracle (oracle/hg_oracle.c) — TEST INFRASTRUCTURE ONLY.

The checker for include/rc_hashgrid.h: the same operations on host arrays laid out as the
device arrays.  Used by the tests only.
"""
from __future__ import annotations

import ctypes

import numpy as np

from oracle import pyoracle


class Config(ctypes.Structure):
    _fields_ = [("zone_lo", ctypes.c_float * 3), ("zone_hi", ctypes.c_float * 3), ("origin", ctypes.c_float * 3),
                ("cell", ctypes.c_float), ("capacity", ctypes.c_uint32), ("max_depth", ctypes.c_int),
                ("acc_frames", ctypes.c_int), ("stale_frames", ctypes.c_int), ("tracing_distance", ctypes.c_float)]


class _State(ctypes.Structure):
    _fields_ = [("keys", ctypes.c_void_p), ("accum", ctypes.c_void_p), ("resolved", ctypes.c_void_p),
                ("bank0", ctypes.c_void_p), ("bank1", ctypes.c_void_p), ("bank", ctypes.c_int)]


def config_from(cfg) -> Config:
    """The oracle's config from the library's rc_hg_config (same leading fields)."""
    c = Config()
    for name, _ in Config._fields_:
        v = getattr(cfg, name)
        if isinstance(v, ctypes.Array):
            getattr(c, name)[:] = v[:]
        else:
            setattr(c, name, v)
    return c


_bound = False


def _lib():
    global _bound
    L = pyoracle.lib()
    if not _bound:
        vp, i, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32
        C, S = ctypes.POINTER(Config), ctypes.POINTER(_State)
        L.hgo_mark_point.argtypes = [C, vp, vp]
        L.hgo_mark_segment.argtypes = [C, vp, vp, vp]
        L.hgo_mark_paths.argtypes = [C, S, vp, vp, i]
        L.hgo_begin_frame.argtypes = [C, S, u32, u32]
        L.hgo_resolve.argtypes = [C, S, vp, vp]
        L.hgo_event_mask.argtypes = [C, vp, vp, i, i, i, vp, vp, vp]
        L.hgo_key.argtypes = [C, vp, vp]
        L.hgo_key.restype = ctypes.c_uint64
        L.hgo_insert.argtypes = [C, S, vp, vp, i, vp]
        L.hgo_accumulate.argtypes = [S, vp, vp, i]
        L.hgo_snapshot.argtypes = [C, S, vp, u32]
        L.hgo_snapshot.restype = u32
        L.hgo_restore.argtypes = [S, vp, u32]
        L.hgo_f2h.argtypes = [ctypes.c_float]
        L.hgo_f2h.restype = ctypes.c_uint16
        L.hgo_h2f.argtypes = [ctypes.c_uint16]
        L.hgo_h2f.restype = ctypes.c_float
        L.hgo_voxels_mark.argtypes = [C, i, vp, vp, vp, i, i]
        _bound = True
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Cache:
    """Host copy of a cache (the arrays of rc_hg_array) and the oracle operations on it."""

    def __init__(self, cfg: Config):
        self.cfg = cfg
        n = cfg.capacity
        self.keys = np.zeros(n, np.uint64)
        self.accum = np.zeros((n, 4), np.uint32)
        self.resolved = np.zeros((n, 4), np.uint32)
        self.bank0 = np.zeros((n, 4), np.uint32)
        self.bank1 = np.zeros((n, 4), np.uint32)
        self.bank = 0

    def _st(self) -> _State:
        s = _State(_p(self.keys).value, _p(self.accum).value, _p(self.resolved).value, _p(self.bank0).value,
                   _p(self.bank1).value, self.bank)
        return s

    def _run(self, fn, *args):
        st = self._st()
        out = fn(ctypes.byref(self.cfg), ctypes.byref(st), *args)
        self.bank = st.bank
        return out

    def mark_paths(self, vertices: np.ndarray, path_start: np.ndarray):
        v = np.ascontiguousarray(vertices)
        ps = np.ascontiguousarray(path_start, np.int32)
        self._run(_lib().hgo_mark_paths, _p(v), _p(ps), len(ps) - 1)

    def begin_frame(self, dep_frame: int, period: int = 16):
        self._run(_lib().hgo_begin_frame, dep_frame, period)

    def resolve(self, inv=None) -> np.ndarray:
        iv = np.zeros(4, np.uint32) if inv is None else np.ascontiguousarray(inv, np.uint32)
        counts = np.zeros(3, np.uint32)
        self._run(_lib().hgo_resolve, _p(iv), _p(counts))
        return counts

    def insert(self, pos: np.ndarray, nrm: np.ndarray) -> np.ndarray:
        pos = np.ascontiguousarray(pos, np.float32)
        nrm = np.ascontiguousarray(nrm, np.float32)
        entry = np.zeros(len(pos), np.uint32)
        self._run(_lib().hgo_insert, _p(pos), _p(nrm), len(pos), _p(entry))
        return entry

    def accumulate(self, entry: np.ndarray, rgb: np.ndarray):
        entry = np.ascontiguousarray(entry, np.uint32)
        rgb = np.ascontiguousarray(rgb, np.float32)
        st = self._st()
        _lib().hgo_accumulate(ctypes.byref(st), _p(entry), _p(rgb), len(entry))

    def snapshot(self, dtype) -> np.ndarray:
        recs = np.zeros(self.cfg.capacity, dtype)
        n = self._run(_lib().hgo_snapshot, _p(recs), self.cfg.capacity)
        return recs[:n]

    def restore(self, recs: np.ndarray):
        recs = np.ascontiguousarray(recs)
        st = self._st()
        _lib().hgo_restore(ctypes.byref(st), _p(recs), len(recs))


def mark_point(cfg: Config, p) -> np.ndarray:
    m = np.zeros(3, np.uint32)
    _lib().hgo_mark_point(ctypes.byref(cfg), _p(m), _p(np.ascontiguousarray(p, np.float32)))
    return m


def mark_segment(cfg: Config, a, b) -> np.ndarray:
    m = np.zeros(3, np.uint32)
    _lib().hgo_mark_segment(ctypes.byref(cfg), _p(m), _p(np.ascontiguousarray(a, np.float32)),
                            _p(np.ascontiguousarray(b, np.float32)))
    return m


def key(cfg: Config, p, n) -> int:
    return int(_lib().hgo_key(ctypes.byref(cfg), _p(np.ascontiguousarray(p, np.float32)), _p(np.ascontiguousarray(n, np.float32))))


def event_mask(cfg: Config, la=None, lb=None, sky_a=0, sky_b=0, obj_a=None, obj_b=None) -> np.ndarray:
    inv = np.zeros(4, np.uint32)
    f = lambda v: None if v is None else np.ascontiguousarray(v, np.float32)
    la, lb, oa, ob = f(la), f(lb), f(obj_a), f(obj_b)
    _lib().hgo_event_mask(ctypes.byref(cfg), _p(la), _p(lb), 0 if la is None else len(la), sky_a, sky_b, _p(oa), _p(ob), _p(inv))
    return inv


def f2h(x: float) -> int:
    return int(_lib().hgo_f2h(x))


def h2f(h: int) -> float:
    return float(_lib().hgo_h2f(h))


def voxels_mark(cfg: Config, res: int, vertices: np.ndarray, lengths: np.ndarray, stride: int) -> np.ndarray:
    """Per-voxel light masks of a batch of paths in fixed slots (rc_hg_voxels_mark), from zero."""
    vox = np.zeros(res ** 3, np.uint64)
    v = np.ascontiguousarray(vertices)
    ln = np.ascontiguousarray(lengths, np.int32)
    _lib().hgo_voxels_mark(ctypes.byref(cfg), res, _p(vox), _p(v), _p(ln), stride, len(ln))
    return vox
