"""ctypes front end of the CPU oracle (oracle/rc_oracle.c) — TEST INFRASTRUCTURE ONLY.

Used by the test suite, the smoke check and the CPU-baseline leg of the benchmark as the
checker.  It is never imported by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "rc_oracle.c")
SRCS = [SRC, os.path.join(HERE, "hg_oracle.c")]
HDRS = [os.path.join(HERE, "rc_oracle.h"), os.path.join(HERE, "hg_oracle.h")]

A_LC, A_LC2, A_M, A_N, A_C0, A_KK, A_PENDING, A_CUR, A_PREV, A_STALE, A_AGE, A_SNAP, A_NEQ, A_COEF, \
    A_RSTAT, A_DSTAT, A_SUMPR, A_NPEND = range(18)
_DT = {A_LC: np.float32, A_LC2: np.float32, A_M: np.float32, A_N: np.float32, A_C0: np.float32,
       A_KK: np.int32, A_PENDING: np.uint8, A_CUR: np.uint32, A_PREV: np.uint32, A_STALE: np.uint32,
       A_AGE: np.float32, A_SNAP: np.float32, A_NEQ: np.float32, A_COEF: np.float32, A_RSTAT: np.float32,
       A_DSTAT: np.float32, A_SUMPR: np.float32, A_NPEND: np.int32}


class RayRec(ctypes.Structure):
    _fields_ = [("point", ctypes.c_int), ("ray", ctypes.c_int), ("q", ctypes.c_int), ("pi", ctypes.c_int),
                ("back", ctypes.c_int), ("t", ctypes.c_float)]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O3, OpenMP, no FP contraction so x86 and Arm agree)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(f) for f in SRCS + HDRS):
        tmp = LIB + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
                               *SRCS, "-o", tmp, "-lm"])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.osc_load_file.restype = ctypes.c_void_p
        L.osc_load_file.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        L.osc_load_mem.restype = ctypes.c_void_p
        L.osc_load_mem.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        L.osc_free.argtypes = [ctypes.c_void_p]
        L.osc_info.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.osc_build.argtypes = [ctypes.c_void_p]
        L.osc_state_array.restype = ctypes.c_void_p
        L.osc_state_array.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.osc_event_list.restype = ctypes.POINTER(ctypes.c_int)
        L.osc_event_list.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.osc_run_new.restype = ctypes.c_void_p
        L.osc_run_new.argtypes = [ctypes.c_void_p]
        L.osc_run_free.argtypes = [ctypes.c_void_p]
        L.osc_run_begin.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32]
        L.osc_frame.restype = ctypes.c_int
        L.osc_frame.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]
        L.osc_run_array.restype = ctypes.c_void_p
        L.osc_run_array.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.osc_run_scalar.restype = ctypes.c_int
        L.osc_run_scalar.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.osc_set_threads.argtypes = [ctypes.c_int]
        L.osc_run_set_scalar.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        fp = ctypes.POINTER(ctypes.c_float)
        L.osc_render.restype = ctypes.c_int
        L.osc_render.argtypes = [ctypes.c_void_p, ctypes.c_int, fp, fp, fp, fp, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                 ctypes.c_int, fp]
        L.osc_probe_rays.restype = ctypes.c_int
        L.osc_probe_rays.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                     ctypes.POINTER(RayRec), ctypes.c_int]
        L.osc_taa_new.restype = ctypes.c_void_p
        L.osc_taa_new.argtypes = [ctypes.c_void_p]
        L.osc_taa_free.argtypes = [ctypes.c_void_p]
        L.osc_taa_begin.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_uint32]
        L.osc_taa_frame.restype = ctypes.c_int
        L.osc_taa_frame.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)]
        L.osc_taa_array.restype = ctypes.c_void_p
        L.osc_taa_array.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
        L.osc_camera_paths.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.osc_frozen_hits.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p]
        L.osc_direct_unit.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        L.osc_trace_rays.restype = ctypes.c_int
        L.osc_trace_rays.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p]
        L.osc_path_trace.restype = ctypes.c_int
        L.osc_path_trace.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().osc_set_threads(int(n))


VERTEX_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("hit", "<f4", 3), ("to_light", "<f4", 3),
                         ("light_dist", "<f4"), ("light_index", "<i4"), ("entry", "<u4"), ("flags", "<u4")])


def dda_voxels(a, b, lo=(0.0, 0.0, 0.0), ext=(8.0, 4.0, 3.0), dims=(8, 4, 4)) -> list[int]:
    """Voxels of the dependency walk of segment a -> b (poc_gpu.cu:171-190), in order, in float32
    with every operation rounded on its own (numpy float32 scalars): the reference's sequence
    as written, against which a GPU walk is checked bit for bit.  Small cases only (pure
    Python)."""
    f = np.float32
    V = [int(x) for x in dims]
    sc = [f(V[k]) / f(ext[k]) for k in range(3)]
    A = [(f(a[k]) - f(lo[k])) * sc[k] for k in range(3)]
    B = [(f(b[k]) - f(lo[k])) * sc[k] for k in range(3)]
    i = [min(max(int(A[k]), 0), V[k] - 1) for k in range(3)]
    e = [min(max(int(B[k]), 0), V[k] - 1) for k in range(3)]
    d = [B[k] - A[k] for k in range(3)]
    st = [1 if d[k] > 0 else -1 for k in range(3)]
    with np.errstate(over="ignore", divide="ignore"):
        td = [abs(f(1) / d[k]) if d[k] != 0 else f(1e30) for k in range(3)]
        tm = [((f(i[k] + 1) - A[k]) if d[k] > 0 else (A[k] - f(i[k]))) * td[k] if d[k] != 0 else f(1e30) for k in range(3)]
    out = []
    for _ in range(sum(V)):
        out.append((i[2] * V[1] + i[1]) * V[0] + i[0])
        if i == e:
            break
        ax = 0 if (tm[0] < tm[1] and tm[0] < tm[2]) else (1 if tm[1] < tm[2] else 2)
        i[ax] += st[ax]
        tm[ax] = f(tm[ax] + td[ax])
        if i[ax] < 0 or i[ax] >= V[ax]:
            break
    return out


class _PathParams(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("fwd", ctypes.c_float * 3), ("right", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("tx", ctypes.c_float), ("ty", ctypes.c_float), ("w", ctypes.c_int), ("h", ctypes.c_int), ("bounces", ctypes.c_int),
                ("seed", ctypes.c_uint32), ("frame", ctypes.c_uint32), ("td", ctypes.c_float),
                ("lpos", (ctypes.c_float * 3) * 32), ("lrgb", (ctypes.c_float * 3) * 32), ("lint", ctypes.c_float * 32),
                ("area_corner", ctypes.c_float * 3), ("area_u", ctypes.c_float * 3), ("area_v", ctypes.c_float * 3),
                ("area_rgb", ctypes.c_float * 3), ("sun_dir", ctypes.c_float * 3), ("sun_rgb", ctypes.c_float * 3),
                ("sky_rgb", ctypes.c_float * 3)]


class Scene:
    def __init__(self, path: str | None = None, data: bytes | None = None, grid=(8, 4, 4)):
        L = lib()
        err = ctypes.create_string_buffer(256)
        if data is not None:
            self._buf = ctypes.create_string_buffer(data, len(data))
            p = L.osc_load_mem(self._buf, len(data), grid[0], grid[1], grid[2], err, 256)
        else:
            p = L.osc_load_file(path.encode(), grid[0], grid[1], grid[2], err, 256)
        if not p:
            raise ValueError("oracle: " + err.value.decode())
        self.p = p
        info = (ctypes.c_int * 10)()
        L.osc_info(p, info)
        (self.Np, self.Nq, self.Nt, self.NS, self.NL, self.NR, self.has_ref, self.fmt, self.NW, self.nst) = list(info)
        self.grid = tuple(grid)
        self.built = False

    def build(self):
        lib().osc_build(self.p)
        self.built = True

    def state_array(self, state: int, which: int) -> np.ndarray:
        nb = ctypes.c_size_t()
        ptr = lib().osc_state_array(self.p, state, which, ctypes.byref(nb))
        dt = {0: np.float32, 1: np.uint32, 2: np.float32, 3: np.uint8, 4: np.float32}[which]
        if not ptr or nb.value == 0:
            return np.zeros(0, dt)
        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)), (nb.value,)).view(dt).copy()

    def camera_paths(self, state: int, basis: dict, width: int, height: int, bounces: int, seed: int, frame: int, td: float,
                     lpos, inten, light_rgb=None, area=None, sun=None, sky=(0.0, 0.0, 0.0)) -> dict:
        """The camera-path pass (rc_hg_camera_paths) on the CPU; basis as native.camera_basis gives it,
        lpos / inten: the scene's light positions and the state's intensities."""
        if not self.built:
            self.build()
        P = _PathParams()
        for k in range(3):
            P.eye[k], P.fwd[k], P.right[k], P.up[k] = basis["eye"][k], basis["fwd"][k], basis["right"][k], basis["up"][k]
        P.tx, P.ty = basis["tx"], basis["ty"]
        P.w, P.h, P.bounces, P.seed, P.frame, P.td = width, height, bounces, seed & 0xFFFFFFFF, frame & 0xFFFFFFFF, td
        L = np.asarray(lpos, np.float32).reshape(-1, 3)
        white = light_rgb is None or not np.any(np.asarray(light_rgb))
        for l in range(self.NL):
            P.lpos[l][:] = [float(x) for x in L[l]]
            P.lrgb[l][:] = [1.0, 1.0, 1.0] if white else [float(x) for x in light_rgb[l]]
            P.lint[l] = float(inten[l])
        if area is not None:
            P.area_corner[:], P.area_u[:], P.area_v[:], P.area_rgb[:] = (list(map(float, v)) for v in area)
        if sun is not None:
            P.sun_dir[:], P.sun_rgb[:] = (list(map(float, v)) for v in sun)
        P.sky_rgb[:] = [float(x) for x in sky]
        S = bounces + 1
        n = width * height * S
        vtx = np.zeros(n, VERTEX_DTYPE)
        pos = np.zeros((n, 3), np.float32)
        nrm = np.zeros((n, 3), np.float32)
        rgb = np.zeros((n, 3), np.float32)
        ln = np.zeros(width * height, np.int32)
        img = np.zeros((width * height, 3), np.float32)
        lib().osc_camera_paths(self.p, state, ctypes.byref(P), vtx.ctypes.data, pos.ctypes.data, nrm.ctypes.data, rgb.ctypes.data,
                               ln.ctypes.data, img.ctypes.data)
        return {"vertices": vtx, "pos": pos, "nrm": nrm, "rgb": rgb, "len": ln, "image": img, "stride": S}

    def frozen_hits(self, state: int, seed: int, K: int) -> np.ndarray:
        """(Np, K) cache point reached by each of the K rays of one reference iteration, -1 = not counted."""
        out = np.empty((self.Np, K), np.int32)
        lib().osc_frozen_hits(self.p, state, seed & 0xFFFFFFFF, K, out.ctypes.data)
        return out

    def trace_rays(self, state: int, rays, watertight: bool = False):
        """Closest hit of (n, 6) rays (origin, direction) in state `state`: (prim, t) as
        rc_trace_rays returns them (prim -2 - j for static triangle j, t = +inf when no hit)."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        prim = np.empty(len(r), np.int32)
        t = np.empty(len(r), np.float32)
        if lib().osc_trace_rays(self.p, state, r.ctypes.data, len(r), 1 if watertight else 0, prim.ctypes.data, t.ctypes.data):
            raise ValueError("state out of range")
        return prim, t

    def direct_unit(self, state: int) -> np.ndarray:
        """(Np, NL) direct light of each light at unit emission (FP32)."""
        out = np.empty((self.Np, self.NL), np.float32)
        lib().osc_direct_unit(self.p, state, out.ctypes.data)
        return out

    def path_trace(self, state: int, points, paths: int = 4096, min_bounces: int = 3, seed: int = 1):
        """FP64 path-traced cache transport (summed over lights) at the points: (mean, standard error)."""
        pts = np.ascontiguousarray(points, np.int32)
        mean = np.empty(len(pts), np.float64)
        sem = np.empty(len(pts), np.float64)
        rc = lib().osc_path_trace(self.p, state, pts.ctypes.data, len(pts), paths, min_bounces, seed, mean.ctypes.data,
                                  sem.ctypes.data)
        if rc != 0:
            raise ValueError("oracle: path_trace arguments")
        return mean, sem

    def event_list(self, pair: int, kind: int) -> np.ndarray:
        n = ctypes.c_int()
        ptr = lib().osc_event_list(self.p, pair, kind, ctypes.byref(n))
        return np.array([ptr[i] for i in range(n.value)], np.int32)

    def __del__(self):
        if getattr(self, "p", None):
            lib().osc_free(self.p)
            self.p = None


class Run:
    def __init__(self, scene: Scene):
        if not scene.built:
            scene.build()
        self.scene = scene
        self.p = lib().osc_run_new(scene.p)

    def begin(self, method, s0: int, seed: int):
        from render_engine_gb300.methods import to_c
        self._cm = to_c(method)
        lib().osc_run_begin(self.p, ctypes.byref(self._cm), s0, seed & 0xFFFFFFFF)

    def frame(self, state: int, want_err: bool = False):
        e3 = (ctypes.c_double * 3)()
        ev = ctypes.c_float()
        have = lib().osc_frame(self.p, state, 1 if want_err else 0, e3, ctypes.byref(ev))
        if have < 0:
            raise ValueError("bad state")
        return (float(ev.value), tuple(e3)) if have else (None, None)

    def run(self, method, seq, seed, want_err=True):
        self.begin(method, seq[0], seed)
        errs = []
        for s in seq:
            e, _ = self.frame(s, want_err)
            if e is not None:
                errs.append(e)
        return errs

    def array(self, which: int) -> np.ndarray:
        nb = ctypes.c_size_t()
        ptr = lib().osc_run_array(self.p, which, ctypes.byref(nb))
        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)), (nb.value,)).view(_DT[which])

    def scalar(self, which: int) -> int:
        return lib().osc_run_scalar(self.p, which)

    def set_scalar(self, which: int, value: int):
        lib().osc_run_set_scalar(self.p, which, int(value))

    def probe(self, state: int, points) -> list[tuple]:
        pts = (ctypes.c_int * len(points))(*[int(x) for x in points])
        cap = 64 * len(points) + 64
        out = (RayRec * cap)()
        n = lib().osc_probe_rays(self.p, state, pts, len(points), out, cap)
        return [(r.point, r.ray, r.q, r.pi, r.back, r.t) for r in out[:n]]

    def render(self, state: int, basis: dict, w: int, h: int) -> np.ndarray:
        """basis: eye, fwd, right, up (3 floats each), tx, ty -- the float camera frame."""
        out = np.empty((h, w), np.float32)
        f = lambda k: (ctypes.c_float * 3)(*[float(x) for x in basis[k]])
        rc = lib().osc_render(self.p, state, f("eye"), f("fwd"), f("right"), f("up"), basis["tx"], basis["ty"], w, h,
                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if rc != 0:
            raise ValueError("render")
        return out

    def __del__(self):
        if getattr(self, "p", None):
            lib().osc_run_free(self.p)
            self.p = None


class Taa:
    """The taa mode of the reference (run_taa_mode, poc_gpu.cu:1175-1282) on the CPU."""

    DT = {0: np.float32, 1: np.float32, 2: np.float32, 3: np.float32, 4: np.int32, 5: np.uint8, 6: np.uint32, 7: np.uint32}

    def __init__(self, scene: Scene):
        if not scene.built:
            scene.build()
        self.scene = scene
        self.p = lib().osc_taa_new(scene.p)
        if not self.p:
            raise ValueError("oracle: taa needs a format-2 scene with references")

    def begin(self, alpha: float, gamma: float, mask: int, s0: int, seed: int):
        lib().osc_taa_begin(self.p, alpha, gamma, mask, s0, seed & 0xFFFFFFFF)

    def frame(self, state: int):
        e3 = (ctypes.c_double * 3)()
        e = ctypes.c_float()
        if lib().osc_taa_frame(self.p, state, e3, ctypes.byref(e)) != 0:
            raise ValueError("oracle: taa frame")
        return float(e.value), np.array(e3[:])

    def array(self, which: int) -> np.ndarray:
        nb = ctypes.c_size_t()
        ptr = lib().osc_taa_array(self.p, which, ctypes.byref(nb))
        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_uint8)), (nb.value,)).view(self.DT[which]).copy()

    def set_array(self, which: int, value: np.ndarray):
        nb = ctypes.c_size_t()
        ptr = lib().osc_taa_array(self.p, which, ctypes.byref(nb))
        v = np.ascontiguousarray(value, self.DT[which]).reshape(-1)
        assert v.nbytes == nb.value
        ctypes.memmove(ptr, v.ctypes.data, v.nbytes)

    def __del__(self):
        if getattr(self, "p", None):
            lib().osc_taa_free(self.p)
            self.p = None
