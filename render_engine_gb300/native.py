"""ctypes binding of the C ABI (include/rc_api.h) for Python callers, tests and the benchmark.

The binding loads ``render_engine_gb300/_build/librc_gb300.so``; when the library is missing
it raises instead of falling back to anything else.  Build it with
``python -m render_engine_gb300.build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .methods import CMethod, Method, to_c

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "librc_gb300.so")

RC_OK = 0
STATUS = {0: "ok", 1: "bad argument", 2: "i/o error", 3: "bad scene format", 4: "CUDA error", 5: "out of memory",
          6: "call out of order", 7: "device guard tripped", 8: "unsupported configuration", 9: "light count mismatch"}

(A_LC, A_LC2, A_M, A_N, A_C0, A_KK, A_PENDING, A_CUR, A_PREV, A_STALE, A_AGE, A_SNAP, A_NEQ, A_COEF, A_RSTAT,
 A_DSTAT, A_SUMPR, A_NPEND) = range(18)
ARRAY_DTYPE = {A_LC: np.float32, A_LC2: np.float32, A_M: np.float32, A_N: np.float32, A_C0: np.float32,
               A_KK: np.int32, A_PENDING: np.uint8, A_CUR: np.uint32, A_PREV: np.uint32, A_STALE: np.uint32,
               A_AGE: np.float32, A_SNAP: np.float32, A_NEQ: np.float32, A_COEF: np.float32, A_RSTAT: np.float32,
               A_DSTAT: np.float32, A_SUMPR: np.float32, A_NPEND: np.int32}
(S_PEND_LEFT, S_DORMANT, S_PROJ_LEFT, S_FRAME, S_NSLOTS, S_LAST_EVENT, S_PROJK, S_LAST_FRAME_KERNELS,
 S_LAST_FRAME_FUSED) = range(9)
SA_EDIR, SA_SV, SA_REF, SA_VALID, SA_PW = range(5)
FLAG_BRUTE_FORCE = 1
FLAG_CHECK_TRACE = 2
FLAG_WATERTIGHT = 4
FLAG_RAY_QUEUE = 8
FLAG_LOAD_ASYNC = 16   # the caller keeps the loaded bytes valid until sync(); the states after the first stream in behind the load

# Exported symbols, one per declaration of include/rc_api.h.
EXPORTS = [
    "rc_abi_version", "rc_status_string", "rc_create", "rc_destroy", "rc_last_error", "rc_device_info_get",
    "rc_scene_load", "rc_scene_load_memory", "rc_scene_info_get", "rc_state_lights", "rc_run_begin", "rc_frame",
    "rc_errors", "rc_run", "rc_sync", "rc_scene_build_states", "rc_render", "rc_array_info", "rc_array_copy", "rc_scalar_get", "rc_scalar_set",
    "rc_state_array_copy", "rc_probe_rays", "rc_trace_rays", "rc_trace_check_count", "rc_run_stats_get", "rc_device_flags",
    "rc_error_sums_noalloc", "rc_reference_build", "rc_adjoint", "rc_adjoint_arrays", "rc_taa_begin", "rc_taa_frame",
    "rc_taa_array_copy", "rc_prep_mesh", "rc_prep_mesh_params",
]
NOALLOC_MAX_POINTS = 4194304


class Config(ctypes.Structure):
    _fields_ = [("grid", ctypes.c_int * 3), ("device", ctypes.c_int), ("stream", ctypes.c_void_p),
                ("flags", ctypes.c_uint), ("expect_lights", ctypes.c_int)]


class Timers(ctypes.Structure):
    _fields_ = [("trace", ctypes.c_double), ("decide", ctypes.c_double), ("update", ctypes.c_double),
                ("swap", ctypes.c_double), ("event", ctypes.c_double), ("frames", ctypes.c_int), ("events", ctypes.c_int)]


class SceneInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("np", "nq", "nt", "ns", "nl", "nr", "has_ref", "fmt", "nw", "nst", "nnodes", "hsize")] + \
               [("scene_bytes", ctypes.c_double), ("cache_bytes", ctypes.c_double)]


class DeviceInfo(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 256), ("sm_count", ctypes.c_int), ("cc_major", ctypes.c_int),
                ("cc_minor", ctypes.c_int), ("mem_used_mb", ctypes.c_double), ("mem_total_mb", ctypes.c_double)]


class Camera(ctypes.Structure):
    _fields_ = [("eye", ctypes.c_float * 3), ("at", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("fov_y_deg", ctypes.c_float), ("width", ctypes.c_int), ("height", ctypes.c_int)]


def camera(eye, at, up=(0.0, 0.0, 1.0), fov_y_deg=70.0, width=1920, height=1080) -> Camera:
    c = Camera()
    c.eye[:] = [float(x) for x in eye]
    c.at[:] = [float(x) for x in at]
    c.up[:] = [float(x) for x in up]
    c.fov_y_deg = float(fov_y_deg)
    c.width, c.height = int(width), int(height)
    return c


class RunStats(ctypes.Structure):
    _fields_ = [("frames", ctypes.c_longlong), ("rays", ctypes.c_longlong), ("launches", ctypes.c_longlong),
                ("last_frame_kernels", ctypes.c_int), ("last_frame_fused", ctypes.c_int), ("last_frame_event", ctypes.c_int)]


class RayRec(ctypes.Structure):
    _fields_ = [("point", ctypes.c_int), ("ray", ctypes.c_int), ("q", ctypes.c_int), ("pi", ctypes.c_int),
                ("back", ctypes.c_int), ("t", ctypes.c_float), ("dir", ctypes.c_float * 3), ("hit", ctypes.c_float * 3)]


_lib = None


def load_library():
    """Load the native library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("render_engine_gb300: native library missing (%s); run the build first" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, i, u32, sz = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_uint32, ctypes.c_size_t
    L.rc_abi_version.restype = i
    L.rc_status_string.restype = ctypes.c_char_p
    L.rc_status_string.argtypes = [i]
    L.rc_create.restype = i
    L.rc_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    L.rc_destroy.argtypes = [vp]
    L.rc_last_error.restype = ctypes.c_char_p
    L.rc_last_error.argtypes = [vp]
    L.rc_device_info_get.restype = i
    L.rc_device_info_get.argtypes = [vp, ctypes.POINTER(DeviceInfo)]
    L.rc_scene_load.restype = i
    L.rc_scene_load.argtypes = [vp, ctypes.c_char_p]
    L.rc_scene_load_memory.restype = i
    L.rc_scene_load_memory.argtypes = [vp, vp, sz]
    L.rc_scene_info_get.restype = i
    L.rc_scene_info_get.argtypes = [vp, ctypes.POINTER(SceneInfo)]
    L.rc_state_lights.restype = i
    L.rc_state_lights.argtypes = [vp, i, ctypes.POINTER(ctypes.c_float), i]
    L.rc_run_begin.restype = i
    L.rc_run_begin.argtypes = [vp, ctypes.POINTER(CMethod), i, u32]
    L.rc_frame.restype = i
    L.rc_frame.argtypes = [vp, i, i]
    L.rc_errors.restype = i
    L.rc_errors.argtypes = [vp, ctypes.POINTER(ctypes.c_float), i, ip]
    L.rc_run.restype = i
    L.rc_run.argtypes = [vp, ctypes.POINTER(CMethod), ip, i, u32, i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(Timers)]
    L.rc_sync.restype = i
    L.rc_sync.argtypes = [vp]
    L.rc_scene_build_states.restype = i
    L.rc_scene_build_states.argtypes = [vp]
    L.rc_render.restype = i
    L.rc_render.argtypes = [vp, i, ctypes.POINTER(Camera), ctypes.POINTER(ctypes.c_float), sz]
    L.rc_array_info.restype = i
    L.rc_array_info.argtypes = [vp, i, ctypes.POINTER(sz), ctypes.POINTER(vp)]
    L.rc_array_copy.restype = i
    L.rc_array_copy.argtypes = [vp, i, vp, sz, i]
    L.rc_scalar_get.restype = i
    L.rc_scalar_get.argtypes = [vp, i, ip]
    L.rc_scalar_set.restype = i
    L.rc_scalar_set.argtypes = [vp, i, i]
    L.rc_state_array_copy.restype = i
    L.rc_state_array_copy.argtypes = [vp, i, i, vp, sz]
    L.rc_probe_rays.restype = i
    L.rc_probe_rays.argtypes = [vp, i, ip, i, ctypes.POINTER(RayRec), i, ip]
    L.rc_trace_check_count.restype = i
    L.rc_trace_check_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_longlong)]
    L.rc_run_stats_get.restype = i
    L.rc_run_stats_get.argtypes = [vp, ctypes.POINTER(RunStats)]
    L.rc_trace_rays.restype = i
    L.rc_trace_rays.argtypes = [vp, i, vp, i, vp, vp]
    L.rc_device_flags.restype = i
    L.rc_device_flags.argtypes = [vp, ctypes.POINTER(ctypes.c_uint)]
    L.rc_reference_build.restype = i
    L.rc_reference_build.argtypes = [vp, ctypes.POINTER(RefParams), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]
    L.rc_error_sums_noalloc.restype = i
    L.rc_error_sums_noalloc.argtypes = [vp, i, i, i, vp, vp, i, vp, vp]
    L.rc_adjoint.restype = i
    L.rc_adjoint.argtypes = [vp, ctypes.POINTER(AdjointParams), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(AdjointResult)]
    L.rc_adjoint_arrays.restype = i
    L.rc_adjoint_arrays.argtypes = [vp, vp, vp, vp]
    L.rc_prep_mesh.restype = i
    L.rc_prep_mesh.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, i, ctypes.POINTER(PrepReport)]
    L.rc_prep_mesh_params.restype = i
    L.rc_prep_mesh_params.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(PrepParams), ctypes.POINTER(PrepReport)]
    L.rc_taa_begin.restype = i
    L.rc_taa_begin.argtypes = [vp, ctypes.POINTER(TaaMethod), i, u32]
    L.rc_taa_frame.restype = i
    L.rc_taa_frame.argtypes = [vp, i, ctypes.POINTER(ctypes.c_float)]
    L.rc_taa_array_copy.restype = i
    L.rc_taa_array_copy.argtypes = [vp, i, vp, sz, i]
    _lib = L
    return L


class RefParams(ctypes.Structure):
    _fields_ = [("K", ctypes.c_int), ("warmup", ctypes.c_int), ("block", ctypes.c_int), ("max_iter", ctypes.c_int),
                ("noise_target", ctypes.c_double)]


class TaaMethod(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_float), ("gamma", ctypes.c_float), ("mask", ctypes.c_int)]


(T_X, T_H, T_MU, T_SG, T_REACT, T_PEND, T_CUR, T_PREV) = range(8)
TAA_DTYPE = {T_X: np.float32, T_H: np.float32, T_MU: np.float32, T_SG: np.float32, T_REACT: np.int32, T_PEND: np.uint8,
             T_CUR: np.uint32, T_PREV: np.uint32}


class PrepReport(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_int), ("np", ctypes.c_int), ("zones", ctypes.c_int), ("bvh_nodes", ctypes.c_int),
                ("ns", ctypes.c_int), ("cell_m", ctypes.c_float), ("diag_m", ctypes.c_float), ("cube_m", ctypes.c_float),
                ("valid_fraction", ctypes.c_double), ("noise", ctypes.c_double * 8), ("iterations", ctypes.c_int * 8),
                ("nl", ctypes.c_int), ("bvh_depth", ctypes.c_int), ("lights", (ctypes.c_float * 3) * 32), ("seconds", ctypes.c_double)]


class PrepParams(ctypes.Structure):
    _fields_ = [("target_points", ctypes.c_int), ("lamps", ctypes.c_int), ("seed", ctypes.c_uint32),
                ("ref_iterations", ctypes.c_int)]


class AdjointParams(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("K", ctypes.c_int), ("seed", ctypes.c_uint32), ("iterations", ctypes.c_int),
                ("emission", ctypes.POINTER(ctypes.c_float))]


class AdjointResult(ctypes.Structure):
    _fields_ = [("J", ctypes.c_double), ("J_grad", ctypes.c_double), ("fwd_change", ctypes.c_double),
                ("adj_change", ctypes.c_double), ("rays", ctypes.c_longlong), ("back", ctypes.c_longlong),
                ("max_incoming", ctypes.c_int)]


class RCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Context:
    """One radiance-cache context on one GPU (rc_create / rc_destroy)."""

    def __init__(self, grid=(8, 4, 4), device: int = 0, flags: int = 0, expect_lights: int = 0, stream: int | None = None):
        self.L = load_library()
        cfg = Config()
        cfg.grid[0], cfg.grid[1], cfg.grid[2] = grid
        cfg.device = device
        cfg.flags = flags
        cfg.expect_lights = expect_lights
        cfg.stream = stream
        h = ctypes.c_void_p()
        st = self.L.rc_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != RC_OK:
            raise RCError(st, "rc_create failed (is a GPU available?)")
        self.h = h
        self.grid = tuple(grid)

    def _chk(self, st: int):
        if st != RC_OK:
            raise RCError(st, self.L.rc_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.L.rc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def device_info(self) -> dict:
        d = DeviceInfo()
        self._chk(self.L.rc_device_info_get(self.h, ctypes.byref(d)))
        return {"name": d.name.decode(), "sm_count": d.sm_count, "cc": (d.cc_major, d.cc_minor),
                "mem_used_mb": d.mem_used_mb, "mem_total_mb": d.mem_total_mb}

    def load(self, path: str):
        self._chk(self.L.rc_scene_load(self.h, path.encode()))
        return self.info()

    def load_bytes(self, data):
        buf = data if isinstance(data, np.ndarray) else np.frombuffer(data, np.uint8)
        self._chk(self.L.rc_scene_load_memory(self.h, buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes))
        return self.info()

    def info(self) -> dict:
        s = SceneInfo()
        self._chk(self.L.rc_scene_info_get(self.h, ctypes.byref(s)))
        self._info = {n: getattr(s, n) for n, _ in SceneInfo._fields_}
        return self._info

    def state_lights(self, state: int) -> np.ndarray:
        nl = self._info["nl"]
        out = (ctypes.c_float * nl)()
        self._chk(self.L.rc_state_lights(self.h, state, out, nl))
        return np.array(out[:], np.float32)

    def begin(self, method: Method, s0: int, seed: int):
        self._cm = to_c(method)
        self._chk(self.L.rc_run_begin(self.h, ctypes.byref(self._cm), s0, seed & 0xFFFFFFFF))

    def frame(self, state: int, want_err: bool = False):
        self._chk(self.L.rc_frame(self.h, state, 1 if want_err else 0))

    def errors(self) -> np.ndarray:
        n = ctypes.c_int()
        self._chk(self.L.rc_errors(self.h, None, 0, ctypes.byref(n)))
        out = (ctypes.c_float * max(n.value, 1))()
        self._chk(self.L.rc_errors(self.h, out, n.value, ctypes.byref(n)))
        return np.array(out[: n.value], np.float32)

    def run(self, method: Method, seq, seed: int, want_err: bool = True, timers: bool = False):
        cm = to_c(method)
        arr = (ctypes.c_int * len(seq))(*[int(x) for x in seq])
        errs = (ctypes.c_float * len(seq))()
        tm = Timers() if timers else None
        self._chk(self.L.rc_run(self.h, ctypes.byref(cm), arr, len(seq), seed & 0xFFFFFFFF, 1 if want_err else 0,
                                errs if want_err else None, ctypes.byref(tm) if timers else None))
        out = np.array(errs[:], np.float32) if want_err else None
        if timers:
            return out, {n: getattr(tm, n) for n, _ in Timers._fields_}
        return out

    def sync(self):
        self._chk(self.L.rc_sync(self.h))

    def build_states(self):
        """Issue every state's build now (rc_scene_build_states); sync() waits for them."""
        self._chk(self.L.rc_scene_build_states(self.h))

    def render(self, state: int, cam: Camera, copy: bool = True):
        """Image pass from the current cache; returns an (h, w) float32 image when copy."""
        if not copy:
            self._chk(self.L.rc_render(self.h, state, ctypes.byref(cam), None, 0))
            return None
        img = np.empty((cam.height, cam.width), np.float32)
        self._chk(self.L.rc_render(self.h, state, ctypes.byref(cam), img.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), img.size))
        return img

    def array(self, which: int, out: np.ndarray | None = None) -> np.ndarray:
        """Copy one cache array to the host; into `out` (for instance a view of pinned memory)
        when given, which must hold exactly the array's bytes."""
        n = ctypes.c_size_t()
        self._chk(self.L.rc_array_info(self.h, which, ctypes.byref(n), None))
        if out is None:
            out = np.empty(n.value // np.dtype(ARRAY_DTYPE[which]).itemsize, ARRAY_DTYPE[which])
        elif out.nbytes != n.value or not out.flags.c_contiguous:
            raise ValueError("out holds %d bytes, the array %d" % (out.nbytes, n.value))
        self._chk(self.L.rc_array_copy(self.h, which, out.ctypes.data_as(ctypes.c_void_p), out.nbytes, 0))
        return out

    def set_array(self, which: int, a: np.ndarray):
        a = np.ascontiguousarray(a, ARRAY_DTYPE[which])
        self._chk(self.L.rc_array_copy(self.h, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1))

    def device_ptr(self, which: int) -> int:
        n = ctypes.c_size_t()
        p = ctypes.c_void_p()
        self._chk(self.L.rc_array_info(self.h, which, ctypes.byref(n), ctypes.byref(p)))
        return p.value

    def scalar(self, which: int) -> int:
        v = ctypes.c_int()
        self._chk(self.L.rc_scalar_get(self.h, which, ctypes.byref(v)))
        return v.value

    def set_scalar(self, which: int, value: int):
        self._chk(self.L.rc_scalar_set(self.h, which, int(value)))

    def state_array(self, state: int, which: int) -> np.ndarray:
        inf = self._info
        np_, nl, nw = inf["np"], inf["nl"], inf["nw"]
        shape, dt = {SA_EDIR: (nl * np_, np.float32), SA_SV: (nw * np_, np.uint32), SA_REF: (np_, np.float32),
                     SA_VALID: (np_, np.uint8), SA_PW: (nl * np_, np.float32)}[which]
        a = np.empty(shape, dt)
        self._chk(self.L.rc_state_array_copy(self.h, state, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes))
        return a

    def probe(self, state: int, points) -> list[tuple]:
        pts = (ctypes.c_int * len(points))(*[int(x) for x in points])
        cap = 64 * len(points) + 64
        out = (RayRec * cap)()
        n = ctypes.c_int()
        self._chk(self.L.rc_probe_rays(self.h, state, pts, len(points), out, cap, ctypes.byref(n)))
        return sorted((r.point, r.ray, r.q, r.pi, r.back, r.t) for r in out[: n.value])

    def trace_rays(self, state: int, rays):
        """rc_trace_rays: closest hit of (n, 6) rays (origin, direction) in state `state`;
        returns (prim, t) with prim -2 - j for static triangle j and t = +inf when no hit."""
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        prim = np.empty(len(r), np.int32)
        t = np.empty(len(r), np.float32)
        self._chk(self.L.rc_trace_rays(self.h, state, r.ctypes.data, len(r), prim.ctypes.data, t.ctypes.data))
        return prim, t

    def probe_full(self, state: int, points) -> list[dict]:
        """rc_probe_rays with every field: also the direction and the end point of each ray."""
        pts = (ctypes.c_int * len(points))(*[int(x) for x in points])
        cap = 64 * len(points) + 64
        out = (RayRec * cap)()
        n = ctypes.c_int()
        self._chk(self.L.rc_probe_rays(self.h, state, pts, len(points), out, cap, ctypes.byref(n)))
        recs = [dict(point=r.point, ray=r.ray, q=r.q, pi=r.pi, back=r.back, t=r.t,
                     dir=np.array(r.dir[:], np.float32), hit=np.array(r.hit[:], np.float32)) for r in out[: n.value]]
        return sorted(recs, key=lambda d: (d["point"], d["ray"]))

    def check_count(self) -> tuple[int, int]:
        a, b = ctypes.c_longlong(), ctypes.c_longlong()
        self._chk(self.L.rc_trace_check_count(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def stats(self) -> dict:
        st = RunStats()
        self._chk(self.L.rc_run_stats_get(self.h, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in RunStats._fields_}

    def build_reference(self, K: int = 32, warmup: int = 16, block: int = 64, max_iter: int = 2048, noise_target: float = 0.03):
        """Converged references of every state (rc_reference_build); returns (noise, iterations) per state."""
        ns = self._info["ns"]
        noise = (ctypes.c_double * ns)()
        iters = (ctypes.c_int * ns)()
        prm = RefParams(K, warmup, block, max_iter, noise_target)
        self._chk(self.L.rc_reference_build(self.h, ctypes.byref(prm), noise, iters))
        self._info = self.info()
        return list(noise), list(iters)

    def adjoint(self, state: int, weights, K: int = 32, seed: int = 0, iterations: int = 64, emission=None):
        """dJ/dE per light for J = sum_i w_i sum_l L_l[i] over K frozen rays per point (rc_adjoint);
        returns (gradient, result dict).  emission: the lights' emissions of the forward solve
        (None = the state's)."""
        nl, np_ = self._info["nl"], self._info["np"]
        w = np.ascontiguousarray(weights, np.float32)
        if w.shape != (np_,):
            raise ValueError("weights must have one entry per cache point")
        g = (ctypes.c_float * nl)()
        res = AdjointResult()
        prm = AdjointParams(state, K, seed & 0xFFFFFFFF, iterations, None)
        if emission is not None:
            em = np.ascontiguousarray(emission, np.float32)
            if em.shape != (nl,):
                raise ValueError("emission must have one entry per light")
            prm.emission = em.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        self._chk(self.L.rc_adjoint(self.h, ctypes.byref(prm), w.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), g, ctypes.byref(res)))
        self._adj_k = K
        return np.array(g[:], np.float32), {n: getattr(res, n) for n, _ in AdjointResult._fields_}

    def adjoint_arrays(self) -> tuple:
        """(L, u, hits) of the last adjoint call: forward solution, importance, frozen hit points (Np x K)."""
        np_ = self._info["np"]
        L = np.empty(np_, np.float32)
        u = np.empty(np_, np.float32)
        h = np.empty((np_, self._adj_k), np.int32)
        self._chk(self.L.rc_adjoint_arrays(self.h, L.ctypes.data, u.ctypes.data, h.ctypes.data))
        return L, u, h

    def prep_mesh(self, mesh_path: str, scene_path: str, points: int = 300000, lamps: int = 3, seed: int = 1,
                  ref_iterations: int = 0) -> dict:
        """Prepare a format-3 scene from an MSH1 mesh (rc_prep_mesh_params); the scene stays loaded.
        ref_iterations < 0: no references."""
        r = PrepReport()
        p = PrepParams(points, lamps, seed & 0xFFFFFFFF, ref_iterations)
        self._chk(self.L.rc_prep_mesh_params(self.h, mesh_path.encode(), scene_path.encode(), ctypes.byref(p), ctypes.byref(r)))
        self.info()
        return {"triangles": r.triangles, "np": r.np, "zones": r.zones, "bvh_nodes": r.bvh_nodes, "bvh_depth": r.bvh_depth,
                "cell_m": r.cell_m, "diag_m": r.diag_m, "cube_m": r.cube_m, "valid_fraction": r.valid_fraction,
                "noise": list(r.noise[:r.ns]), "iterations": list(r.iterations[:r.ns]),
                "lights": [list(r.lights[l]) for l in range(r.nl)], "seconds": r.seconds}

    def taa_begin(self, alpha: float, gamma: float, mask: int, s0: int, seed: int):
        """Start a run of the taa mode (rc_taa_begin)."""
        m = TaaMethod(alpha, gamma, mask)
        self._chk(self.L.rc_taa_begin(self.h, ctypes.byref(m), s0, seed & 0xFFFFFFFF))

    def taa_frame(self, state: int, want_err: bool = False):
        e = ctypes.c_float()
        self._chk(self.L.rc_taa_frame(self.h, state, ctypes.byref(e) if want_err else None))
        return float(e.value) if want_err else None

    def taa_array(self, which: int, value: np.ndarray | None = None) -> np.ndarray:
        """Copy a taa array out (value None) or in."""
        np_, nw = self._info["np"], self._info["nw"]
        n = np_ * nw if which in (T_CUR, T_PREV) else np_
        dt = TAA_DTYPE[which]
        if value is None:
            out = np.empty(n, dt)
            self._chk(self.L.rc_taa_array_copy(self.h, which, out.ctypes.data, out.nbytes, 0))
            return out
        v = np.ascontiguousarray(value, dt).reshape(-1)
        self._chk(self.L.rc_taa_array_copy(self.h, which, v.ctypes.data, v.nbytes, 1))
        return v

    def device_flags(self) -> int:
        v = ctypes.c_uint()
        self._chk(self.L.rc_device_flags(self.h, ctypes.byref(v)))
        return v.value


def camera_basis(cam: Camera) -> dict:
    """The float camera frame rc_render derives from a Camera (same double arithmetic)."""
    import math
    f = [float(cam.at[k]) - float(cam.eye[k]) for k in range(3)]
    fl = math.sqrt(sum(x * x for x in f))
    f = [x / fl for x in f]
    u0 = [float(cam.up[k]) for k in range(3)]
    r = [f[1] * u0[2] - f[2] * u0[1], f[2] * u0[0] - f[0] * u0[2], f[0] * u0[1] - f[1] * u0[0]]
    rl = math.sqrt(sum(x * x for x in r))
    r = [x / rl for x in r]
    u = [r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]]
    ty = np.float32(math.tan(0.5 * float(cam.fov_y_deg) * math.pi / 180.0))
    tx = np.float32(ty * np.float32(cam.width) / np.float32(cam.height))
    return {"eye": [float(cam.eye[k]) for k in range(3)], "fwd": [float(np.float32(x)) for x in f],
            "right": [float(np.float32(x)) for x in r], "up": [float(np.float32(x)) for x in u], "tx": float(tx), "ty": float(ty)}


def error_sums_noalloc(lc_ptr: int, lc_stride: int, nl: int, dormant: int, ref_ptr: int, valid_ptr: int, np_: int,
                       out3_ptr: int, stream: int | None = None) -> None:
    """rc_error_sums_noalloc on caller-owned device buffers (raw device addresses); the three
    FP64 sums land in out3 asynchronously on `stream`.  Allocates no device memory."""
    L = load_library()
    st = L.rc_error_sums_noalloc(lc_ptr, lc_stride, nl, dormant, ref_ptr, valid_ptr, np_, out3_ptr, stream)
    if st != RC_OK:
        raise RCError(st, "rc_error_sums_noalloc (np=%d, limit %d)" % (np_, NOALLOC_MAX_POINTS))
