"""ctypes front end of the hash-grid cache with dependency masks (include/rc_hashgrid.h).

The cache lives on the GPU; the calls take device buffers (torch CUDA tensors, or raw device
pointers as ints) and run on the cache's stream.  The library must be built
(``__graft_entry__.build()``); nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native

EXPORTS = ["rc_hg_create", "rc_hg_destroy", "rc_hg_last_error", "rc_hg_array", "rc_hg_array_copy", "rc_hg_clear", "rc_hg_insert",
           "rc_hg_accumulate", "rc_hg_begin_frame", "rc_hg_mark_paths", "rc_hg_resolve", "rc_hg_event_mask",
           "rc_hg_snapshot", "rc_hg_restore", "rc_hg_mark_paths_strided", "rc_hg_voxels_init", "rc_hg_voxels_clear",
           "rc_hg_voxels_mark", "rc_hg_voxels_box_lights", "rc_hg_voxels_copy", "rc_hg_camera_paths", "rc_hg_camera_arrays"]

INVALID = 0xFFFFFFFF
EVICTED = 0xFFFFFFFFFFFFFFFF
MISS, LIGHT_VISIBLE, STOP = 1, 2, 4
SKY_BIT = 0x80000000
A_KEYS, A_ACCUM, A_RESOLVED, A_BANK0, A_BANK1 = range(5)


class Config(ctypes.Structure):
    _fields_ = [("zone_lo", ctypes.c_float * 3), ("zone_hi", ctypes.c_float * 3), ("origin", ctypes.c_float * 3),
                ("cell", ctypes.c_float), ("capacity", ctypes.c_uint32), ("max_depth", ctypes.c_int),
                ("acc_frames", ctypes.c_int), ("stale_frames", ctypes.c_int), ("tracing_distance", ctypes.c_float),
                ("device", ctypes.c_int), ("stream", ctypes.c_void_p)]


# rc_hg_vertex as a numpy record (64 bytes), for building path batches on the host
VERTEX_DTYPE = np.dtype([("origin", "<f4", 3), ("dir", "<f4", 3), ("hit", "<f4", 3), ("to_light", "<f4", 3),
                         ("light_dist", "<f4"), ("light_index", "<i4"), ("entry", "<u4"), ("flags", "<u4")])
SNAP_DTYPE = np.dtype([("index", "<u4"), ("sample_data", "<u4"), ("key", "<u4", 2), ("radiance", "<u4", 2)])
assert VERTEX_DTYPE.itemsize == 64 and SNAP_DTYPE.itemsize == 24


def make_config(zone_lo=(0.0, 0.0, 0.0), zone_hi=(8.0, 4.0, 3.0), origin=(0.0, 0.0, 0.0), cell=0.25, capacity=1 << 16,
                max_depth=4, acc_frames=64, stale_frames=32, tracing_distance=1000.0, device=0, stream=None) -> Config:
    c = Config()
    c.zone_lo[:] = zone_lo
    c.zone_hi[:] = zone_hi
    c.origin[:] = origin
    c.cell = cell
    c.capacity = capacity
    c.max_depth = max_depth
    c.acc_frames = acc_frames
    c.stale_frames = stale_frames
    c.tracing_distance = tracing_distance
    c.device = device
    c.stream = stream
    return c


_bound = False


def _lib():
    global _bound
    L = native.load_library()
    if not _bound:
        vp, i, u32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32
        fp = ctypes.POINTER(ctypes.c_float)
        L.rc_hg_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.rc_hg_destroy.argtypes = [vp]
        L.rc_hg_destroy.restype = None
        L.rc_hg_last_error.argtypes = [vp]
        L.rc_hg_last_error.restype = ctypes.c_char_p
        L.rc_hg_array.argtypes = [vp, i, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t)]
        L.rc_hg_array_copy.argtypes = [vp, i, vp, ctypes.c_size_t, i]
        L.rc_hg_clear.argtypes = [vp]
        L.rc_hg_insert.argtypes = [vp, vp, vp, i, vp]
        L.rc_hg_accumulate.argtypes = [vp, vp, vp, i]
        L.rc_hg_begin_frame.argtypes = [vp, u32, u32]
        L.rc_hg_mark_paths.argtypes = [vp, vp, vp, i]
        L.rc_hg_resolve.argtypes = [vp, ctypes.POINTER(u32), vp]
        fp = ctypes.POINTER(ctypes.c_float)
        L.rc_hg_event_mask.argtypes = [ctypes.POINTER(Config), fp, fp, i, i, i, fp, fp, ctypes.POINTER(u32)]
        L.rc_hg_event_mask.restype = None
        L.rc_hg_snapshot.argtypes = [vp, vp, u32, ctypes.POINTER(u32)]
        L.rc_hg_restore.argtypes = [vp, vp, u32]
        L.rc_hg_mark_paths_strided.argtypes = [vp, vp, vp, i, i]
        L.rc_hg_voxels_init.argtypes = [vp, i]
        L.rc_hg_voxels_clear.argtypes = [vp]
        L.rc_hg_voxels_mark.argtypes = [vp, vp, vp, i, i]
        L.rc_hg_voxels_box_lights.argtypes = [vp, fp, fp, ctypes.POINTER(ctypes.c_uint64)]
        L.rc_hg_voxels_copy.argtypes = [vp, vp, ctypes.c_size_t]
        L.rc_hg_camera_paths.argtypes = [vp, vp, i, ctypes.POINTER(PathParams), vp]
        L.rc_hg_camera_arrays.argtypes = [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                          ctypes.POINTER(i), ctypes.POINTER(i)]
        _bound = True
    return L


class PathParams(ctypes.Structure):
    """rc_hg_path_params: camera, bounces, seed/frame, light colours, rectangle light, sun, sky."""
    _fields_ = [("cam", native.Camera), ("bounces", ctypes.c_int), ("seed", ctypes.c_uint32), ("frame", ctypes.c_uint32),
                ("light_rgb", (ctypes.c_float * 3) * 32), ("area_corner", ctypes.c_float * 3), ("area_u", ctypes.c_float * 3),
                ("area_v", ctypes.c_float * 3), ("area_rgb", ctypes.c_float * 3), ("sun_dir", ctypes.c_float * 3),
                ("sun_rgb", ctypes.c_float * 3), ("sky_rgb", ctypes.c_float * 3)]


def path_params(cam, bounces=2, seed=1, frame=0, light_rgb=None, area=None, sun=None, sky=(0.0, 0.0, 0.0)) -> PathParams:
    """area = (corner, u, v, rgb), sun = (direction, rgb); None = absent."""
    p = PathParams()
    p.cam = cam
    p.bounces = bounces
    p.seed = seed & 0xFFFFFFFF
    p.frame = frame & 0xFFFFFFFF
    if light_rgb is not None:
        for l, c in enumerate(light_rgb):
            p.light_rgb[l][:] = [float(x) for x in c]
    if area is not None:
        p.area_corner[:], p.area_u[:], p.area_v[:], p.area_rgb[:] = (list(map(float, v)) for v in area)
    if sun is not None:
        p.sun_dir[:], p.sun_rgb[:] = (list(map(float, v)) for v in sun)
    p.sky_rgb[:] = [float(x) for x in sky]
    return p


def _ptr(x) -> int:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def event_mask(cfg: Config, lights_a=None, lights_b=None, sky_a=0, sky_b=0, obj_a=None, obj_b=None) -> np.ndarray:
    """Zones and lights an event between two states invalidates (host only)."""
    L = _lib()
    fp = ctypes.POINTER(ctypes.c_float)

    def arr(v):
        if v is None:
            return None
        a = np.ascontiguousarray(v, np.float32)
        return a.ctypes.data_as(fp), a

    la, lb, oa, ob = arr(lights_a), arr(lights_b), arr(obj_a), arr(obj_b)
    n = 0 if la is None else len(la[1])
    inv = (ctypes.c_uint32 * 4)()
    L.rc_hg_event_mask(ctypes.byref(cfg), la[0] if la else None, lb[0] if lb else None, n, sky_a, sky_b,
                       oa[0] if oa else None, ob[0] if ob else None, inv)
    return np.array(inv[:], np.uint32)


class HashGrid:
    """One hash-grid cache on one GPU (rc_hg_create / rc_hg_destroy)."""

    def __init__(self, cfg: Config):
        self.L = _lib()
        self.cfg = cfg
        h = ctypes.c_void_p()
        st = self.L.rc_hg_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != native.RC_OK:
            raise native.RCError(st, "rc_hg_create failed")
        self.h = h

    def _chk(self, st):
        if st != native.RC_OK:
            raise native.RCError(st, self.L.rc_hg_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.L.rc_hg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def array_ptr(self, which: int) -> tuple[int, int]:
        p, n = ctypes.c_void_p(), ctypes.c_size_t()
        self._chk(self.L.rc_hg_array(self.h, which, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    _DT = {A_KEYS: (np.uint64, 1), A_ACCUM: (np.uint32, 4), A_RESOLVED: (np.uint32, 4), A_BANK0: (np.uint32, 4),
           A_BANK1: (np.uint32, 4)}

    def download(self, which: int) -> np.ndarray:
        dt, w = self._DT[which]
        a = np.empty((self.cfg.capacity, w) if w > 1 else self.cfg.capacity, dt)
        self._chk(self.L.rc_hg_array_copy(self.h, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 0))
        return a

    def upload(self, which: int, a: np.ndarray):
        dt, _ = self._DT[which]
        a = np.ascontiguousarray(a, dt)
        self._chk(self.L.rc_hg_array_copy(self.h, which, a.ctypes.data_as(ctypes.c_void_p), a.nbytes, 1))

    def clear(self):
        self._chk(self.L.rc_hg_clear(self.h))

    def insert(self, pos, nrm, entry):
        self._chk(self.L.rc_hg_insert(self.h, _ptr(pos), _ptr(nrm), int(entry.shape[0]), _ptr(entry)))

    def accumulate(self, entry, rgb):
        self._chk(self.L.rc_hg_accumulate(self.h, _ptr(entry), _ptr(rgb), int(entry.shape[0])))

    def begin_frame(self, dep_frame: int, period: int = 16):
        self._chk(self.L.rc_hg_begin_frame(self.h, dep_frame, period))

    def mark_paths(self, vertices, path_start, npaths: int):
        self._chk(self.L.rc_hg_mark_paths(self.h, _ptr(vertices), _ptr(path_start), npaths))

    def resolve(self, inv=None, counts=None):
        iv = (ctypes.c_uint32 * 4)(*([0, 0, 0, 0] if inv is None else [int(x) for x in inv]))
        self._chk(self.L.rc_hg_resolve(self.h, iv, _ptr(counts)))

    def snapshot(self, recs, cap: int) -> int:
        n = ctypes.c_uint32()
        self._chk(self.L.rc_hg_snapshot(self.h, _ptr(recs), cap, ctypes.byref(n)))
        return n.value

    def restore(self, recs, count: int):
        self._chk(self.L.rc_hg_restore(self.h, _ptr(recs), count))

    def mark_paths_strided(self, vertices, lengths, stride: int, npaths: int):
        self._chk(self.L.rc_hg_mark_paths_strided(self.h, _ptr(vertices), _ptr(lengths), stride, npaths))

    # per-voxel light masks
    def voxels_init(self, res: int):
        self._chk(self.L.rc_hg_voxels_init(self.h, res))
        self.vres = res

    def voxels_clear(self):
        self._chk(self.L.rc_hg_voxels_clear(self.h))

    def voxels_mark(self, vertices, lengths, stride: int, npaths: int):
        self._chk(self.L.rc_hg_voxels_mark(self.h, _ptr(vertices), _ptr(lengths), stride, npaths))

    def voxels_box_lights(self, lo, hi) -> int:
        fp = ctypes.POINTER(ctypes.c_float)
        a = np.ascontiguousarray(lo, np.float32)
        b = np.ascontiguousarray(hi, np.float32)
        m = ctypes.c_uint64()
        self._chk(self.L.rc_hg_voxels_box_lights(self.h, a.ctypes.data_as(fp), b.ctypes.data_as(fp), ctypes.byref(m)))
        return m.value

    def voxels(self) -> np.ndarray:
        n = self.vres ** 3
        out = np.empty(n, np.uint64)
        self._chk(self.L.rc_hg_voxels_copy(self.h, out.ctypes.data_as(ctypes.c_void_p), n))
        return out

    # camera paths over a context's scene
    def camera_paths(self, ctx, state: int, params: PathParams, image=None):
        self._chk(self.L.rc_hg_camera_paths(self.h, ctx.h, state, ctypes.byref(params), _ptr(image)))


def camera_arrays(ctx) -> dict:
    """Host copies of the last camera pass: vertices (VERTEX_DTYPE), rgb, entry (per slot), lengths (per path)."""
    import torch
    L = _lib()
    vp = ctypes.c_void_p
    v, r, e, ln = vp(), vp(), vp(), vp()
    stride, npaths = ctypes.c_int(), ctypes.c_int()
    st = L.rc_hg_camera_arrays(ctx.h, ctypes.byref(v), ctypes.byref(r), ctypes.byref(e), ctypes.byref(ln), ctypes.byref(stride),
                               ctypes.byref(npaths))
    if st != native.RC_OK:
        raise native.RCError(st, ctx.L.rc_last_error(ctx.h).decode())
    ns = stride.value * npaths.value

    class _Dev:   # a device buffer torch can view (CUDA array interface)
        def __init__(self, ptr, nbytes):
            self.__cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False), "strides": None,
                                             "version": 3}

    def grab(ptr, nbytes):
        torch.cuda.synchronize()
        return torch.as_tensor(_Dev(ptr, nbytes), device="cuda").cpu().numpy()

    return {"vertices": grab(v.value, 64 * ns).view(VERTEX_DTYPE), "rgb": grab(r.value, 12 * ns).view(np.float32).reshape(-1, 3),
            "entry": grab(e.value, 4 * ns).view(np.uint32), "len": grab(ln.value, 4 * npaths.value).view(np.int32),
            "stride": stride.value, "npaths": npaths.value}
