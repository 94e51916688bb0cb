"""ctypes front end of the tensor-core radiance cache (include/rc_mlp.h).

Calls take CUDA tensors (or raw device pointers as ints); the library must be built
(``__graft_entry__.build()``); nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native

EXPORTS = ["rc_mlp_tile_product", "rc_mlp_wait_check", "rc_mlp_create", "rc_mlp_destroy", "rc_mlp_last_error", "rc_mlp_train", "rc_mlp_infer",
           "rc_mlp_weights", "rc_mlp_gradients", "rc_mlp_error_flags", "rc_mlp_loss_scale"]
NWEIGHT = 24576
LAYERS = [(176, 64), (64, 64), (64, 64), (64, 64), (64, 16)]   # (inputs, outputs)


class Config(ctypes.Structure):
    _fields_ = [("box_lo", ctypes.c_float * 3), ("box_hi", ctypes.c_float * 3), ("n_out", ctypes.c_int), ("lr", ctypes.c_float),
                ("seed", ctypes.c_uint32), ("max_batch", ctypes.c_int), ("device", ctypes.c_int), ("stream", ctypes.c_void_p),
                ("loss_scale", ctypes.c_float)]


_bound = False


def _lib():
    global _bound
    L = native.load_library()
    if not _bound:
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.rc_mlp_tile_product.argtypes = [vp, vp, vp, i, i, vp, vp]
        L.rc_mlp_wait_check.argtypes = [ctypes.c_uint32, i, vp, vp]
        L.rc_mlp_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
        L.rc_mlp_destroy.argtypes = [vp]
        L.rc_mlp_destroy.restype = None
        L.rc_mlp_last_error.argtypes = [vp]
        L.rc_mlp_last_error.restype = ctypes.c_char_p
        L.rc_mlp_train.argtypes = [vp, vp, vp, vp, vp, i, vp, i, vp]
        L.rc_mlp_infer.argtypes = [vp, vp, vp, vp, i, vp, i]
        L.rc_mlp_weights.argtypes = [vp, vp, ctypes.c_size_t, i]
        L.rc_mlp_gradients.argtypes = [vp, vp, ctypes.c_size_t]
        L.rc_mlp_error_flags.argtypes = [vp, ctypes.POINTER(ctypes.c_uint)]
        L.rc_mlp_loss_scale.argtypes = [vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(ctypes.c_longlong)]
        _bound = True
    return L


def _ptr(x):
    return x if isinstance(x, int) or x is None else x.data_ptr()


def tile_product(a, b, d, err, stream=None):
    """d[128 x N] = a[128 x K] b[N x K]^T on the tensor cores (a, b: bf16 CUDA tensors; d: float32)."""
    K, N = int(a.shape[1]), int(b.shape[0])
    st = _lib().rc_mlp_tile_product(_ptr(a), _ptr(b), _ptr(d), K, N, _ptr(err), stream)
    if st != native.RC_OK:
        raise native.RCError(st, "rc_mlp_tile_product")


def wait_check(polls: int, arrive: bool, err, stream=None):
    """The bounded mbarrier wait on its own (rc_mlp_wait_check): err (a CUDA uint32/int32 tensor)
    gets bit 0 when the wait gave up."""
    st = _lib().rc_mlp_wait_check(polls, 1 if arrive else 0, _ptr(err), stream)
    if st != native.RC_OK:
        raise native.RCError(st, "rc_mlp_wait_check")


def split_weights(w: np.ndarray) -> list[np.ndarray]:
    """The flat master weights as the five [out, in] matrices."""
    out, o = [], 0
    for k, n in LAYERS:
        out.append(w[o:o + k * n].reshape(n, k))
        o += k * n
    return out


class Mlp:
    """One network on one GPU (rc_mlp_create / rc_mlp_destroy)."""

    def __init__(self, box_lo=(0.0, 0.0, 0.0), box_hi=(8.0, 4.0, 3.0), n_out=3, lr=1e-2, seed=1, max_batch=1 << 16, device=0,
                 stream=None, loss_scale=0.0):
        c = Config()
        c.box_lo[:] = box_lo
        c.box_hi[:] = box_hi
        c.n_out, c.lr, c.seed, c.max_batch, c.device, c.stream = n_out, lr, seed, max_batch, device, stream
        c.loss_scale = loss_scale
        self.L = _lib()
        h = ctypes.c_void_p()
        st = self.L.rc_mlp_create(ctypes.byref(c), ctypes.byref(h))
        if st != native.RC_OK:
            raise native.RCError(st, "rc_mlp_create failed")
        self.h, self.cfg = h, c

    def _chk(self, st):
        if st != native.RC_OK:
            raise native.RCError(st, self.L.rc_mlp_last_error(self.h).decode(errors="replace"))

    def close(self):
        if getattr(self, "h", None):
            self.L.rc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def train(self, pos4, nrm4, aux4, target, idx=None, loss=None):
        self._chk(self.L.rc_mlp_train(self.h, _ptr(pos4), _ptr(nrm4), _ptr(aux4), _ptr(target), int(target.shape[-1]), _ptr(idx),
                                      int(target.shape[0]) if idx is None else int(idx.shape[0]), _ptr(loss)))

    def train_raw(self, pos4, nrm4, aux4, target_ptr: int, tstride: int, idx, n: int, loss=None):
        """A training step whose targets are tstride floats per point at a raw device address
        (for instance a context's cache buffer, rc_array_info)."""
        self._chk(self.L.rc_mlp_train(self.h, _ptr(pos4), _ptr(nrm4), _ptr(aux4), target_ptr, int(tstride), _ptr(idx), int(n),
                                      _ptr(loss)))

    def infer_raw(self, pos4, nrm4, aux4, n: int, out_ptr: int, ostride: int):
        self._chk(self.L.rc_mlp_infer(self.h, _ptr(pos4), _ptr(nrm4), _ptr(aux4), int(n), out_ptr, int(ostride)))

    def loss_scale(self) -> tuple[float, int, int]:
        """(current loss scale, steps applied, steps skipped for a non-finite gradient)."""
        sc, st, sk = ctypes.c_float(), ctypes.c_longlong(), ctypes.c_longlong()
        self._chk(self.L.rc_mlp_loss_scale(self.h, ctypes.byref(sc), ctypes.byref(st), ctypes.byref(sk)))
        return sc.value, st.value, sk.value

    def infer(self, pos4, nrm4, aux4, out):
        self._chk(self.L.rc_mlp_infer(self.h, _ptr(pos4), _ptr(nrm4), _ptr(aux4), int(out.shape[0]), _ptr(out), int(out.shape[1])))

    def weights(self) -> np.ndarray:
        w = np.empty(NWEIGHT, np.float32)
        self._chk(self.L.rc_mlp_weights(self.h, w.ctypes.data_as(ctypes.c_void_p), w.size, 0))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        self._chk(self.L.rc_mlp_weights(self.h, w.ctypes.data_as(ctypes.c_void_p), w.size, 1))

    def gradients(self) -> np.ndarray:
        g = np.empty(NWEIGHT, np.float32)
        self._chk(self.L.rc_mlp_gradients(self.h, g.ctypes.data_as(ctypes.c_void_p), g.size))
        return g

    def error_flags(self) -> int:
        f = ctypes.c_uint()
        self._chk(self.L.rc_mlp_error_flags(self.h, ctypes.byref(f)))
        return f.value
