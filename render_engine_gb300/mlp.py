"""ctypes front end of the tensor-core radiance cache (include/rc_mlp.h).

Calls take CUDA tensors (or raw device pointers as ints); the library must be built
(``__graft_entry__.build()``); nothing here falls back to a CPU path.
"""
from __future__ import annotations

import ctypes

from . import native

EXPORTS = ["rc_mlp_tile_product"]

_bound = False


def _lib():
    global _bound
    L = native.load_library()
    if not _bound:
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.rc_mlp_tile_product.argtypes = [vp, vp, vp, i, i, vp, vp]
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
