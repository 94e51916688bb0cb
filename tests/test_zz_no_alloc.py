"""rc_error_sums_noalloc: the error sums for callers that cannot allocate device memory.

Such callers (a per-frame path with a device-memory budget fixed at start-up, or a host
process whose memory manager owns all device memory) pass their own device buffers; the
entry point keeps its scratch space in a fixed array inside the library.  Here the test
plays that caller: the cache is the context's own device buffer, the reference, valid flags
and the output are device tensors the test allocated beforehand, and the sums must equal
those rc_frame recorded for the same frame, on two calls in a row (the second one reusing
the scratch array the first one left behind).

This file is named to be collected last, so that a run that stops at its first failure has
already run every other test.
"""
import math

import numpy as np
import pytest

from render_engine_gb300 import methods as M
from render_engine_gb300 import native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    from render_engine_gb300 import build
    build.build()


def test_noalloc_error_sums_match_rc_frame(scene_main_bytes):
    torch = pytest.importorskip("torch")
    ctx = N.Context()
    info = ctx.load_bytes(scene_main_bytes)
    np_, nl = info["np"], info["nl"]
    lc_stride = (nl + 3) // 4 * 4
    m = M.by_name(M.scen_methods(), "v4-A2C memoire verifiee+rampe")
    seq = [0] * 4 + [1] * 3
    dev = torch.device("cuda", 0)
    out3 = torch.zeros(3, dtype=torch.float64, device=dev)
    ctx.begin(m, seq[0], 2000)
    checked = 0
    for f, s in enumerate(seq):
        ctx.frame(s, want_err=True)
        if f < len(seq) - 2:
            continue
        ref = torch.from_numpy(ctx.state_array(s, N.SA_REF)).to(dev)
        valid = torch.from_numpy(ctx.state_array(s, N.SA_VALID)).to(dev)
        torch.cuda.synchronize()
        N.error_sums_noalloc(ctx.device_ptr(N.A_LC), lc_stride, nl, ctx.scalar(N.S_DORMANT), ref.data_ptr(),
                             valid.data_ptr(), np_, out3.data_ptr(), None)
        torch.cuda.synchronize()
        d2, rs, cnt = out3.cpu().numpy().tolist()
        err = float(np.float32(math.sqrt(d2 / cnt) / (rs / cnt)))
        want = float(ctx.errors()[f])
        assert cnt == float(ctx.state_array(s, N.SA_VALID).sum())
        assert abs(err - want) <= 1e-6 * abs(want), (f, err, want)
        checked += 1
    assert checked == 2


def test_noalloc_rejects_sizes_beyond_its_scratch():
    N.load_library()
    with pytest.raises(N.RCError):
        N.error_sums_noalloc(16, 4, 3, 0, 16, 16, N.NOALLOC_MAX_POINTS + 1, 16, None)
