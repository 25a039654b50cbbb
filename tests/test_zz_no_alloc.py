"""The alias build that allocates nothing (dr_alias_build_noalloc).

Callers that may not call cudaMalloc -- a host application that owns all
device memory and passes a plugin only pre-allocated buffers, or a frame loop
that cannot afford cudaMalloc's implicit synchronisation -- build their light
tables through this entry point, whose scratch is a fixed array inside the
library (limit: 65,536 weights). Here it is called through the C ABI and
compared with the allocating entry point, dr_alias_build in sweep mode, bit for
bit, on two calls in a row (the second must not see the first call's
leftovers). This file is collected last on purpose.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _noalloc(native, w: torch.Tensor, n: int) -> np.ndarray:
    out = torch.full((max(n, 1) * 5,), -7, dtype=torch.int32, device="cuda")
    st = native.load().dr_alias_build_noalloc(w.data_ptr(), n, out.data_ptr(), None)
    native.check(st)
    torch.cuda.synchronize()
    return out.cpu().numpy()[: n * 5].view(native.ALIAS_DTYPE)


def _allocating(native, ctx, w: torch.Tensor, n: int) -> np.ndarray:
    out = torch.zeros(max(n, 1) * 5, dtype=torch.int32, device="cuda")
    ctx.alias_build(w, n, out, native.DR_ALIAS_SWEEP)
    torch.cuda.synchronize()
    return out.cpu().numpy()[: n * 5].view(native.ALIAS_DTYPE)


def test_noalloc_matches_allocating_build_twice(native, ctx):
    rng = np.random.default_rng(2024)
    # first call: the full 65,536-weight limit; second call: a smaller,
    # differently distributed input that would expose stale scratch
    w1 = rng.lognormal(0.0, 1.5, 65536).astype(np.float32)
    w2 = rng.random(3001).astype(np.float32)
    w2[rng.random(3001) < 0.3] = 0.0
    for w in (w1, w2):
        dw = torch.from_numpy(w).cuda()
        got = _noalloc(native, dw, w.size)
        want = _allocating(native, ctx, dw, w.size)
        assert got.tobytes() == want.tobytes()


def test_noalloc_allocates_no_device_memory(native, ctx):
    """After the first call (which only looks up the array's address), further
    calls leave the device's free memory unchanged; one of them runs on a
    non-default stream and still equals the allocating build."""
    rng = np.random.default_rng(7)
    w = rng.lognormal(0.0, 1.0, 40000).astype(np.float32)
    dw = torch.from_numpy(w).cuda()
    out = torch.zeros(40000 * 5, dtype=torch.int32, device="cuda")
    lib = native.load()
    native.check(lib.dr_alias_build_noalloc(dw.data_ptr(), 40000, out.data_ptr(), None))
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    s = torch.cuda.Stream()
    for _ in range(3):
        native.check(lib.dr_alias_build_noalloc(dw.data_ptr(), 40000, out.data_ptr(), s.cuda_stream))
    s.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    got = out.cpu().numpy().view(native.ALIAS_DTYPE)
    assert got.tobytes() == _allocating(native, ctx, dw, 40000).tobytes()


def test_noalloc_rejects_sizes_beyond_its_limit(native):
    w = torch.ones(65537, dtype=torch.float32, device="cuda")
    out = torch.zeros(65537 * 5, dtype=torch.int32, device="cuda")
    st = native.load().dr_alias_build_noalloc(w.data_ptr(), 65537, out.data_ptr(), None)
    assert st == 8  # DR_ERR_TOO_LARGE
    assert b"65536" in ctypes.c_char_p(native.load().dr_last_error_string()).value
