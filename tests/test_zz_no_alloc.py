"""GPU: hgb_reduce_noalloc, the reduction entry point that allocates nothing.

Callers that cannot allocate device memory (real-time frame loops that must
never block in the CUDA allocator, plug-ins whose host program owns the device
memory through its own allocator) use it instead of hgb_reduce, which grows a
library workspace with cudaMalloc.  Its scratch is a
fixed array in the library's device memory.  Checked here through the C ABI
against hgb_reduce on the same inputs, on two calls in a row (the second call
reuses the array the first one left behind), and the device's free memory is
unchanged across the calls.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C
import struct

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9  # float sums: the tolerance of the float reduction tests


def _reduce(name, t, op, win=None):
    from hipacc_gb300 import _lib as L
    from hipacc_gb300 import api

    v = api.view(t)
    out = C.create_string_buffer(8)
    w = None if win is None else C.byref(L.Window(*win))
    L.check(getattr(L.load(), name)(C.byref(v), w, op, None, out, C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out.raw


def test_noalloc_matches_reduce_twice(gpu):
    from hipacc_gb300 import _lib as L

    rng = np.random.default_rng(2026)
    f = torch.from_numpy(rng.random((1537, 2049), dtype=np.float32)).cuda()
    u = torch.from_numpy(rng.integers(0, 256, (777, 1031), dtype=np.uint8)).cuda()
    i = torch.from_numpy(rng.integers(-30000, 30000, (333, 517)).astype(np.int32)).cuda()
    cases = [(f, L.SUM, None), (f, L.MAX, None), (f, L.SUM, (17, 5, 1000, 1200)), (u, L.SUM, None),
             (u, L.MAX, None), (u, L.MIN, (3, 3, 500, 400)), (i, L.SUM, None), (i, L.MIN, None)]
    # the workspace entry point first: it may allocate its workspace now
    expected = [_reduce("hgb_reduce", t, op, win) for (t, op, win) in cases]
    # the first call on the device is the set-up call: it resolves the array's
    # address, and the driver loads the code module that holds the array
    _reduce("hgb_reduce_noalloc", u, L.SUM)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for call in range(2):
        for (t, op, win), ref in zip(cases, expected):
            got = _reduce("hgb_reduce_noalloc", t, op, win)
            if t.dtype == torch.float32:
                a, b = struct.unpack("<d", got)[0], struct.unpack("<d", ref)[0]
                assert abs(a - b) <= REL_TOL * abs(b), (call, op, win, a, b)
            else:
                assert got == ref, (call, op, win)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after >= free_before  # nothing was allocated on the device


def test_noalloc_device_result_and_errors(gpu):
    from hipacc_gb300 import _lib as L
    from hipacc_gb300 import api

    rng = np.random.default_rng(7)
    a = rng.integers(0, 256, (300, 400), dtype=np.uint8)
    t = torch.from_numpy(a).cuda()
    res = torch.zeros(2, dtype=torch.int64, device="cuda")
    lib = L.load()
    sp = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    v = api.view(t)
    for k in range(2):
        L.check(lib.hgb_reduce_noalloc(C.byref(v), None, L.SUM, C.c_void_p(res[k:k + 1].data_ptr()), None, sp))
    torch.cuda.synchronize()
    assert res.tolist() == [int(a.sum())] * 2
    # no destination at all is rejected on the host
    assert lib.hgb_reduce_noalloc(C.byref(v), None, L.SUM, None, None, sp) == L.ERR_INVALID
