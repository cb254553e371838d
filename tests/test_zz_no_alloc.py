"""The allocation-free sort entry point (apbf_sort_pairs_noalloc), called through
the C ABI, must give exactly what the context-based apbf_sort_pairs gives, on two
calls in a row (the second call reuses the shared scratch array the first one
left behind).  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sorted_by_context(ctx, keys, vals, ub):
    from apbf_gb300.api import algorithms

    n = keys.numel()
    ok, ov = torch.empty_like(keys), torch.empty_like(vals)
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    algorithms.sort(ctx, keys, vals, cnt, n, ok, ov, ub)
    torch.cuda.synchronize()
    return ok.cpu().numpy(), ov.cpu().numpy()


def _sorted_noalloc(lib, keys, vals, ub):
    from apbf_gb300 import _native

    n = keys.numel()
    ok, ov = torch.empty_like(keys), torch.empty_like(vals)
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    st = lib.apbf_sort_pairs_noalloc(C.c_void_p(keys.data_ptr()), C.c_void_p(vals.data_ptr()),
                                     C.c_void_p(cnt.data_ptr()), n, ub, C.c_void_p(ok.data_ptr()),
                                     C.c_void_p(ov.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    _native.check(st, "apbf_sort_pairs_noalloc")
    torch.cuda.synchronize()
    return ok.cpu().numpy(), ov.cpu().numpy()


def test_noalloc_sort_matches_context_sort_twice(native_lib, cuda):
    from apbf_gb300.api import Context

    ctx = Context(particle_capacity=1 << 20, max_neighbors=1, max_log2res=1)
    rng = np.random.default_rng(2024)
    for call, (n, ub) in enumerate([(700_001, 0xFFFFFFFF), (1 << 20, (1 << 21) - 1)]):
        k = rng.integers(0, 1 << 32, size=n, dtype=np.uint64) & np.uint64(ub)
        keys = torch.from_numpy(k.astype(np.uint32).view(np.int32)).cuda()
        vals = torch.arange(n, dtype=torch.int32, device="cuda")
        ref_k, ref_v = _sorted_by_context(ctx, keys, vals, ub)
        got_k, got_v = _sorted_noalloc(native_lib, keys, vals, ub)
        assert np.array_equal(got_k, ref_k), call
        assert np.array_equal(got_v, ref_v), call
        order = np.argsort(k.astype(np.uint32), kind="stable")
        assert np.array_equal(got_v.view(np.uint32), order.astype(np.uint32)), call
    ctx.close()


def test_noalloc_sort_rejects_oversize(native_lib, cuda):
    t = torch.zeros(4, dtype=torch.int32, device="cuda")
    p = C.c_void_p(t.data_ptr())
    o = torch.zeros(4, dtype=torch.int32, device="cuda")
    q = C.c_void_p(o.data_ptr())
    r = torch.zeros(4, dtype=torch.int32, device="cuda")
    st = native_lib.apbf_sort_pairs_noalloc(p, C.c_void_p(t.data_ptr() + 4), p, (1 << 20) + 1, 255, q,
                                            C.c_void_p(r.data_ptr()), None)
    assert st == 1
    assert b"1048576" in native_lib.apbf_last_error()


def test_noalloc_sort_rejects_overlapping_outputs(native_lib, cuda):
    """Outputs that are the same buffer, or overlap an input or each other by part of
    their length, are rejected before any work is queued."""
    buf = torch.zeros(64, dtype=torch.int32, device="cuda")
    base = buf.data_ptr()
    cnt = torch.tensor([16], dtype=torch.int32, device="cuda")
    keys = torch.zeros(16, dtype=torch.int32, device="cuda")
    vals = torch.zeros(16, dtype=torch.int32, device="cuda")

    def call(out_k, out_v, k=keys.data_ptr(), v=vals.data_ptr()):
        return native_lib.apbf_sort_pairs_noalloc(C.c_void_p(k), C.c_void_p(v), C.c_void_p(cnt.data_ptr()), 16,
                                                  255, C.c_void_p(out_k), C.c_void_p(out_v), None)

    assert call(base, base) == 1                       # the two outputs are one buffer
    assert call(base, base + 8 * 4) == 1               # they overlap by half
    assert call(base, base + 32 * 4, k=base + 4) == 1  # the keys overlap the key output
    assert b"overlaps" in native_lib.apbf_last_error()
