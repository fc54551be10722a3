"""The allocation-free multi-dot entry point, through the C ABI.

Some callers hand the whole device budget to their own memory pool before a
solve and cannot call cudaMalloc afterwards; qcm_multi_dot_noalloc serves
them with a fixed library-owned scratch array.  This file is collected last
so that a run stopping at the first failure has already run every other test.
It must pass alone in a fresh process and after the other tests.
"""
import ctypes as C

import pytest
import torch

from qcmaquis_gb300 import native as N

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the FP64 tolerance of the other GPU tests


def _ptrs(ts):
    return (C.c_void_p * len(ts))(*[C.c_void_p(t.data_ptr()) for t in ts])


def test_noalloc_multi_dot_matches_allocating_entry_point_twice():
    lib = N.lib()
    g = torch.Generator(device="cuda").manual_seed(1234)
    n = 2_000_003
    vs = [torch.randn(n, dtype=torch.float64, device="cuda", generator=g) for _ in range(7)]
    y = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    ref = torch.zeros(7, dtype=torch.float64, device="cuda")
    N.check(lib.qcm_multi_dot(_ptrs(vs), 7, C.c_void_p(y.data_ptr()), n, C.c_void_p(ref.data_ptr()), None),
            "qcm_multi_dot")
    for call in range(2):
        out = torch.full((7,), float("nan"), dtype=torch.float64, device="cuda")
        N.check(lib.qcm_multi_dot_noalloc(_ptrs(vs), 7, C.c_void_p(y.data_ptr()), n, C.c_void_p(out.data_ptr()),
                                          None), "qcm_multi_dot_noalloc")
        torch.cuda.synchronize()
        assert torch.all(torch.isfinite(out)), call
        assert torch.allclose(out, ref, rtol=REL_TOL, atol=REL_TOL * float(ref.abs().max())), (call, out, ref)
    # a smaller call after a larger one still reads only what it wrote
    out2 = torch.zeros(2, dtype=torch.float64, device="cuda")
    N.check(lib.qcm_multi_dot_noalloc(_ptrs(vs[:2]), 2, C.c_void_p(y.data_ptr()), 1000,
                                      C.c_void_p(out2.data_ptr()), None), "qcm_multi_dot_noalloc")
    torch.cuda.synchronize()
    exp = torch.stack([torch.dot(v[:1000], y[:1000]) for v in vs[:2]])
    assert torch.allclose(out2, exp, rtol=REL_TOL, atol=1e-12)


def test_noalloc_multi_dot_allocates_no_device_memory():
    """After a first call (which looks up the scratch array and may load the
    library's device code), further calls of different sizes leave both torch's
    allocator and the device's free memory unchanged."""
    lib = N.lib()
    g = torch.Generator(device="cuda").manual_seed(99)
    sizes = [17, 4096, 1_000_003, 65_536]
    vs = [torch.randn(max(sizes), dtype=torch.float64, device="cuda", generator=g) for _ in range(32)]
    y = torch.randn(max(sizes), dtype=torch.float64, device="cuda", generator=g)
    out = torch.zeros(32, dtype=torch.float64, device="cuda")
    N.check(lib.qcm_multi_dot_noalloc(_ptrs(vs), 32, C.c_void_p(y.data_ptr()), 8, C.c_void_p(out.data_ptr()), None),
            "qcm_multi_dot_noalloc")
    torch.cuda.synchronize()
    torch_before = torch.cuda.memory_allocated()
    free_before, _ = torch.cuda.mem_get_info()
    for k, n in enumerate(sizes):
        nv = (5 * k + 3) % 32 + 1
        N.check(lib.qcm_multi_dot_noalloc(_ptrs(vs[:nv]), nv, C.c_void_p(y.data_ptr()), n,
                                          C.c_void_p(out.data_ptr()), None), "qcm_multi_dot_noalloc")
        torch.cuda.synchronize()
        exp = torch.stack([torch.dot(v[:n], y[:n]) for v in vs[:nv]])
        assert torch.allclose(out[:nv], exp, rtol=1e-11, atol=1e-11 * float(exp.abs().max()))
    del exp
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert torch.cuda.memory_allocated() == torch_before
    assert free_after == free_before, (free_before, free_after)


def test_noalloc_multi_dot_rejects_too_many_vectors():
    lib = N.lib()
    y = torch.zeros(16, dtype=torch.float64, device="cuda")
    vs = [y] * 33
    out = torch.zeros(33, dtype=torch.float64, device="cuda")
    rc = lib.qcm_multi_dot_noalloc(_ptrs(vs), 33, C.c_void_p(y.data_ptr()), 16, C.c_void_p(out.data_ptr()), None)
    assert rc == -5
    assert b"capacity" in lib.qcm_last_error()
