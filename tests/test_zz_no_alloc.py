"""The allocation-free divergence check (cans_chkdiv_noalloc) against the allocating one.

Some callers of this library cannot call cudaMalloc: a Fortran host whose device memory
belongs to the OpenACC runtime's pool, or a run that fixes its memory budget at start-up.
cans_chkdiv_noalloc serves them from a fixed 1 MiB device array inside the library (at most
16,777,216 interior cells).  Like cans_chkdiv it synchronises its stream before returning.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_V = C.c_void_p


def _lib():
    from cans_gb300 import build
    L = C.CDLL(build.build())
    for name in ("cans_chkdiv", "cans_chkdiv_noalloc"):
        getattr(L, name).argtypes = [_I, _D, _D, _V, _V, _V, _V, _D, _D, _V]
    return L


def _call(fn, n, l, dli, dzfi, u, v, w, stream):
    tot, mx = C.c_double(), C.c_double()
    rc = fn((C.c_int * 3)(*n), (C.c_double * 3)(*l), (C.c_double * 3)(*dli), C.c_void_p(dzfi.data_ptr()),
            C.c_void_p(u.data_ptr()), C.c_void_p(v.data_ptr()), C.c_void_p(w.data_ptr()), C.byref(tot),
            C.byref(mx), C.c_void_p(stream))
    return rc, tot.value, mx.value


def test_size_limit_rejected_before_any_device_work():
    """Beyond the fixed scratch the call returns CANS_EINVAL (1) before touching CUDA."""
    L = _lib()
    dummy = (C.c_double * 4)()
    p = C.cast(dummy, C.c_void_p)
    tot, mx = C.c_double(), C.c_double()
    rc = L.cans_chkdiv_noalloc((C.c_int * 3)(4096, 4096, 2), (C.c_double * 3)(1, 1, 1),
                               (C.c_double * 3)(1, 1, 1), p, p, p, p, C.byref(tot), C.byref(mx), None)
    assert rc == 1
    # extents whose product would overflow a 64-bit count are rejected, not wrapped
    big = 2 ** 31 - 1
    rc = L.cans_chkdiv_noalloc((C.c_int * 3)(big, big, big), (C.c_double * 3)(1, 1, 1),
                               (C.c_double * 3)(1, 1, 1), p, p, p, p, C.byref(tot), C.byref(mx), None)
    assert rc == 1


@pytest.mark.gpu
def test_chkdiv_noalloc_matches_allocating_entry_point(require_gpu):
    import torch
    L = _lib()
    st = torch.cuda.current_stream().cuda_stream
    n, l = (40, 36, 30), (2.0, 1.5, 1.0)
    dli = [n[d] / l[d] for d in range(3)]
    dzfi = torch.linspace(25., 35., n[2] + 2, dtype=torch.float64, device="cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    for call in range(2):  # two calls in a row share (and reuse) the fixed scratch
        u, v, w = (torch.randn((n[2] + 2, n[1] + 2, n[0] + 2), generator=g, dtype=torch.float64, device="cuda")
                   for _ in range(3))
        rc0, tot0, mx0 = _call(L.cans_chkdiv, n, l, dli, dzfi, u, v, w, st)
        rc1, tot1, mx1 = _call(L.cans_chkdiv_noalloc, n, l, dli, dzfi, u, v, w, st)
        assert rc0 == 0 and rc1 == 0, (call, rc0, rc1)
        assert mx1 == mx0 and abs(tot1 - tot0) <= 1e-13 * abs(tot0), (call, tot0, tot1, mx0, mx1)
        assert np.isfinite(tot1) and tot1 > 0
