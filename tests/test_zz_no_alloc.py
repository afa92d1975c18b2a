"""The allocation-free search entry point, searchIdxsNoAllocGpu.

Some callers cannot allocate device memory while they query (their device memory
belongs to another allocator or a fixed pool, or their query thread must not call
cudaMalloc).  This entry point serves them: it keeps its scratch in a fixed device
array inside the library and allocates nothing.  The test calls it through the
C-ABI twice in a row and checks each result, bit for bit (integer output), against
the allocating entry point searchDeviceGpu on the same device buffers, and checks
that the library's device allocator did not grow during those calls.  This file
is collected last so that a failure here does not stop the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(lib, check, arr=None, nbytes=None, stream=None):
    p = C.c_void_p()
    n = arr.nbytes if arr is not None else nbytes
    check(lib.deviceMallocGpu(C.byref(p), max(int(n), 1)))
    if arr is not None:
        check(lib.memcpyGpu(p, C.c_void_p(arr.ctypes.data), arr.nbytes, stream))
    return p


def _host(lib, check, p, n, dtype, stream):
    out = np.empty(n, dtype)
    if n:
        check(lib.memcpyGpu(C.c_void_p(out.ctypes.data), p, out.nbytes, stream))
    check(lib.streamSynchronizeGpu(stream))
    return out


@pytest.mark.parametrize("bits", [32, 64])
def test_no_alloc_search_matches_allocating_entry_point(bits):
    import __graft_entry__ as g
    g.build()
    from superintervals_gb300 import _capi, workloads as W
    from superintervals_gb300.interval_map import GpuIndex
    lib, check = _capi.load(), _capi.check
    dt = np.int64 if bits == 64 else np.int32
    wl = W.config3(n=300_000, nq=60_000) if bits == 32 else W.random_nested(7, 40_000, 30_000, dtype=dt)
    idx = GpuIndex(bits)
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None)
    idx.build()
    st = idx.stream
    nq = wl.nq
    d_qs = _dev(lib, check, np.ascontiguousarray(wl.q_starts, dt), stream=st)
    d_qe = _dev(lib, check, np.ascontiguousarray(wl.q_ends, dt), stream=st)
    d_qc = None if wl.q_contig is None else _dev(lib, check, wl.q_contig, stream=st)
    d_off = _dev(lib, check, nbytes=8 * (nq + 1))
    total = C.c_size_t(0)
    for order in (0, 1):
        st_ = lib.searchDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, order, 0, d_off, None, 0, C.byref(total), st)
        assert st_ in (0, _capi.SI_ERR_CAPACITY)
        P = int(total.value)
        d_ref = _dev(lib, check, nbytes=4 * max(P, 1))
        check(lib.searchDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, order, 0, d_off, d_ref, P, C.byref(total), st))
        ref_off = _host(lib, check, d_off, nq + 1, np.int64, st)
        ref_out = _host(lib, check, d_ref, P, np.int32, st)
        d_off2 = _dev(lib, check, nbytes=8 * (nq + 1))
        d_out2 = _dev(lib, check, nbytes=4 * max(P, 1))
        poison = np.full(max(P, 1), -7, np.int32)
        for _ in range(2):   # two calls in a row share (and reuse) the library's scratch
            check(lib.memcpyGpu(d_out2, C.c_void_p(poison.ctypes.data), poison.nbytes, st))
            check(lib.streamSynchronizeGpu(st))
            used = lib.deviceBytesInUseGpu()
            t2 = C.c_size_t(0)
            check(lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, nq, order, d_off2, d_out2, P, C.byref(t2), st))
            assert lib.deviceBytesInUseGpu() == used
            assert int(t2.value) == P
            assert np.array_equal(_host(lib, check, d_off2, nq + 1, np.int64, st), ref_off)
            assert np.array_equal(_host(lib, check, d_out2, P, np.int32, st), ref_out)
        for p in (d_ref, d_off2, d_out2):
            lib.deviceFreeGpu(p)
    # too many queries: rejected before any device work
    t3 = C.c_size_t(0)
    st_ = lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, (1 << 22) + 1, 0, d_off, None, 0, C.byref(t3), st)
    assert st_ == _capi.SI_ERR_TOO_LARGE
    for p in (d_qs, d_qe, d_qc, d_off):
        if p is not None:
            lib.deviceFreeGpu(p)
    idx.close()
