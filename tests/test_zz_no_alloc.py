"""The allocation-free search entry point, searchIdxsNoAllocGpu.

Some callers cannot allocate device memory while they query (their device memory
belongs to another allocator or a fixed pool, or their query thread must not call
cudaMalloc).  This entry point serves them: it keeps its scratch in a fixed device
array inside the library and allocates nothing.  The tests call it through the
C-ABI twice in a row and check each result, bit for bit (integer output), against
the allocating entry point searchDeviceGpu on the same device buffers and against
the oracle, and check that the library's device allocator did not grow during those
calls.  They also cover a result one value larger than the output (rejected, output
untouched), a query naming a contig outside the index, and an empty index.  This file
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


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    from superintervals_gb300 import _capi
    return _capi


@pytest.mark.parametrize("bits", [32, 64])
def test_no_alloc_search_matches_allocating_entry_point(lib, bits):
    from oracle.oracle import Oracle
    from superintervals_gb300 import workloads as W
    from superintervals_gb300.interval_map import GpuIndex
    _capi = lib
    lib, check = _capi.load(), _capi.check
    dt = np.int64 if bits == 64 else np.int32
    wl = W.config3(n=300_000, nq=60_000) if bits == 32 else W.random_nested(7, 40_000, 30_000, dtype=dt)
    idx = GpuIndex(bits)
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None)
    idx.build()
    o = Oracle()
    m = o.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
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
        o_off, o_out = o.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=order, nthreads=8)
        assert np.array_equal(ref_off, o_off) and np.array_equal(ref_out, o_out)
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
            got_off = _host(lib, check, d_off2, nq + 1, np.int64, st)
            got_out = _host(lib, check, d_out2, P, np.int32, st)
            assert np.array_equal(got_off, ref_off) and np.array_equal(got_out, ref_out)
            assert np.array_equal(got_off, o_off) and np.array_equal(got_out, o_out)
        # one value short: SI_ERR_CAPACITY with the size reported, the output left as it was
        assert P > 0
        check(lib.memcpyGpu(d_out2, C.c_void_p(poison.ctypes.data), poison.nbytes, st))
        t4 = C.c_size_t(0)
        st_ = lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, nq, order, d_off2, d_out2, P - 1, C.byref(t4), st)
        assert st_ == _capi.SI_ERR_CAPACITY and int(t4.value) == P
        assert np.array_equal(_host(lib, check, d_out2, P, np.int32, st), poison[:P])
        assert np.array_equal(_host(lib, check, d_off2, nq + 1, np.int64, st), ref_off)
        # a null value buffer with room claimed is rejected before any device work
        st_ = lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, nq, order, d_off2, None, P, C.byref(t4), st)
        assert st_ == _capi.SI_ERR_INVALID
        for p in (d_ref, d_off2, d_out2):
            lib.deviceFreeGpu(p)
    # too many queries: rejected before any device work
    t3 = C.c_size_t(0)
    st_ = lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, (1 << 22) + 1, 0, d_off, None, 0, C.byref(t3), st)
    assert st_ == _capi.SI_ERR_TOO_LARGE
    # a query naming a contig outside the index: SI_ERR_INVALID, the call after it works again
    G = len(wl.seg) - 1
    bad_c = np.zeros(4, np.int32)
    bad_c[2] = G
    few = np.ascontiguousarray(wl.q_starts[:4], dt), np.ascontiguousarray(wl.q_ends[:4], dt)
    d_bs, d_be = _dev(lib, check, few[0], stream=st), _dev(lib, check, few[1], stream=st)
    d_bc = _dev(lib, check, bad_c, stream=st)
    want_off, want_out = o.search_batch(m, few[0], few[1], np.zeros(4, np.int32), order=0)
    cap = max(int(want_off[-1]), 1)
    d_bo, d_bv = _dev(lib, check, nbytes=8 * 5), _dev(lib, check, nbytes=4 * cap)
    st_ = lib.searchIdxsNoAllocGpu(idx.h, d_bs, d_be, d_bc, 4, 0, d_bo, d_bv, cap, C.byref(t3), st)
    assert st_ == _capi.SI_ERR_INVALID
    bad_c[2] = 0
    check(lib.memcpyGpu(d_bc, C.c_void_p(bad_c.ctypes.data), bad_c.nbytes, st))
    check(lib.searchIdxsNoAllocGpu(idx.h, d_bs, d_be, d_bc, 4, 0, d_bo, d_bv, cap, C.byref(t3), st))
    assert int(t3.value) == int(want_off[-1])
    assert np.array_equal(_host(lib, check, d_bv, int(want_off[-1]), np.int32, st), want_out)
    for p in (d_qs, d_qe, d_qc, d_off, d_bs, d_be, d_bc, d_bo, d_bv):
        if p is not None:
            lib.deviceFreeGpu(p)
    idx.close()


def test_no_alloc_search_on_empty_index(lib):
    """An empty built index: every count is zero, and a contig id outside the index is
    still rejected, as searchDeviceGpu does."""
    from superintervals_gb300.interval_map import GpuIndex
    _capi = lib
    lib, check = _capi.load(), _capi.check
    idx = GpuIndex(32)
    idx.build()
    st = idx.stream
    qs = np.array([1, 5, 10], np.int32)
    qe = np.array([2, 50, 10], np.int32)
    qc = np.zeros(3, np.int32)
    d_qs, d_qe = _dev(lib, check, qs, stream=st), _dev(lib, check, qe, stream=st)
    d_qc = _dev(lib, check, qc, stream=st)
    d_off = _dev(lib, check, nbytes=8 * 4)
    poison = np.full(4, 99, np.int64)
    for _ in range(2):
        check(lib.memcpyGpu(d_off, C.c_void_p(poison.ctypes.data), poison.nbytes, st))
        t = C.c_size_t(7)
        check(lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, 3, 0, d_off, None, 0, C.byref(t), st))
        assert int(t.value) == 0
        assert np.array_equal(_host(lib, check, d_off, 4, np.int64, st), np.zeros(4, np.int64))
    qc[1] = 1   # the empty index has one contig
    check(lib.memcpyGpu(d_qc, C.c_void_p(qc.ctypes.data), qc.nbytes, st))
    t = C.c_size_t(0)
    assert lib.searchIdxsNoAllocGpu(idx.h, d_qs, d_qe, d_qc, 3, 0, d_off, None, 0, C.byref(t), st) == \
        _capi.SI_ERR_INVALID
    ref = lib.searchDeviceGpu(idx.h, d_qs, d_qe, d_qc, 3, 0, 0, d_off, None, 0, C.byref(t), st)
    assert ref == _capi.SI_ERR_INVALID
    for p in (d_qs, d_qe, d_qc, d_off):
        lib.deviceFreeGpu(p)
    idx.close()
