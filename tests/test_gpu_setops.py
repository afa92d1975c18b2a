"""GPU parity of the operations over hit lists through the C-ABI: set operations
(intersection / difference of map A against the index B), key gathers
(search_keys / search_items) and coverage.  Against the golden fixtures made by the
reference's own C++ class and C API, and against the oracle on seeded multi-contig
inputs."""
import ctypes as C

import numpy as np
import pytest

from golden_util import fixture_names, load

pytestmark = pytest.mark.gpu

PATHS = ["plain", "batched"]


@pytest.fixture(scope="module")
def api():
    import __graft_entry__ as g
    g.build()
    from superintervals_gb300 import interval_map as im
    return im


@pytest.fixture(scope="module")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


def _index(api, starts, ends, data=None, seg=None, path="plain"):
    bits = 64 if np.asarray(starts).dtype == np.int64 else 32
    idx = api.GpuIndex(bits)
    idx.add_arrays(starts, ends, data, seg=seg)
    idx.build()
    idx.set_path(api.PATH_PLAIN if path == "plain" else api.PATH_BATCHED)
    return idx


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", fixture_names("setops_"))
def test_setops_fixture_parity(api, name, path):
    g = load(name)
    idx = _index(api, g["b_starts"], g["b_ends"], g["b_data"], path=path)
    bs, be, _, _ = idx.arrays()
    a_s, a_e, a_d = g["ref_a_sorted_starts"], g["ref_a_sorted_ends"], g["ref_a_sorted_data"]
    # C++ class order
    off, s, e, h = idx.intersect(a_s, a_e, order=api.ORDER_IDXS_CPP)
    assert np.array_equal(s, g["ref_isect_starts"]) and np.array_equal(e, g["ref_isect_ends"])
    owner = np.repeat(np.arange(len(a_s)), np.diff(off))
    assert np.array_equal(a_d[owner], g["ref_isect_data"])
    bd = g["ref_isect_bdata_data"]   # B's insertion index: the hit has its coordinates
    assert np.array_equal(g["b_starts"][bd], bs[h]) and np.array_equal(g["b_ends"][bd], be[h])
    off, s, e = idx.difference(a_s, a_e)
    assert np.array_equal(s, g["ref_diff_starts"]) and np.array_equal(e, g["ref_diff_ends"])
    owner = np.repeat(np.arange(len(a_s)), np.diff(off))
    assert np.array_equal(a_d[owner], g["ref_diff_data"])
    if "ref_c_isect_starts" in g:     # the C API (fully descending hit order)
        _, s, e, _ = idx.intersect(a_s, a_e, order=api.ORDER_DESC)
        assert np.array_equal(s, g["ref_c_isect_starts"]) and np.array_equal(e, g["ref_c_isect_ends"])
    idx.close()


def _oracle_setops(oracle, wl, order):
    """Per-contig oracle results, reassembled in batch order."""
    nq = wl.nq
    qc = wl.q_contig if wl.q_contig is not None else np.zeros(nq, np.int32)
    isect = [None] * nq
    diff = [None] * nq
    for gi in range(len(wl.seg) - 1):
        lo, hi = int(wl.seg[gi]), int(wl.seg[gi + 1])
        m = oracle.build(wl.starts[lo:hi], wl.ends[lo:hi], wl.data[lo:hi])
        sel = np.nonzero(qc == gi)[0]
        off, s, e, h = oracle.intersection(m, wl.q_starts[sel], wl.q_ends[sel], order)
        for k, q in enumerate(sel):
            a, b = off[k], off[k + 1]
            isect[q] = (s[a:b], e[a:b], h[a:b])
        off, s, e = oracle.difference(m, wl.q_starts[sel], wl.q_ends[sel])
        for k, q in enumerate(sel):
            a, b = off[k], off[k + 1]
            diff[q] = (s[a:b], e[a:b])
    return isect, diff


def _check(api, oracle, wl, path, order=0):
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None, path=path)
    isect, diff = _oracle_setops(oracle, wl, order)
    off, s, e, h = idx.intersect(wl.q_starts, wl.q_ends, wl.q_contig, order=order)
    for q in range(wl.nq):
        a, b = off[q], off[q + 1]
        ws, we, wh = isect[q]
        assert np.array_equal(s[a:b], ws) and np.array_equal(e[a:b], we) and np.array_equal(h[a:b], wh), q
    off, s, e = idx.difference(wl.q_starts, wl.q_ends, wl.q_contig)
    for q in range(wl.nq):
        a, b = off[q], off[q + 1]
        ws, we = diff[q]
        assert np.array_equal(s[a:b], ws) and np.array_equal(e[a:b], we), q
    idx.close()


@pytest.mark.parametrize("path", PATHS)
def test_setops_multicontig_vs_oracle(api, oracle, path):
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=120_000, nq=20_000, contigs=W.HUMAN_CONTIGS[18:24])
    _check(api, oracle, wl, path, order=0)


@pytest.mark.parametrize("seed,dt", [(31, np.int32), (32, np.int64)])
def test_setops_random_nested_desc_order(api, oracle, seed, dt):
    from superintervals_gb300 import workloads as W
    wl = W.random_nested(seed, 5000, 3000, dtype=dt, span=300_000, max_len=3_000)
    _check(api, oracle, wl, "batched", order=1)


def test_setops_inverted_intervals_vs_oracle(api, oracle):
    """B with start > end intervals takes the exact sequential sweep."""
    from superintervals_gb300 import workloads as W
    wl = W.random_nested(33, 4000, 2000, dtype=np.int32, span=200_000, max_len=2_000)
    r = np.random.Generator(np.random.PCG64(5))
    inv = r.random(wl.n) < 0.03
    wl.starts[inv], wl.ends[inv] = wl.ends[inv] + 2, wl.starts[inv]
    qinv = r.random(wl.nq) < 0.03
    wl.q_starts[qinv], wl.q_ends[qinv] = wl.q_ends[qinv] + 1, wl.q_starts[qinv]
    _check(api, oracle, wl, "plain", order=0)


def test_setops_device_form_and_capacity(api):
    """The device-buffer entry points give the host forms' results; a short
    capacity reports the needed size; a bad contig id is an error."""
    lib = api._capi.load()
    s = np.array([10, 15, 30, 100], np.int32)
    e = np.array([20, 25, 40, 120], np.int32)
    idx = _index(api, s, e)
    qs = np.array([12, 0, 35, 90], np.int32)
    qe = np.array([33, 5, 130, 95], np.int32)
    off_h, s_h, e_h, h_h = idx.intersect(qs, qe)
    doff_h, ds_h, de_h = idx.difference(qs, qe)

    def dev(a):
        p = C.c_void_p()
        api.check(lib.deviceMallocGpu(C.byref(p), max(a.nbytes, 4)))
        api.check(lib.memcpyGpu(p, C.c_void_p(a.ctypes.data), a.nbytes, None))
        return p

    def host(p, n, dt):
        out = np.empty(n, dt)
        if n:
            api.check(lib.memcpyGpu(C.c_void_p(out.ctypes.data), p, out.nbytes, None))
        return out
    d_qs, d_qe = dev(qs), dev(qe)
    d_off = dev(np.zeros(5, np.int64))
    d_s, d_e, d_h = dev(np.zeros(16, np.int32)), dev(np.zeros(16, np.int32)), dev(np.zeros(16, np.int32))
    tot = C.c_size_t(0)
    st = lib.intersectDeviceGpu(idx.h, d_qs, d_qe, None, 4, 0, d_off, d_s, d_e, d_h, 1, C.byref(tot), None)
    assert st == api._capi.SI_ERR_CAPACITY and tot.value == len(s_h)
    api.check(lib.intersectDeviceGpu(idx.h, d_qs, d_qe, None, 4, 0, d_off, d_s, d_e, d_h, 16, C.byref(tot), None))
    k = tot.value
    assert np.array_equal(host(d_off, 5, np.int64), off_h)
    assert np.array_equal(host(d_s, k, np.int32), s_h) and np.array_equal(host(d_e, k, np.int32), e_h)
    assert np.array_equal(host(d_h, k, np.int32), h_h)
    api.check(lib.differenceDeviceGpu(idx.h, d_qs, d_qe, None, 4, d_off, d_s, d_e, 16, C.byref(tot), None))
    k = tot.value
    assert np.array_equal(host(d_off, 5, np.int64), doff_h)
    assert np.array_equal(host(d_s, k, np.int32), ds_h) and np.array_equal(host(d_e, k, np.int32), de_h)
    d_qc = dev(np.array([0, 0, 3, 0], np.int32))      # contig 3 does not exist
    st = lib.differenceDeviceGpu(idx.h, d_qs, d_qe, d_qc, 4, d_off, d_s, d_e, 16, C.byref(tot), None)
    assert st == api._capi.SI_ERR_INVALID
    for p in (d_qs, d_qe, d_off, d_s, d_e, d_h, d_qc):
        lib.deviceFreeGpu(p)
    idx.close()


def test_python_intervalmap_setops(api):
    """IntervalMap.intersection / difference against the reference fixture
    (results are built maps: compared as sorted (start, end, data) lists)."""
    g = load("setops_sparse_int32")
    A = api.IntervalMap.from_arrays(g["a_starts"], g["a_ends"], list(g["a_data"].tolist()))
    B = api.IntervalMap.from_arrays(g["b_starts"], g["b_ends"], list(g["b_data"].tolist()))
    got = A.intersection(B, combine=lambda a, b: a)
    want = sorted(zip(g["ref_isect_starts"].tolist(), g["ref_isect_ends"].tolist(), g["ref_isect_data"].tolist()))
    assert sorted(got.at(i) for i in range(got.size())) == want
    got = A.difference(B)
    want = sorted(zip(g["ref_diff_starts"].tolist(), g["ref_diff_ends"].tolist(), g["ref_diff_data"].tolist()))
    assert sorted(got.at(i) for i in range(got.size())) == want


@pytest.mark.parametrize("name", fixture_names())
def test_keys_and_coverage_fixture_parity(api, name):
    """search_keys (both orders) and coverage against the reference's own outputs."""
    g = load(name)
    idx = _index(api, g["starts"], g["ends"], g["data"], path="batched")
    rs, re_ = g["ref_sorted_starts"], g["ref_sorted_ends"]
    qs, qe = g["q_starts"], g["q_ends"]
    off, s, e = idx.search_keys(qs, qe, order=api.ORDER_IDXS_CPP)
    assert np.array_equal(off, g["ref_search_idxs_off"])
    pos = g["ref_search_idxs"].astype(np.int64)
    assert np.array_equal(s, rs[pos]) and np.array_equal(e, re_[pos])
    cnt, cov = idx.coverage(qs, qe)
    assert np.array_equal(cnt.astype(np.int64), g["ref_coverage_count"].astype(np.int64))
    assert np.array_equal(cov, g["ref_coverage"].astype(cov.dtype))
    if "ref_c_search_idxs" in g:      # the fully descending order
        off, s, e = idx.search_keys(qs, qe, order=api.ORDER_DESC)
        pos = g["ref_c_search_idxs"].astype(np.int64)
        assert np.array_equal(s, rs[pos]) and np.array_equal(e, re_[pos])
    idx.close()


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_coverage_from_ranks_extremes(api, oracle, dt):
    """Coverage from ranks and prefix sums (no interval and no query with start > end) against
    the oracle, with coordinates at both ends of the type (wrapped sums, qe at the maximum);
    then the same batch with some start > end queries, which takes the hit-list path."""
    r = np.random.default_rng(31)
    info = np.iinfo(dt)
    n = 20_000
    lo_part = info.min + r.integers(0, 2_000_000, n // 2)
    hi_part = info.max - r.integers(0, 2_000_000, n // 2)
    starts = np.concatenate([lo_part, hi_part]).astype(np.int64)
    lens = r.integers(0, 300_000, n)
    ends = np.where(starts > info.max - lens, info.max, starts + lens).astype(dt)   # no overflow
    starts = starts.astype(dt)
    ends[:50] = info.max                                  # reaching the maximum
    assert (starts <= ends).all()
    nq = 6_000
    qs = np.concatenate([info.min + r.integers(0, 2_500_000, nq // 2),
                         info.max - r.integers(0, 2_500_000, nq // 2)]).astype(np.int64)
    qln = r.integers(0, 400_000, nq)
    qe = np.where(qs > info.max - qln, info.max, qs + qln)
    qe[:40] = info.max
    qs, qe = qs.astype(dt), qe.astype(dt)
    assert (qs <= qe).all()
    idx = _index(api, starts, ends, None, path="batched")
    m = oracle.build(starts, ends, np.arange(n, dtype=np.int32))
    cnt, cov = idx.coverage(qs, qe)
    rc, rv = oracle.coverage(m, qs, qe)
    assert np.array_equal(cnt.astype(np.int64), rc) and np.array_equal(cov, rv)
    flip = r.random(nq) < 0.05
    qs2, qe2 = qs.copy(), qe.copy()
    qs2[flip], qe2[flip] = qe[flip], qs[flip]
    cnt, cov = idx.coverage(qs2, qe2)
    rc, rv = oracle.coverage(m, qs2, qe2)
    assert np.array_equal(cnt.astype(np.int64), rc) and np.array_equal(cov, rv)
    idx.close()


def test_keys_and_coverage_multicontig(api, oracle):
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=100_000, nq=20_000, contigs=W.HUMAN_CONTIGS[20:24])
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    bs, be, bd, _ = idx.arrays()
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_DESC)
    koff, ks, ke, kd = idx.search_keys(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_DESC, with_data=True)
    glo = wl.seg[wl.q_contig].repeat(np.diff(off)) + out    # global positions of the hits
    assert np.array_equal(koff, off)
    assert np.array_equal(ks, bs[glo]) and np.array_equal(ke, be[glo]) and np.array_equal(kd, bd[glo])
    cnt, cov = idx.coverage(wl.q_starts, wl.q_ends, wl.q_contig)
    for gi in range(len(wl.seg) - 1):
        lo, hi = int(wl.seg[gi]), int(wl.seg[gi + 1])
        m = oracle.build(wl.starts[lo:hi], wl.ends[lo:hi], wl.data[lo:hi])
        sel = np.nonzero(wl.q_contig == gi)[0][:500]
        rc, rv = oracle.coverage(m, wl.q_starts[sel], wl.q_ends[sel])
        assert np.array_equal(cnt[sel].astype(np.int64), rc) and np.array_equal(cov[sel], rv)
    idx.close()


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_keys_records_both_widths(api, dt):
    """Keys gathered through the (start, end, payload) records, both coordinate widths, both
    orders, against the index's own arrays at the hit positions."""
    from superintervals_gb300 import workloads as W
    wl = W.random_nested(41, 20_000, 5_000, dtype=dt, span=1_000_000, max_len=20_000)
    idx = _index(api, wl.starts, wl.ends, wl.data, path="batched")
    bs, be, bd, _ = idx.arrays()
    for order in (api.ORDER_DESC, api.ORDER_IDXS_CPP):
        off, out = idx.search(wl.q_starts, wl.q_ends, order=order)
        koff, ks, ke, kd = idx.search_keys(wl.q_starts, wl.q_ends, order=order, with_data=True)
        assert np.array_equal(koff, off)
        assert np.array_equal(ks, bs[out]) and np.array_equal(ke, be[out]) and np.array_equal(kd, bd[out])
    idx.close()


def test_python_keys_items_coverage(api):
    """The Python mirror's single-query search_keys / search_items / coverage (pyx:302-361)."""
    g = load("kat_coverage_int32")
    imap = api.IntervalMap.from_arrays(g["starts"], g["ends"], ["v%d" % i for i in g["data"].tolist()])
    q0, q1 = int(g["q_starts"][0]), int(g["q_ends"][0])
    assert imap.coverage(q0, q1) == (int(g["ref_coverage_count"][0]), int(g["ref_coverage"][0]))
    idxs = imap.search_idxs(q0, q1)
    assert imap.search_keys(q0, q1) == [(imap.starts_at(i), imap.ends_at(i)) for i in idxs]
    assert imap.search_items(q0, q1) == [imap.at(i) for i in idxs]
