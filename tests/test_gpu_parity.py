"""GPU parity: the CUDA path (called through the C-ABI) against the golden
fixtures made by the reference itself and against the oracle on seeded
inputs.  Integer work: everything is compared bit-exactly, except payload
order inside runs of exact (start, end) duplicates, where the reference's
std::sort leaves it unspecified (checked as a permutation)."""
import numpy as np
import pytest

from golden_util import assert_data_parity, fixture_names, load

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
    idx.set_path({"plain": api.PATH_PLAIN, "batched": api.PATH_BATCHED, "auto": api.PATH_AUTO}[path])
    return idx


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("name", fixture_names())
def test_fixture_parity(api, name, path):
    g = load(name)
    idx = _index(api, g["starts"], g["ends"], g["data"], path=path)
    s, e, d, b = idx.arrays()
    assert np.array_equal(s, g["ref_sorted_starts"])
    assert np.array_equal(e, g["ref_sorted_ends"])
    assert np.array_equal(b, g["ref_branch"].astype(np.int64))
    assert_data_parity(s, e, g["ref_sorted_data"], d)
    qs, qe = g["q_starts"], g["q_ends"]
    cnt = idx.count(qs, qe)
    assert np.array_equal(cnt.astype(np.int64), g["ref_count"].astype(np.int64))
    off, out = idx.search(qs, qe, order=api.ORDER_IDXS_CPP)
    assert np.array_equal(off, g["ref_search_idxs_off"])
    assert np.array_equal(out, g["ref_search_idxs"])
    offd, outd = idx.search(qs, qe, order=api.ORDER_DESC)
    assert np.array_equal(offd, off)
    if "ref_c_search_idxs" in g:
        assert np.array_equal(outd, g["ref_c_search_idxs"])
    offv, outv = idx.search(qs, qe, order=api.ORDER_DESC, values=True)
    assert np.array_equal(offv, g["ref_search_values_off"])
    assert np.array_equal(outv, d[outd])                       # own payload at the hit positions
    assert np.array_equal(g["ref_search_values"], g["ref_sorted_data"][outd])
    hv = idx.has_overlaps(qs, qe)
    assert np.array_equal(hv.astype(np.int32), g["ref_has_overlaps"].astype(np.int32))
    idx.close()


@pytest.mark.parametrize("path", PATHS)
def test_multicontig_stream(api, path):
    s = load("contigs3_stream_int32")
    idx = _index(api, s["starts"], s["ends"], s["data"], seg=s["seg"], path=path)
    off, out = idx.search(s["q_starts"], s["q_ends"], s["q_contig"], order=api.ORDER_IDXS_CPP)
    for gi in range(3):
        g = load(f"contigs3_g{gi}_int32")
        got = [out[off[q]:off[q + 1]].tolist() for q in g["q_index"]]
        ro, rv = g["ref_search_idxs_off"], g["ref_search_idxs"]
        assert got == [rv[ro[i]:ro[i + 1]].tolist() for i in range(len(ro) - 1)]
    cnt = idx.count(s["q_starts"], s["q_ends"], s["q_contig"])
    assert np.array_equal(cnt.astype(np.int64), np.diff(off))
    idx.close()


def _oracle_case(api, oracle, wl, path, orders=(0, 1)):
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path=path)
    m = oracle.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    s, e, d, b = idx.arrays()
    assert np.array_equal(s, m["starts"]) and np.array_equal(e, m["ends"])
    assert np.array_equal(b, m["branch"])
    assert np.array_equal(d, m["data"])          # both sorts are stable
    cnt = idx.count(wl.q_starts, wl.q_ends, wl.q_contig)
    rc = oracle.count_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, nthreads=8)
    assert np.array_equal(cnt, rc)
    for order in orders:
        off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=order)
        ro, rv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=order,
                                     nthreads=8, counts=rc)
        assert np.array_equal(off, ro)
        assert np.array_equal(out, rv)
    idx.close()


@pytest.mark.parametrize("path", PATHS)
def test_config1_full(api, oracle, path):
    from superintervals_gb300 import workloads as W
    _oracle_case(api, oracle, W.config1(), path)


@pytest.mark.parametrize("path", PATHS)
def test_config2_scaled(api, oracle, path):
    from superintervals_gb300 import workloads as W
    _oracle_case(api, oracle, W.config2(n=1_000_000, nq=200_000), path, orders=(0,))


@pytest.mark.parametrize("path", PATHS)
def test_config3_scaled(api, oracle, path):
    from superintervals_gb300 import workloads as W
    _oracle_case(api, oracle, W.config3(n=1_000_000, nq=300_000), path, orders=(0, 1))


def _host_threads():
    import os
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def test_config3_full_density_contig_subset(api, oracle):
    """The headline configuration's density on two of its contigs: 50 M intervals and queries
    over the 24 contigs, scaled to chr21 + chr22 by their share of the genome (1.58 M of each),
    so ~500 hits per query from the 1% of 1-5 Mb intervals (nesting depth ~500).  This runs the
    batched path the way the full workload does: rank counts, the automatic tile size at its
    densest, long candidate lists holding nearly every hit, and the per-query miss handling of
    long candidates.  The whole batch is compared with the oracle (superintervals.hpp:879-905
    order, the fully descending order and payloads), with the default and the autotuned
    tunables and the learned upper bound."""
    import ctypes as C
    from superintervals_gb300 import autotune, workloads as W
    wl = W.config3_subset(["chr21", "chr22"])
    nth = _host_threads()
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    idx.set_upper_bound(api.UB_LEARNED)
    m = oracle.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    rc = oracle.count_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, nthreads=nth)
    assert rc.sum() / wl.nq > 400                      # the headline's hits per query
    assert np.array_equal(idx.count(wl.q_starts, wl.q_ends, wl.q_contig), rc)
    ro, rv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=0, nthreads=nth, counts=rc)
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_IDXS_CPP)
    assert np.array_equal(off, ro) and np.array_equal(out, rv)
    del out
    # the autotuned tunables, as the benchmark runs them (timed on the whole device batch)
    lib = idx.lib
    dev = []
    for a in (wl.q_starts, wl.q_ends, wl.q_contig):
        p = C.c_void_p()
        api.check(lib.deviceMallocGpu(C.byref(p), a.nbytes))
        api.check(lib.memcpyGpu(p, C.c_void_p(a.ctypes.data), a.nbytes, idx.stream))
        dev.append(p)
    choice = autotune.tune(idx, dev[0], dev[1], dev[2], wl.nq, sample=0, use_cache=False, keep_upper_bound=True)
    for p in dev:
        lib.deviceFreeGpu(p)
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_IDXS_CPP)
    assert np.array_equal(off, ro) and np.array_equal(out, rv), choice
    del out, rv
    ro1, rv1 = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=1, nthreads=nth, counts=rc)
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_DESC)
    assert np.array_equal(off, ro1) and np.array_equal(out, rv1)
    del out, rv1
    _, rvv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=1, values=True, nthreads=nth,
                                 counts=rc)
    _, outv = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=api.ORDER_DESC, values=True)
    assert np.array_equal(outv, rvv)
    idx.close()


@pytest.mark.parametrize("path", PATHS)
def test_config3_long_queries_scaled(api, oracle, path):
    from superintervals_gb300 import workloads as W
    _oracle_case(api, oracle, W.config3(n=200_000, nq=50_000, long_queries=True), path, orders=(0,))


@pytest.mark.parametrize("inverted_intervals", [False, True])
def test_query_classes_both_count_modes(api, oracle, inverted_intervals):
    """Short, long and start > end queries in one batch.  Without inverted intervals the
    batched path counts every query with start <= end from two ranks (and the count pass
    only the start > end ones); with some, it counts all of them from the tile lists."""
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=200_000, nq=60_000, long_queries=True)
    r = np.random.default_rng(5)
    flip = r.random(wl.nq) < 0.03
    wl.q_starts[flip], wl.q_ends[flip] = wl.q_ends[flip].copy(), wl.q_starts[flip].copy()
    assert (wl.q_starts > wl.q_ends).any()
    if inverted_intervals:
        inv = r.random(wl.n) < 0.005
        wl.starts[inv], wl.ends[inv] = wl.ends[inv].copy(), wl.starts[inv].copy()
        assert (wl.starts > wl.ends).any()
    _oracle_case(api, oracle, wl, "batched", orders=(0, 1))


@pytest.mark.parametrize("layout,dt", [("reads_24_contigs", np.int32), ("many_small_contigs", np.int32),
                                       ("many_small_contigs", np.int64)])
def test_branch_fixed_length_reads_multicontig(api, oracle, layout, dt):
    """Fixed-length reads: every end exceeds all earlier ends of its contig, so the branch pass's
    cross-tile step decides nearly every position (-1 unless an earlier read of the same contig
    reaches it).  Its prefix maxima are per contig: a contig's first positions must not see the
    larger ends of the contig before it.  Many small contigs put contig starts inside tiles, and
    some contigs are empty."""
    from superintervals_gb300 import workloads as W
    r = np.random.default_rng(17)
    if layout == "reads_24_contigs":
        sizes = np.array([c[1] for c in W.HUMAN_CONTIGS], np.int64)
        counts = np.maximum(1, (300_000 * sizes / sizes.sum()).astype(np.int64))
        lens = sizes
    else:
        counts = r.integers(0, 1500, 600)
        counts[r.random(600) < 0.1] = 0
        lens = r.integers(10_000, 2_000_000, 600)
    seg = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    starts = np.concatenate([r.integers(0, ln - 200, c) for c, ln in zip(counts, lens)]).astype(dt)
    ln = np.where(r.random(starts.size) < 0.02, 5_000, 150)      # a few longer reads
    ends = (starts + ln - 1).astype(dt)
    n = starts.size
    qc = r.integers(0, len(counts), 20_000).astype(np.int32)
    qs = (r.random(20_000) * lens[qc]).astype(dt)
    wl = W.Workload(name=layout, starts=starts, ends=ends, data=np.arange(n, dtype=np.int32), seg=seg,
                    q_starts=qs, q_ends=(qs + 300).astype(dt), q_contig=qc)
    _oracle_case(api, oracle, wl, "batched", orders=(0,))


@pytest.mark.parametrize("path", ["plain", "auto"])
@pytest.mark.parametrize("inverted_intervals", [False, True])
@pytest.mark.parametrize("nq", [1, 20_000, 40_000])
def test_small_batches_dense(api, oracle, inverted_intervals, nq, path):
    """Small batches at the headline density (chr21's share of configuration 3, ~500 hits per
    query from deeply nested 1-5 Mb intervals).  On the plain path, batches of up to 32768 queries
    take one warp per query: the count from two ranks (no interval with start > end and query
    start <= end) or a 32-wide ballot walk that skips misses through the branch array, and the
    emit's 32-wide head run and walk; larger batches one thread per query.  The automatic path
    sends searches of fewer than 4096 queries over such deeply nested long intervals to the
    batched path and their counts to the plain one.  Some queries have start > end, and in one
    case some intervals too."""
    import dataclasses
    from superintervals_gb300 import workloads as W
    wl = W.config3_subset(["chr21"])
    r = np.random.default_rng(11)
    qs, qe = wl.q_starts[:nq].copy(), wl.q_ends[:nq].copy()
    flip = r.random(nq) < 0.03
    qs[flip], qe[flip] = qe[flip].copy(), qs[flip].copy()
    starts, ends = wl.starts.copy(), wl.ends.copy()
    if inverted_intervals:
        inv = r.random(wl.n) < 0.005
        starts[inv], ends[inv] = ends[inv].copy(), starts[inv].copy()
    small = dataclasses.replace(wl, starts=starts, ends=ends, q_starts=qs, q_ends=qe,
                                q_contig=None if wl.q_contig is None else wl.q_contig[:nq].copy())
    _oracle_case(api, oracle, small, path, orders=(0, 1))


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("seed,dt", [(21, np.int32), (22, np.int64), (23, np.int32)])
def test_random_nested(api, oracle, seed, dt, path):
    from superintervals_gb300 import workloads as W
    _oracle_case(api, oracle, W.random_nested(seed, 30_000, 20_000, dtype=dt, span=2_000_000,
                                              max_len=3_000), path)


@pytest.mark.parametrize("path", PATHS)
def test_config4_scaled_int64(api, oracle, path):
    from superintervals_gb300 import workloads as W
    wl = W.config4(n=300_000, nq=20_000, span=3_100_000_000)
    idx = _index(api, wl.starts, wl.ends, wl.data, path=path)
    m = oracle.build(wl.starts, wl.ends, wl.data)
    s, e, d, b = idx.arrays()
    assert np.array_equal(s, m["starts"]) and np.array_equal(b, m["branch"])
    cnt = idx.count(wl.q_starts, wl.q_ends)
    assert np.array_equal(cnt, oracle.count_batch(m, wl.q_starts, wl.q_ends, nthreads=8))
    hv = idx.has_overlaps(wl.q_starts, wl.q_ends)
    assert np.array_equal(hv.astype(np.int32), oracle.has_overlaps_batch(m, wl.q_starts, wl.q_ends))
    idx.close()


UB_MODES = ["binary", "eytzinger", "learned"]


def _ub_const(api, mode):
    return {"binary": api.UB_BINARY, "eytzinger": api.UB_EYTZINGER, "learned": api.UB_LEARNED}[mode]


@pytest.mark.parametrize("mode", UB_MODES)
@pytest.mark.parametrize("name", ["config1_plain_small_int32", "nested_dups_int64", "edges_int32",
                                  "edges_int64", "kat_single_int32", "presorted_int32"])
def test_batched_upper_bound_modes(api, name, mode):
    """Batched search_idxs is bit-identical whatever provider finds the upper bounds."""
    g = load(name)
    idx = _index(api, g["starts"], g["ends"], g["data"], path="batched")
    idx.set_upper_bound(_ub_const(api, mode))
    off, out = idx.search(g["q_starts"], g["q_ends"], order=api.ORDER_IDXS_CPP)
    assert np.array_equal(off, g["ref_search_idxs_off"])
    assert np.array_equal(out, g["ref_search_idxs"])
    idx.close()


def _device_ub(api, idx, qe, qc, mode):
    import ctypes as C
    lib = idx.lib
    qe = np.ascontiguousarray(qe, dtype=idx.dtype)
    n = qe.shape[0]
    d_qe, d_qc, d_out = C.c_void_p(), C.c_void_p(), C.c_void_p()
    api.check(lib.deviceMallocGpu(C.byref(d_qe), max(qe.nbytes, 1)))
    api.check(lib.deviceMallocGpu(C.byref(d_out), max(4 * n, 1)))
    api.check(lib.memcpyGpu(d_qe, C.c_void_p(qe.ctypes.data), qe.nbytes, idx.stream))
    if qc is not None:
        qc = np.ascontiguousarray(qc, dtype=np.int32)
        api.check(lib.deviceMallocGpu(C.byref(d_qc), max(qc.nbytes, 1)))
        api.check(lib.memcpyGpu(d_qc, C.c_void_p(qc.ctypes.data), qc.nbytes, idx.stream))
    api.check(lib.upperBoundDeviceGpu(idx.h, d_qe, d_qc if qc is not None else None, n, mode, d_out,
                                      idx.stream))
    out = np.empty(n, np.int32)
    api.check(lib.memcpyGpu(C.c_void_p(out.ctypes.data), d_out, 4 * n, idx.stream))
    api.check(lib.streamSynchronizeGpu(idx.stream))
    for p in (d_qe, d_qc, d_out):
        if p.value:
            lib.deviceFreeGpu(p)
    return out


@pytest.mark.parametrize("path", PATHS)
@pytest.mark.parametrize("mode", UB_MODES)
def test_upper_bound_providers_exact(api, mode, path):
    """Every provider returns the reference's upper_bound (hpp:501-516) for every query,
    including values before the first start, after the last one and on duplicates: per query
    (plain path) and through the sorted batch (batched path)."""
    from superintervals_gb300 import workloads as W
    for wl in (W.config4(n=400_000, nq=100_000), W.config3(n=300_000, nq=100_000),
               W.random_nested(41, 5000, 5000, dtype=np.int64)):
        idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None,
                     path=path)
        idx.set_upper_bound(_ub_const(api, mode))
        s, _, _, _ = idx.arrays()
        qe = np.concatenate([wl.q_ends, s[:1000], s[:1000] - 1, [s.min() - 5, s.max() + 5]]).astype(idx.dtype)
        qc = None
        if wl.q_contig is not None:
            qc = np.concatenate([wl.q_contig, np.zeros(2002, np.int32)])
        got = _device_ub(api, idx, qe, qc, _ub_const(api, mode))
        segs = wl.seg
        exp = np.empty(qe.shape[0], np.int64)
        cid = np.zeros(qe.shape[0], np.int64) if qc is None else qc
        for gi in range(len(segs) - 1):
            sel = cid == gi
            ss = s[segs[gi]:segs[gi + 1]]
            exp[sel] = np.searchsorted(ss, qe[sel], side="right") - 1
        assert np.array_equal(got.astype(np.int64), exp)
        idx.close()


@pytest.mark.parametrize("nq", [3_000, 40_000, 400_000])
def test_automatic_tile_size_is_exact(api, oracle, nq):
    """The per-batch tile size (from intervals and hits per query) against a fixed one and
    the oracle, from sparse batches (small tiles, walks) to dense ones."""
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=2_000_000, nq=nq)
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig)
    api.check(idx.lib.setBatchedParamsGpu(idx.h, 256, 0, 0, -1))
    off2, out2 = idx.search(wl.q_starts, wl.q_ends, wl.q_contig)
    assert np.array_equal(off, off2) and np.array_equal(out, out2)
    api.check(idx.lib.setBatchedParamsGpu(idx.h, -1, 0, 0, -1))
    m = oracle.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    sel = np.arange(0, nq, max(1, nq // 2000))
    ro, rv = oracle.search_batch(m, wl.q_starts[sel], wl.q_ends[sel], wl.q_contig[sel], order=0, nthreads=8)
    got = [out[off[q]:off[q + 1]].tolist() for q in sel]
    assert got == [rv[ro[i]:ro[i + 1]].tolist() for i in range(len(sel))]
    idx.close()


@pytest.mark.parametrize("tile_q,cap,long_len,split", [(32, 256, 1 << 40, 2048), (64, 256, 50, 0),
                                                       (1024, 8192, 1 << 14, 1), (128, 512, 2000, 1 << 40),
                                                       (256, 2048, 1 << 14, 300)])
def test_batched_params_and_overflow_walks(api, oracle, tile_q, cap, long_len, split):
    """Small candidate capacity forces the per-query warp walk, a tiny long-query
    threshold sends most queries there, large tiles stress the shared gather: every
    setting returns the same bit-exact result."""
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=200_000, nq=40_000, long_queries=True)
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    api.check(idx.lib.setBatchedParamsGpu(idx.h, tile_q, cap, long_len, split))
    m = oracle.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    rc = oracle.count_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, nthreads=8)
    assert np.array_equal(idx.count(wl.q_starts, wl.q_ends, wl.q_contig), rc)
    for order in (0, 1):
        off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=order)
        ro, rv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=order, nthreads=8,
                                     counts=rc)
        assert np.array_equal(off, ro) and np.array_equal(out, rv)
    offv, outv = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=1, values=True)
    _, rv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, order=1, values=True,
                                nthreads=8, counts=rc)
    assert np.array_equal(outv, rv)
    idx.close()


@pytest.mark.parametrize("path", PATHS)
def test_chunked_emit_matches_unchunked(api, oracle, path):
    from superintervals_gb300 import workloads as W
    wl = W.random_nested(31, 20_000, 20_000, span=500_000, max_len=5_000)
    idx = _index(api, wl.starts, wl.ends, wl.data, path=path)
    off1, out1 = idx.search(wl.q_starts, wl.q_ends)
    idx.set_output_budget(1 << 20)       # 1 MiB: forces many chunks
    off2, out2 = idx.search(wl.q_starts, wl.q_ends)
    assert int(off1[-1]) * 4 > (1 << 21)
    assert np.array_equal(off1, off2) and np.array_equal(out1, out2)
    idx.close()


def test_rebuild_after_more_adds(api, oracle):
    g = load("nested_dups_int32")
    n = g["starts"].shape[0]
    idx = api.GpuIndex(32)
    idx.add_arrays(g["starts"][: n // 2], g["ends"][: n // 2], g["data"][: n // 2])
    idx.build()
    idx.add_arrays(g["starts"][n // 2:], g["ends"][n // 2:], g["data"][n // 2:])
    with pytest.raises(api.SIError):
        idx.count(g["q_starts"], g["q_ends"])         # added after build: must rebuild
    idx.build()
    off, out = idx.search(g["q_starts"], g["q_ends"])
    assert np.array_equal(off, g["ref_search_idxs_off"]) and np.array_equal(out, g["ref_search_idxs"])
    idx.close()


def test_errors_are_reported(api):
    idx = api.GpuIndex(32)
    idx.add_arrays(np.array([1, 5], np.int32), np.array([3, 9], np.int32))
    with pytest.raises(api.SIError) as ei:
        idx.count([1], [2])
    assert ei.value.status == 3                       # NOT_BUILT
    idx.build()
    with pytest.raises(api.SIError) as ei:
        idx.count([1], [2], qc=[1])                   # only contig 0 exists
    assert ei.value.status == 1
    idx64 = api.GpuIndex(64)
    assert idx64.lib.addIntervalGpu(idx64.h, 1, 2, 3) == 1   # 32-bit add on a 64-bit handle
    assert int(idx.count([1], [2])[0]) == 1           # the handle is still usable
    idx.close()
    idx64.close()


def test_device_budget_rejects_oversize(api):
    lib = api._capi.load()
    used = lib.deviceBytesInUseGpu()
    lib.setDeviceBudgetGpu(used + (1 << 20))
    try:
        idx = api.GpuIndex(32)
        n = 2_000_000
        idx.add_arrays(np.arange(n, dtype=np.int32), np.arange(n, dtype=np.int32) + 5)
        with pytest.raises(api.SIError) as ei:
            idx.build()
        assert ei.value.status == 2                   # OOM by admission, no fault
    finally:
        lib.setDeviceBudgetGpu(0)
    idx.build()
    assert int(idx.count([10], [10])[0]) == 6
    idx.close()


def test_python_intervalmap_dropin(api):
    """The README batch example of the reference Python API (README.md:16-27)."""
    from array import array
    IM = api.IntervalMap
    imap = IM()
    imap.add(10, 20, "A")
    imap.add(15, 25, "B")
    imap.build()
    assert imap.search_values(8, 20) == ["B", "A"]
    imap = IM.from_arrays(array("i", [10, 15, 30]), array("i", [20, 25, 40]), ["A", "B", "C"])
    qs, qe = array("i", [5, 18, 35]), array("i", [12, 22, 45])
    assert imap.count_batch(qs, qe) == [1, 2, 1]
    assert imap.search_idxs_batch(qs, qe) == [[0], [0, 1], [2]]
    assert imap.search_values_batch(qs, qe) == [["A"], ["B", "A"], ["C"]]
    assert imap.at(1) == (15, 25, "B")
    with pytest.raises(IndexError):
        imap.at(3)
    with pytest.raises(ValueError):
        imap.count_batch(array("i", [1, 2]), array("i", [3]))


@pytest.mark.parametrize("path", PATHS)
def test_pinned_host_output_matches(api, oracle, path):
    """searchBatchIntoGpu into pinned host buffers (written directly by the emit kernel)
    gives the same CSR as into pageable buffers."""
    import ctypes as C
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=200_000, nq=50_000)
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path=path)
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig)
    lib = idx.lib
    P, nq = int(off[-1]), wl.nq
    h_off, h_out = C.c_void_p(), C.c_void_p()
    api.check(lib.hostMallocPinnedGpu(C.byref(h_off), 8 * (nq + 1)))
    api.check(lib.hostMallocPinnedGpu(C.byref(h_out), 4 * P))
    qs, qe, qc = (np.ascontiguousarray(a) for a in (wl.q_starts, wl.q_ends, wl.q_contig))
    tot = C.c_size_t()
    for order in (0, 1):
        api.check(lib.searchBatchIntoGpu(idx.h, C.c_void_p(qs.ctypes.data), C.c_void_p(qe.ctypes.data),
                                         C.c_void_p(qc.ctypes.data), nq, order, 0, h_off, h_out, P, C.byref(tot)))
        got_off = np.ctypeslib.as_array(C.cast(h_off, C.POINTER(C.c_int64)), shape=(nq + 1,)).copy()
        got_out = np.ctypeslib.as_array(C.cast(h_out, C.POINTER(C.c_int32)), shape=(P,)).copy()
        ro, rv = idx.search(wl.q_starts, wl.q_ends, wl.q_contig, order=order)
        assert np.array_equal(got_off, ro) and np.array_equal(got_out, rv)
    lib.hostFreePinnedGpu(h_off)
    lib.hostFreePinnedGpu(h_out)
    idx.close()


class _Dev:
    """Device copies of a query batch plus result buffers, through the C-ABI helpers."""

    def __init__(self, api, idx, wl):
        import ctypes as C
        self.C, self.api, self.lib, self.idx = C, api, idx.lib, idx
        self.ptrs = []
        dt = idx.dtype
        self.nq = wl.nq
        self.qs = self.put(np.ascontiguousarray(wl.q_starts, dt))
        self.qe = self.put(np.ascontiguousarray(wl.q_ends, dt))
        self.qc = None if wl.q_contig is None else self.put(np.ascontiguousarray(wl.q_contig, np.int32))
        self.off = self.alloc(8 * (self.nq + 1))

    def alloc(self, nbytes):
        p = self.C.c_void_p()
        self.api.check(self.lib.deviceMallocGpu(self.C.byref(p), max(int(nbytes), 1)))
        self.ptrs.append(p)
        return p

    def put(self, arr):
        p = self.alloc(arr.nbytes)
        self.api.check(self.lib.memcpyGpu(p, self.C.c_void_p(arr.ctypes.data), arr.nbytes, self.idx.stream))
        return p

    def get(self, p, n, dtype):
        out = np.empty(n, dtype)
        if n:
            self.api.check(self.lib.memcpyGpu(self.C.c_void_p(out.ctypes.data), p, out.nbytes, self.idx.stream))
        self.api.check(self.lib.streamSynchronizeGpu(self.idx.stream))
        return out

    def close(self):
        for p in self.ptrs:
            self.lib.deviceFreeGpu(p)


def test_autotuner_keeps_results_exact(api, oracle):
    import ctypes as C
    import json
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=400_000, nq=120_000)
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    d = _Dev(api, idx, wl)
    rep = C.create_string_buffer(512)
    api.check(idx.lib.autotuneBatchedGpu(idx.h, d.qs, d.qe, d.qc, d.nq, 50_000, 0, rep, 512))
    tuned = json.loads(rep.value.decode())
    assert tuned["trials"] >= 10 and tuned["upper_bound"] in (0, 1, 2)
    m = oracle.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    off, out = idx.search(wl.q_starts, wl.q_ends, wl.q_contig)
    ro, rv = oracle.search_batch(m, wl.q_starts, wl.q_ends, wl.q_contig, nthreads=8)
    assert np.array_equal(off, ro) and np.array_equal(out, rv)
    d.close()
    idx.close()


@pytest.mark.parametrize("path,inverted", [("plain", False), ("batched", False), ("batched", True)])
def test_graph_replay_matches_and_respects_capacity(api, path, inverted):
    """searchDeviceGraphGpu: the plain path, or the whole batched path (prepare, count, scan,
    emit) captured once and replayed, also on new query contents in the same buffers."""
    import ctypes as C
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=200_000, nq=30_000)
    if inverted:        # intervals with start > end: the batched path counts from its tile lists
        inv = np.random.default_rng(4).random(wl.n) < 0.003
        wl.starts[inv], wl.ends[inv] = wl.ends[inv].copy(), wl.starts[inv].copy()
    idx = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path=path)
    d = _Dev(api, idx, wl)
    off_ref, out_ref = idx.search(wl.q_starts, wl.q_ends, wl.q_contig)
    P = int(off_ref[-1])
    # a second batch of the same shape (the same queries permuted), answered eagerly first
    perm = np.random.default_rng(8).permutation(d.nq)
    qs2, qe2 = wl.q_starts[perm], wl.q_ends[perm]
    qc2 = None if wl.q_contig is None else wl.q_contig[perm]
    off2, out2 = idx.search(qs2, qe2, qc2)
    d_out = d.alloc(4 * P + 4096)
    tot = C.c_size_t()
    launches0 = idx.lib.getLaunchCountGpu()
    for _ in range(3):   # first call captures, the others replay
        api.check(idx.lib.searchDeviceGraphGpu(idx.h, d.qs, d.qe, d.qc, d.nq, 0, d.off, d_out, P + 1024,
                                               C.byref(tot), None))
        assert int(tot.value) == P
        assert np.array_equal(d.get(d.off, d.nq + 1, np.int64), off_ref)
        assert np.array_equal(d.get(d_out, P, np.int32), out_ref)
    assert idx.lib.getLaunchCountGpu() > launches0
    # new queries in the same buffers: a replay, not a new capture
    if int(off2[-1]) <= P + 1024:
        for arr, ptr in ((qs2, d.qs), (qe2, d.qe), (qc2, d.qc)):
            if arr is not None:
                a = np.ascontiguousarray(arr)
                api.check(idx.lib.memcpyGpu(ptr, C.c_void_p(a.ctypes.data), a.nbytes, idx.stream))
        api.check(idx.lib.searchDeviceGraphGpu(idx.h, d.qs, d.qe, d.qc, d.nq, 0, d.off, d_out, P + 1024,
                                               C.byref(tot), None))
        assert np.array_equal(d.get(d.off, d.nq + 1, np.int64), off2)
        assert np.array_equal(d.get(d_out, int(off2[-1]), np.int32), out2)
    # too small an output: reported, nothing written past the end
    small = P // 2
    guard = d.alloc(4 * (small + 1024))
    sentinel = np.full(small + 1024, -9, np.int32)
    api.check(idx.lib.memcpyGpu(guard, C.c_void_p(sentinel.ctypes.data), sentinel.nbytes, idx.stream))
    st = idx.lib.searchDeviceGraphGpu(idx.h, d.qs, d.qe, d.qc, d.nq, 0, d.off, guard, small, C.byref(tot), None)
    assert st == 5 and int(tot.value) == P
    tail = d.get(guard, small + 1024, np.int32)[small:]
    assert (tail == -9).all()
    d.close()
    idx.close()


def test_index_image_roundtrip(api, tmp_path):
    """An index saved as an image and loaded into a new handle answers identically; the
    load skips the sort; corrupt, truncated or wrong-width images are rejected."""
    from superintervals_gb300 import workloads as W
    wl = W.config3(n=150_000, nq=20_000, contigs=W.HUMAN_CONTIGS[19:24])
    a = _index(api, wl.starts, wl.ends, wl.data, seg=wl.seg, path="batched")
    want = a.search(wl.q_starts, wl.q_ends, wl.q_contig)
    img = a.to_bytes()
    b = api.GpuIndex(32)
    b.from_bytes(img)
    b.set_path(api.PATH_BATCHED)
    got = b.search(wl.q_starts, wl.q_ends, wl.q_contig)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    for x, y in zip(a.arrays(), b.arrays()):
        assert np.array_equal(x, y)
    p = str(tmp_path / "index.sig")
    a.save(p)
    c = api.GpuIndex(32)
    c.load(p)
    assert np.array_equal(c.count(wl.q_starts, wl.q_ends, wl.q_contig),
                          a.count(wl.q_starts, wl.q_ends, wl.q_contig))
    bad = bytearray(img)
    bad[-8 - 5] ^= 0x40                                 # inside the branch array (before the name count)
    with pytest.raises(api.SIError):
        api.GpuIndex(32).from_bytes(bytes(bad))
    with pytest.raises(api.SIError):
        api.GpuIndex(32).from_bytes(img[: len(img) // 2])
    with pytest.raises(api.SIError):
        api.GpuIndex(64).from_bytes(img)
    for h in (a, b, c):
        h.close()
