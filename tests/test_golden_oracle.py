"""The oracle pinned against the reference: every golden fixture (produced by
the reference's own header and C API, tests/golden/make_golden.py) and the
known answers asserted by the reference's unit tests (test/tests.cpp)."""
import numpy as np
import pytest

from golden_util import (assert_data_parity, assert_values_parity, csr_lists, fixture_names,
                         load)
from oracle.oracle import ORDER_DESC, ORDER_IDXS_CPP, Oracle


@pytest.fixture(scope="module")
def oracle():
    return Oracle()


@pytest.mark.parametrize("name", fixture_names())
def test_oracle_matches_reference_fixture(oracle, name):
    g = load(name)
    m = oracle.build(g["starts"], g["ends"], g["data"])
    n = g["starts"].shape[0]
    assert np.array_equal(m["starts"], g["ref_sorted_starts"])
    assert np.array_equal(m["ends"], g["ref_sorted_ends"])
    assert np.array_equal(m["branch"], g["ref_branch"].astype(np.int64))
    assert_data_parity(m["starts"], m["ends"], g["ref_sorted_data"], m["data"])
    if n == 0:
        return
    qs, qe = g["q_starts"], g["q_ends"]
    cnt = oracle.count_batch(m, qs, qe)
    assert np.array_equal(cnt.astype(np.int64), g["ref_count"].astype(np.int64))
    off, out = oracle.search_batch(m, qs, qe, order=ORDER_IDXS_CPP)
    assert np.array_equal(off, g["ref_search_idxs_off"])
    assert np.array_equal(out, g["ref_search_idxs"])
    offd, outd = oracle.search_batch(m, qs, qe, order=ORDER_DESC)
    assert np.array_equal(offd, off)
    if "ref_c_search_idxs" in g:
        assert np.array_equal(outd, g["ref_c_search_idxs"])
        assert np.array_equal(offd, g["ref_c_search_idxs_off"])
    offv, outv = oracle.search_batch(m, qs, qe, order=ORDER_DESC, values=True)
    assert np.array_equal(offv, g["ref_search_values_off"])
    assert_values_parity(outd, offd, g["ref_sorted_data"], m["data"], g["ref_search_values"], outv)
    hv = oracle.has_overlaps_batch(m, qs, qe)
    assert np.array_equal(hv, g["ref_has_overlaps"].astype(np.int32))
    ccount, ccov = oracle.coverage(m, qs[:2000], qe[:2000])
    assert np.array_equal(ccount, g["ref_coverage_count"][:2000].astype(np.int64))
    assert np.array_equal(ccov, g["ref_coverage"][:2000])


def _vals(g, key, q):
    off = g[f"ref_{key}_off"]
    return g[f"ref_{key}"][off[q]:off[q + 1]].tolist()


@pytest.mark.parametrize("dt", ["int32", "int64"])
def test_reference_unit_test_known_answers(dt):
    """The assertions of test/tests.cpp, checked on the stored reference outputs."""
    g = load(f"kat_basics_{dt}")
    assert _vals(g, "search_values", 0) == [4, 0]          # tests.cpp:84-86
    assert int(g["ref_count"][0]) == 2                        # tests.cpp:89
    assert _vals(g, "search_idxs", 0) == [4, 0]              # tests.cpp:94-95
    assert int(g["ref_has_overlaps"][0]) == 1 and int(g["ref_has_overlaps"][1]) == 0
    assert int(g["ref_coverage"][2]) == 17                    # tests.cpp:105-106
    g = load(f"kat_nested_{dt}")
    v = _vals(g, "search_values", 0)
    assert v[-1] == 0 and len(v) == 12                        # tests.cpp:154-155
    g = load(f"kat_shared_endpoints_{dt}")
    assert [len(_vals(g, "search_values", q)) for q in range(3)] == [3, 2, 3]
    g = load(f"kat_duplicates_{dt}")
    assert [len(_vals(g, "search_values", q)) for q in range(2)] == [6, 3]
    g = load(f"kat_coverage_{dt}")
    assert int(g["ref_coverage_count"][0]) == 3 and int(g["ref_coverage"][0]) == 25
    g = load(f"kat_single_{dt}")
    assert int(g["ref_count"][0]) == 1 and int(g["ref_count"][1]) == 0
    g = load(f"kat_readme_batch_{dt}")
    assert [int(c) for c in g["ref_count"][:3]] == [1, 2, 1]  # README.md:26
    assert csr_lists(g["ref_search_idxs_off"][:4], g["ref_search_idxs"]) == [[0], [0, 1], [2]]


def test_multicontig_stream_matches_per_contig_fixtures(oracle):
    s = load("contigs3_stream_int32")
    m = oracle.build(s["starts"], s["ends"], s["data"], seg=s["seg"])
    off, out = oracle.search_batch(m, s["q_starts"], s["q_ends"], qc=s["q_contig"],
                                   order=ORDER_IDXS_CPP, nthreads=2)
    for gi in range(3):
        g = load(f"contigs3_g{gi}_int32")
        qi = g["q_index"]
        got = [out[off[q]:off[q + 1]].tolist() for q in qi]
        assert got == csr_lists(g["ref_search_idxs_off"], g["ref_search_idxs"])


def test_oracle_threads_agree(oracle):
    g = load("nested_dups_int32")
    m = oracle.build(g["starts"], g["ends"], g["data"])
    a = oracle.search_batch(m, g["q_starts"], g["q_ends"], nthreads=1)
    b = oracle.search_batch(m, g["q_starts"], g["q_ends"], nthreads=4)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_planted_mistake_is_caught(oracle):
    """The parity check is not vacuous: a branch array with one planted error
    changes the reference-order output."""
    g = load("nested_dups_int32")
    m = oracle.build(g["starts"], g["ends"], g["data"])
    bad = dict(m)
    bad["branch"] = m["branch"].copy()
    k = int(np.nonzero(m["branch"] > 0)[0][len(m["branch"]) // 2 % max(1, (m["branch"] > 0).sum())])
    bad["branch"][k] = -1
    off, out = oracle.search_batch(bad, g["q_starts"], g["q_ends"])
    assert not (np.array_equal(off, g["ref_search_idxs_off"]) and
                np.array_equal(out, g["ref_search_idxs"]))


@pytest.mark.parametrize("name", ["nested_dups_int32", "edges_int64", "config1_plain_small_int32"])
def test_oracle_upper_bound_batch(oracle, name):
    """upper_bound (hpp:501-516): the last start <= qe, -1 before the first start."""
    if name not in fixture_names():
        pytest.skip(f"no fixture {name}")
    g = load(name)
    m = oracle.build(g["starts"], g["ends"], g["data"])
    st = m["starts"]
    lim = np.iinfo(st.dtype)
    extra = list(st[:3]) + [v + 1 for v in st[-3:] if v < lim.max] + ([st[0] - 1] if st[0] > lim.min else [])
    qe = np.concatenate([g["q_ends"], np.array(extra, dtype=st.dtype)])
    got = oracle.upper_bound_batch(m, qe, nthreads=3)
    want = np.searchsorted(m["starts"], qe.astype(m["starts"].dtype), side="right") - 1
    assert np.array_equal(got, want)


SETOP_FIXTURES = fixture_names("setops_")


@pytest.mark.parametrize("name", SETOP_FIXTURES)
def test_oracle_setops_match_reference(oracle, name):
    """intersection / difference (hpp:1158-1211, c:921-974) of the reference's
    built A against B: pieces, their order and their data."""
    g = load(name)
    m = oracle.build(g["b_starts"], g["b_ends"], g["b_data"])
    a_s, a_e, a_d = g["ref_a_sorted_starts"], g["ref_a_sorted_ends"], g["ref_a_sorted_data"]
    off, os_, oe_, ob = oracle.intersection(m, a_s, a_e, ORDER_IDXS_CPP)
    assert np.array_equal(os_, g["ref_isect_starts"]) and np.array_equal(oe_, g["ref_isect_ends"])
    owner = np.repeat(np.arange(len(a_s)), np.diff(off))
    assert np.array_equal(a_d[owner], g["ref_isect_data"])
    # b's data names the B interval by insertion index: same coordinates as the hit
    bd = g["ref_isect_bdata_data"]
    assert np.array_equal(g["b_starts"][bd], m["starts"][ob]) and np.array_equal(g["b_ends"][bd], m["ends"][ob])
    off, os_, oe_ = oracle.difference(m, a_s, a_e)
    assert np.array_equal(os_, g["ref_diff_starts"]) and np.array_equal(oe_, g["ref_diff_ends"])
    owner = np.repeat(np.arange(len(a_s)), np.diff(off))
    assert np.array_equal(a_d[owner], g["ref_diff_data"])
    if "ref_c_isect_starts" in g:   # the C API: searchIdxs order (fully descending)
        _, os_, oe_, _ = oracle.intersection(m, a_s, a_e, ORDER_DESC)
        assert np.array_equal(os_, g["ref_c_isect_starts"]) and np.array_equal(oe_, g["ref_c_isect_ends"])
        assert np.array_equal(g["ref_c_diff_starts"], g["ref_diff_starts"])


@pytest.mark.parametrize("dt", [np.int32, np.int64])
def test_coverage_rank_identity(oracle, dt):
    """The identity behind the GPU's coverage from ranks (no interval and no query with
    start > end): over the hits {start <= qe} minus {end < qs},
      count = a_u - r_qs,
      sum min(end, qe) = PE[r_qe] - PE[r_qs] + qe (a_u - r_qe),
      sum max(start, qs) = PS[a_u] - PS[ls] + qs (ls - r_qs),
    with prefix sums mod 2^64 truncated to the coordinate width, equals the reference's
    per-hit wrapped sum (hpp:979-1006), coordinate extremes included."""
    r = np.random.default_rng(17)
    info = np.iinfo(dt)
    n = 3000
    s = np.concatenate([info.min + r.integers(0, 200_000, n // 2), info.max - r.integers(0, 200_000, n // 2)])
    ln = r.integers(0, 40_000, n)
    e = np.where(s > info.max - ln, info.max, s + ln)    # no overflow at the top of the type
    e[:20] = info.max
    m = oracle.build(s.astype(dt), e.astype(dt), np.arange(n, dtype=np.int32))
    st, en = m["starts"].astype(np.int64), m["ends"].astype(np.int64)
    q0 = np.concatenate([info.min + r.integers(0, 250_000, 300), info.max - r.integers(0, 250_000, 300)])
    qln = r.integers(0, 60_000, 600)
    q1 = np.where(q0 > info.max - qln, info.max, q0 + qln)
    q1[:10] = info.max
    qs, qe = q0.astype(dt), q1.astype(dt)
    assert (st <= en).all() and (qs <= qe).all()
    rc, rv = oracle.coverage(m, qs, qe)
    es = np.sort(en)
    u64 = lambda a: a.astype(np.int64).view(np.uint64)  # noqa: E731  (two's complement, mod 2^64)
    zero = np.zeros(1, np.uint64)
    ps = np.concatenate([zero, np.cumsum(u64(st), dtype=np.uint64)])
    pe = np.concatenate([zero, np.cumsum(u64(es), dtype=np.uint64)])
    a_u = np.searchsorted(st, qe.astype(np.int64), side="right")
    r_qs = np.searchsorted(es, qs.astype(np.int64), side="left")
    r_qe = np.searchsorted(es, qe.astype(np.int64), side="right")
    ls = np.searchsorted(st, qs.astype(np.int64), side="left")
    with np.errstate(over="ignore"):
        smin = pe[r_qe] - pe[r_qs] + u64(qe) * (a_u - r_qe).astype(np.uint64)
        smax = ps[a_u] - ps[ls] + u64(qs) * (ls - r_qs).astype(np.uint64)
        cov = (smin - smax).astype(np.uint64)
    bits = np.dtype(dt).itemsize * 8
    cov = (cov & np.uint64((1 << bits) - 1)) if bits < 64 else cov
    got = cov.astype(np.uint64).view(np.int64) if bits == 64 else cov.astype(np.uint32).view(np.int32)
    assert np.array_equal(a_u - r_qs, rc)
    assert np.array_equal(got.astype(dt), rv)
