"""Generate the golden fixtures in tests/golden/ from the REFERENCE ITSELF.

Run in a checkout that has the reference sources (default /root/reference/src):

    python tests/golden/make_golden.py [--ref-src DIR]

It compiles oracle/ref_shim.cpp + oracle/ref_shim_c.c against the unmodified
reference headers (src/superintervals.hpp, src/c_superintervals.h) into
oracle/_ref/libsi_ref.so, runs every case below through the reference's
si::IntervalMap<S,int32_t> (build, count, count_linear, count_large,
has_overlaps, search_idxs, search_values, search_values_large, coverage) and
through its C API (indexSuperIntervals, searchIdxs, searchValues,
countOverlaps), and stores inputs and outputs as compressed .npz files.

The known-answer cases restate the inputs of the reference's unit tests
(test/tests.cpp:63-238) and of its Python README batch example
(src/superintervals/README.md:24-27); the expected answers those tests assert
are re-checked in tests/test_golden_oracle.py.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from superintervals_gb300 import workloads as W  # noqa: E402


def kat_cases():
    """(name, refs[(s,e,d)], queries[(qs,qe)]) restated from test/tests.cpp."""
    cases = []
    cases.append(("kat_basics",  # tests.cpp:63-107
                  [(10, 20, 0), (11, 12, -1), (13, 14, -1), (15, 16, -1), (25, 29, 4)],
                  [(17, 30), (1, 3), (10, 29), (0, 1)]))
    nested = [(0, 250000, 0)] + [(s, s + 1000, -1) for s in
                                  (55, 115, 130, 281, 639, 842, 999, 1094, 1157, 1161,
                                   1265, 1532, 1590, 1665, 1945, 2384, 2515)]
    cases.append(("kat_nested", nested, [(1377, 2377)]))  # tests.cpp:146-157
    cases.append(("kat_shared_endpoints",  # tests.cpp:161-171
                  [(3, 40, 0), (4, 5, 4), (6, 7, 4), (10, 31, 5), (31, 32, 5)],
                  [(31, 32), (10, 11), (4, 7)]))
    cases.append(("kat_duplicates",  # tests.cpp:174-186
                  [(3, 40, 0), (3, 40, 4), (3, 40, 4), (3, 4, 4), (35, 50, 4), (40, 400, 5),
                   (40, 400, 4)],
                  [(38, 41), (41, 42)]))
    cases.append(("kat_coverage",  # tests.cpp:194-213
                  [(1, 100, 0), (30, 200, 7), (40, 50, 6), (60, 70, 7)], [(55, 65)]))
    cases.append(("kat_empty", [], [(1, 5)]))  # tests.cpp:222-228
    cases.append(("kat_single", [(1, 10, 1)], [(1, 5), (11, 20), (5, 11)]))  # tests.cpp:229-236
    cases.append(("kat_readme_batch",  # src/superintervals/README.md:16-27
                  [(10, 20, 0), (15, 25, 1), (30, 40, 2)], [(5, 12), (18, 22), (35, 45), (8, 20)]))
    return cases


def edge_case(dtype):
    """Edges the reference semantics define: qs > qe, queries before the first
    start and after the last end, negative coordinates, type extremes."""
    info = np.iinfo(dtype)
    refs = [(-50, -10, 0), (-20, 5, 1), (0, 0, 2), (0, 0, 3), (7, 7, 4), (5, 100, 5),
            (100, 100, 6), (info.max - 10, info.max, 7), (info.min, info.min + 5, 8),
            (60, 40, 9)]  # the last one has end < start: accepted by the reference
    qs = [(-100, -60), (-60, -50), (0, 0), (1, 6), (6, 1), (100, 100), (101, 200),
          (info.max, info.max), (info.min, info.min), (info.min, info.max), (45, 45),
          (-10, -10), (7, 6)]
    return refs, qs


def sorted_inputs(seed, n, dtype):
    wl = W.random_nested(seed, n, n, dtype=dtype, span=50_000, max_len=400)
    o = np.lexsort((-wl.ends.astype(np.int64), wl.starts))
    return wl.starts[o], wl.ends[o], wl.q_starts, wl.q_ends


def start_sorted_end_unsorted(seed, n, dtype):
    wl = W.random_nested(seed, n, n, dtype=dtype, span=50_000, max_len=400, dup_frac=0.3)
    o = np.argsort(wl.starts, kind="stable")
    return wl.starts[o], wl.ends[o], wl.q_starts, wl.q_ends


def save_case(ref, name, starts, ends, data, qs, qe, extra=None):
    starts = np.asarray(starts)
    res = ref.run(starts, ends, data, qs, qe)
    payload = dict(starts=starts, ends=np.asarray(ends, dtype=starts.dtype),
                   data=np.asarray(data, np.int32), q_starts=np.asarray(qs, starts.dtype),
                   q_ends=np.asarray(qe, starts.dtype))
    # count_linear / count_large and search_values_large must agree with
    # count / search_values; they are checked here and not stored twice.
    for k, base in (("count_linear", "count"), ("count_large", "count"),
                    ("search_values_large", "search_values")):
        assert np.array_equal(res.pop(k), res[base]), f"{name}: {k} != {base}"
    res.pop("search_values_large_off")
    # the C API builds the same sorted coordinates and branch array (its
    # payload order may differ: qsort vs std::sort); store them once.
    for k in ("sorted_starts", "sorted_ends", "branch"):
        if "c_" + k in res:
            assert np.array_equal(res.pop("c_" + k), res[k]), f"{name}: C API {k} differs"
    res["branch"] = res["branch"].astype(np.int32)
    for k, v in res.items():
        if v.dtype == np.int64 and not k.endswith("_off") and k not in ("branch", "c_branch") \
                and not k.startswith("sorted_") and not k.startswith("c_sorted_") \
                and k != "coverage":
            v = v.astype(np.int32)
        payload["ref_" + k] = v
    if extra:
        payload.update(extra)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **payload)
    print(f"{name}: n={starts.shape[0]} q={len(qs)} P={int(res['search_idxs_off'][-1])} "
          f"{os.path.getsize(path) / 1024:.0f} KiB")


def setop_cases():
    """(name, A triples, B triples) for intersection / difference."""
    cases = [
        ("setops_small", [(1, 10, 0), (5, 20, 1), (30, 40, 2), (50, 55, 3)],
         [(3, 4, 0), (8, 12, 1), (15, 35, 2), (52, 53, 3)]),
        # touching, not overlapping; a cover that reaches past A on both sides; duplicates
        ("setops_touching", [(5, 35, 0), (10, 19, 1), (40, 60, 2), (40, 60, 3)],
         [(10, 19, 0), (20, 29, 1), (0, 100, 2), (45, 45, 3), (45, 45, 4), (61, 70, 5)]),
        ("setops_emptyb", [(1, 5, 0), (7, 9, 1)], []),
        ("setops_emptya", [], [(1, 5, 0)]),
    ]
    return cases


def random_setop(seed, na, nb, dt, span=60_000, max_len=1_500, inverted=0.0):
    r = np.random.Generator(np.random.PCG64(seed))

    def draw(n):
        s = r.integers(0, span, n)
        ln = np.minimum(np.rint(np.exp(r.normal(np.log(200), 1.2, n))), max_len).astype(np.int64)
        k = np.nonzero(r.random(n - 1) < 0.05)[0] + 1  # exact duplicates of the previous interval
        s[k], ln[k] = s[k - 1], ln[k - 1]
        k = np.nonzero(r.random(n - 1) < 0.05)[0] + 1  # shared start, own length
        s[k] = s[k - 1]
        e = s + ln - 1
        inv = r.random(n) < inverted                  # start > end
        s[inv], e[inv] = e[inv] + 3, s[inv]
        return s.astype(dt), e.astype(dt), np.arange(n, dtype=np.int32)
    return draw(na), draw(nb)


def save_setop(ref, name, a, b):
    res = ref.setops(a, b)
    payload = dict(a_starts=np.asarray(a[0]), a_ends=np.asarray(a[1]), a_data=np.asarray(a[2], np.int32),
                   b_starts=np.asarray(b[0]), b_ends=np.asarray(b[1]), b_data=np.asarray(b[2], np.int32))
    payload.update({"ref_" + k: v for k, v in res.items()})
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **payload)
    print(f"{name}: |A|={len(a[0])} |B|={len(b[0])} isect={len(res['isect_starts'])} "
          f"diff={len(res['diff_starts'])} {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=O.REF_SRC_DEFAULT)
    a = ap.parse_args()
    if not O.build_ref(a.ref_src):
        sys.exit(f"reference sources not found under {a.ref_src}")
    ref = O.Reference()

    for name, refs, qs in kat_cases():
        for dt in (np.int32, np.int64):
            s = np.array([r[0] for r in refs], dtype=dt)
            e = np.array([r[1] for r in refs], dtype=dt)
            d = np.array([r[2] for r in refs], dtype=np.int32)
            save_case(ref, f"{name}_{np.dtype(dt).name}", s, e, d,
                      [q[0] for q in qs], [q[1] for q in qs])

    for dt in (np.int32, np.int64):
        refs, qs = edge_case(dt)
        save_case(ref, f"edges_{np.dtype(dt).name}",
                  np.array([r[0] for r in refs], dtype=dt), np.array([r[1] for r in refs], dtype=dt),
                  np.array([r[2] for r in refs], dtype=np.int32),
                  [q[0] for q in qs], [q[1] for q in qs])

    wl = W.config1()
    save_case(ref, "config1_plain_small_int32", wl.starts, wl.ends, wl.data, wl.q_starts, wl.q_ends)

    for seed, dt in ((11, np.int32), (12, np.int64)):
        wl = W.random_nested(seed, 4000, 4000, dtype=dt, span=200_000, max_len=2_000)
        save_case(ref, f"nested_dups_{np.dtype(dt).name}", wl.starts, wl.ends, wl.data,
                  wl.q_starts, wl.q_ends)

    for seed, dt in ((13, np.int32), (14, np.int64)):
        s, e, qs, qe = sorted_inputs(seed, 3000, dt)
        save_case(ref, f"presorted_{np.dtype(dt).name}", s, e, np.arange(len(s), dtype=np.int32),
                  qs, qe)
        s, e, qs, qe = start_sorted_end_unsorted(seed + 10, 3000, dt)
        save_case(ref, f"start_sorted_end_unsorted_{np.dtype(dt).name}", s, e,
                  np.arange(len(s), dtype=np.int32), qs, qe)

    # multi-contig: three independent per-contig maps (the reference's usage
    # pattern, one IntervalMap per contig); stored as three cases plus a
    # combined query stream, checked contig by contig.
    wl = W.config3(n=30_000, nq=30_000, contigs=W.HUMAN_CONTIGS[20:23])
    for g in range(3):
        lo, hi = int(wl.seg[g]), int(wl.seg[g + 1])
        sel = wl.q_contig == g
        save_case(ref, f"contigs3_g{g}_int32", wl.starts[lo:hi], wl.ends[lo:hi],
                  wl.data[lo:hi], wl.q_starts[sel], wl.q_ends[sel],
                  extra=dict(q_index=np.nonzero(sel)[0].astype(np.int64)))
    # set operations: intersection / difference of map A against map B
    for name, a, b in setop_cases():
        for dt in (np.int32, np.int64):
            tr = [tuple(np.array([t[i] for t in m], dtype=(dt if i < 2 else np.int32)) for i in range(3))
                  for m in (a, b)]
            save_setop(ref, f"{name}_{np.dtype(dt).name}", tr[0], tr[1])
    for seed, dt in ((21, np.int32), (22, np.int64)):
        a, b = random_setop(seed, 1500, 3000, dt)                       # dense: B covers ~20x
        save_setop(ref, f"setops_random_{np.dtype(dt).name}", a, b)
        a, b = random_setop(seed + 10, 1500, 3000, dt, span=1_500_000)  # sparse: many gaps
        save_setop(ref, f"setops_sparse_{np.dtype(dt).name}", a, b)
    # B (and A) holding some start > end intervals: the sweep order inside equal-start runs matters
    a, b = random_setop(23, 800, 2000, np.int32, span=300_000, inverted=0.03)
    save_setop(ref, "setops_inverted_int32", a, b)

    np.savez_compressed(os.path.join(HERE, "contigs3_stream_int32.npz"), starts=wl.starts,
                        ends=wl.ends, data=wl.data, seg=wl.seg, q_starts=wl.q_starts,
                        q_ends=wl.q_ends, q_contig=wl.q_contig)


if __name__ == "__main__":
    main()
