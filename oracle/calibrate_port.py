"""Time the oracle port (oracle/si_oracle.c) against the reference's own header on the
same inputs, single-threaded: search_idxs (C++ order, superintervals.hpp:879-905) over a
query sample of configuration 3 at its full density (chr1's share of the 50 M intervals and
queries).  TEST INFRASTRUCTURE: it needs the reference checkout (oracle/_ref is built from
it by oracle/Makefile), so it runs only where those sources are present.  The port is the
CPU baseline wherever the reference cannot be compiled; this script states how its speed
compares with the reference's on one machine.

    python oracle/calibrate_port.py [--queries 100000] [--contig chr1]
"""
import argparse
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import oracle as O  # noqa: E402
from superintervals_gb300 import workloads as W  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--queries", type=int, default=100_000)
    ap.add_argument("--contig", default="chr1")
    ap.add_argument("--repeats", type=int, default=3)
    a = ap.parse_args()
    wl = W.config3_subset([a.contig])
    k = min(a.queries, wl.nq)
    qs, qe = np.ascontiguousarray(wl.q_starts[:k]), np.ascontiguousarray(wl.q_ends[:k])
    o = O.Oracle()
    m = o.build(wl.starts, wl.ends, wl.data)
    ref = O.Reference()
    L = ref.lib
    h = L.ref_map_i32_new(wl.n, O._ptr(wl.starts), O._ptr(wl.ends), O._ptr(wl.data))
    try:
        best_ref, best_port = 1e30, 1e30
        for _ in range(a.repeats):
            off_r = np.empty(k + 1, np.int64)
            tot = L.ref_map_i32_search(h, 0, k, O._ptr(qs), O._ptr(qe), O._ptr(off_r), None, 0)
            out_r = np.empty(max(tot, 1), np.int64)
            t0 = time.perf_counter()
            L.ref_map_i32_search(h, 0, k, O._ptr(qs), O._ptr(qe), O._ptr(off_r), O._ptr(out_r), tot)
            best_ref = min(best_ref, time.perf_counter() - t0)
            t0 = time.perf_counter()
            off_p, out_p = o.search_lists(m, qs, qe, order=O.ORDER_IDXS_CPP, nthreads=1)
            best_port = min(best_port, time.perf_counter() - t0)
        same = np.array_equal(off_p, off_r) and np.array_equal(out_p.astype(np.int64), out_r[:tot])
    finally:
        L.ref_map_i32_free(h)
    print(f"machine: {platform.machine()} {platform.processor() or ''}".strip())
    print(f"workload: configuration 3 at full density on {a.contig}: {wl.n} intervals; "
          f"first {k} of {wl.nq} queries; {tot} result pairs ({tot / k:.1f} per query)")
    print(f"reference header search_idxs, 1 thread: {k / best_ref:,.0f} queries/s ({best_ref:.3f} s)")
    print(f"oracle port search_idxs (one walk per query), 1 thread: {k / best_port:,.0f} queries/s ({best_port:.3f} s)")
    print(f"port / reference speed: {best_ref / best_port:.2f}; identical output: {same}")


if __name__ == "__main__":
    main()
