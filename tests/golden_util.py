"""Helpers shared by the parity tests: fixture loading and the parity rules."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fixture_names(prefix=""):
    """Single-map query fixtures (prefix "setops_" selects the set-operation ones)."""
    names = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, prefix + "*.npz"))
                   if not os.path.basename(p).startswith("contigs3_stream"))
    return names if prefix.startswith("setops") else [n for n in names if not n.startswith("setops_")]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def csr_lists(off, out):
    return [out[off[i]:off[i + 1]].tolist() for i in range(len(off) - 1)]


def duplicate_runs(starts, ends):
    """[lo, hi) runs of identical (start, end) in sorted order."""
    n = len(starts)
    if n == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    brk = np.ones(n, dtype=bool)
    brk[1:] = (starts[1:] != starts[:-1]) | (ends[1:] != ends[:-1])
    lo = np.nonzero(brk)[0]
    hi = np.append(lo[1:], n)
    return lo, hi


def assert_data_parity(starts, ends, data_ref, data_new):
    """Payload parity: the reference sorts with std::sort (unstable,
    src/superintervals.hpp:1403), so inside runs of exact (start, end)
    duplicates only the multiset of payloads is defined.  Outside those
    runs the payload must be identical."""
    lo, hi = duplicate_runs(starts, ends)
    single = (hi - lo) == 1
    assert np.array_equal(data_ref[lo[single]], data_new[lo[single]])
    for a, b in zip(lo[~single], hi[~single]):
        assert sorted(data_ref[a:b].tolist()) == sorted(data_new[a:b].tolist())


def assert_values_parity(pos_desc, off, data_ref, data_new, vals_ref, vals_new):
    """search_values parity: each side's values must be its own payload
    gathered at the (bit-identical) descending hit positions."""
    assert np.array_equal(vals_ref, data_ref[pos_desc])
    assert np.array_equal(vals_new, data_new[pos_desc])
