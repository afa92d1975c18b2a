"""ctypes front-end of the ORACLE (oracle/si_oracle.c) and of the reference shim.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline -- never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsi_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsi_ref.so")
# the reference checkout's src/ directory; SI_REF_SRC overrides the default location
REF_SRC_DEFAULT = os.environ.get("SI_REF_SRC", "/root/reference/src")

ORDER_IDXS_CPP = 0   # C++ search_idxs: ascending head run, then descending
ORDER_DESC = 1       # search_values / C-API searchIdxs: fully descending

_P = C.c_void_p
_I64 = C.c_int64


def build_oracle(quiet=True):
    """Compile the C restatement into oracle/_build (gcc, seconds)."""
    out = subprocess.run(["make", "-C", HERE, "_build/libsi_oracle.so"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


def build_ref(ref_src=REF_SRC_DEFAULT):
    """Compile the reference's own header into oracle/_ref when its sources
    are present (not on machines without the reference checkout)."""
    if not os.path.isfile(os.path.join(ref_src, "superintervals.hpp")):
        return False
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF_SRC={ref_src}"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference shim build failed:\n" + out.stdout + out.stderr)
    return True


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


class Oracle:
    """The C restatement, loaded from oracle/_build/libsi_oracle.so."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.isfile(path):
            build_oracle()
        self.lib = C.CDLL(path)
        self.lib.sio_lists_copy.restype = None
        self.lib.sio_lists_copy.argtypes = [_P, _P, _P, C.c_int]
        self.lib.sio_lists_free.restype = None
        self.lib.sio_lists_free.argtypes = [_P]
        for sfx in ("i32", "i64"):
            f = getattr(self.lib, f"sio_build_{sfx}")
            f.restype = C.c_int
            f.argtypes = [_I64] + [_P] * 8
            f = getattr(self.lib, f"sio_build_segments_{sfx}")
            f.restype = None
            f.argtypes = [_I64] + [_P] * 9
            f = getattr(self.lib, f"sio_count_batch_{sfx}")
            f.restype = None
            f.argtypes = [_P, _P, _P, _P, _I64, _P, _P, _P, _P, C.c_int]
            f = getattr(self.lib, f"sio_search_batch_{sfx}")
            f.restype = None
            f.argtypes = [_P, _P, _P, _P, _P, _I64, _P, _P, _P, C.c_int, _P, _P, C.c_int]
            f = getattr(self.lib, f"sio_search_lists_{sfx}")
            f.restype = _P
            f.argtypes = [_P, _P, _P, _P, _P, _I64, _P, _P, _P, C.c_int, _P, C.c_int]
            f = getattr(self.lib, f"sio_intersection_{sfx}")
            f.restype = _I64
            f.argtypes = [_I64, _P, _P, _P, _I64, _P, _P, C.c_int, _P, _P, _P, _P, _I64]
            f = getattr(self.lib, f"sio_difference_{sfx}")
            f.restype = _I64
            f.argtypes = [_I64, _P, _P, _P, _I64, _P, _P, _P, _P, _P, _I64]
            f = getattr(self.lib, f"sio_upper_bound_batch_{sfx}")
            f.restype = None
            f.argtypes = [_P, _P, _I64, _P, _P, _P, C.c_int]
            f = getattr(self.lib, f"sio_coverage_{sfx}")
            f.restype = None
            f.argtypes = [_I64, _P, _P, _P, C.c_int64 if sfx == "i64" else C.c_int32,
                          C.c_int64 if sfx == "i64" else C.c_int32, _P, _P]

    @staticmethod
    def _sfx(dtype):
        return "i64" if np.dtype(dtype) == np.int64 else "i32"

    def build(self, starts, ends, data=None, seg=None):
        """Per-contig build.  Returns dict(starts, ends, data, perm, branch) with
        contig-local branch indices (-1 = none)."""
        starts = np.ascontiguousarray(starts)
        ends = np.ascontiguousarray(ends, dtype=starts.dtype)
        n = starts.shape[0]
        if data is None:
            data = np.arange(n, dtype=np.int32)
        data = np.ascontiguousarray(data, dtype=np.int32)
        if seg is None:
            seg = np.array([0, n], dtype=np.int64)
        seg = np.ascontiguousarray(seg, dtype=np.int64)
        so, eo = np.empty_like(starts), np.empty_like(ends)
        do = np.empty(n, dtype=np.int32)
        perm = np.empty(n, dtype=np.int64)
        br = np.empty(n, dtype=np.int64)
        getattr(self.lib, f"sio_build_segments_{self._sfx(starts.dtype)}")(
            seg.shape[0] - 1, _ptr(seg), _ptr(starts), _ptr(ends), _ptr(data),
            _ptr(so), _ptr(eo), _ptr(do), _ptr(perm), _ptr(br))
        return dict(starts=so, ends=eo, data=do, perm=perm, branch=br, seg=seg)

    def count_batch(self, m, qs, qe, qc=None, nthreads=1):
        qs = np.ascontiguousarray(qs, dtype=m["starts"].dtype)
        qe = np.ascontiguousarray(qe, dtype=m["starts"].dtype)
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.int32)
        out = np.empty(qs.shape[0], dtype=np.uint32)
        getattr(self.lib, f"sio_count_batch_{self._sfx(qs.dtype)}")(
            _ptr(m["seg"]), _ptr(m["starts"]), _ptr(m["ends"]), _ptr(m["branch"]),
            qs.shape[0], _ptr(qc), _ptr(qs), _ptr(qe), _ptr(out), nthreads)
        return out

    def search_batch(self, m, qs, qe, qc=None, order=ORDER_IDXS_CPP, values=False,
                     nthreads=1, counts=None):
        """CSR result (offsets int64[nq+1], out int32[P]).  ``values`` gathers
        the payload instead of the contig-local position."""
        qs = np.ascontiguousarray(qs, dtype=m["starts"].dtype)
        qe = np.ascontiguousarray(qe, dtype=m["starts"].dtype)
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.int32)
        if counts is None:
            counts = self.count_batch(m, qs, qe, qc, nthreads)
        off = np.zeros(qs.shape[0] + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        out = np.empty(int(off[-1]), dtype=np.int32)
        getattr(self.lib, f"sio_search_batch_{self._sfx(qs.dtype)}")(
            _ptr(m["seg"]), _ptr(m["starts"]), _ptr(m["ends"]), _ptr(m["branch"]),
            _ptr(m["data"]) if values else None, qs.shape[0], _ptr(qc), _ptr(qs), _ptr(qe),
            order, _ptr(off), _ptr(out), nthreads)
        return off, out

    def search_lists(self, m, qs, qe, qc=None, order=ORDER_IDXS_CPP, values=False, nthreads=1):
        """Same result as search_batch, in one walk per query: each thread appends its
        queries' hits to a growable buffer (as the reference's search_idxs appends to a
        vector, hpp:879-905), then the buffers are copied into the CSR arrays.  This is the
        form the CPU baseline times."""
        qs = np.ascontiguousarray(qs, dtype=m["starts"].dtype)
        qe = np.ascontiguousarray(qe, dtype=m["starts"].dtype)
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.int32)
        nq = qs.shape[0]
        counts = np.empty(nq, dtype=np.uint32)
        h = getattr(self.lib, f"sio_search_lists_{self._sfx(qs.dtype)}")(
            _ptr(m["seg"]), _ptr(m["starts"]), _ptr(m["ends"]), _ptr(m["branch"]),
            _ptr(m["data"]) if values else None, nq, _ptr(qc), _ptr(qs), _ptr(qe), order,
            _ptr(counts), nthreads)
        if not h:
            raise MemoryError("oracle list search: host allocation failed")
        try:
            off = np.zeros(nq + 1, dtype=np.int64)
            np.cumsum(counts, out=off[1:])
            out = np.empty(int(off[-1]), dtype=np.int32)
            self.lib.sio_lists_copy(h, _ptr(off), _ptr(out), nthreads)
        finally:
            self.lib.sio_lists_free(h)
        return off, out

    def intersection(self, m, a_s, a_e, order=ORDER_IDXS_CPP):
        """intersection (hpp:1158-1177): CSR over the A intervals of pieces
        (start, end, b position), single-contig map m."""
        st = m["starts"]
        a_s = np.ascontiguousarray(a_s, dtype=st.dtype)
        a_e = np.ascontiguousarray(a_e, dtype=st.dtype)
        f = getattr(self.lib, f"sio_intersection_{self._sfx(st.dtype)}")
        off = np.zeros(a_s.shape[0] + 1, np.int64)
        args = (st.shape[0], _ptr(st), _ptr(m["ends"]), _ptr(m["branch"]), a_s.shape[0], _ptr(a_s), _ptr(a_e),
                order, _ptr(off))
        tot = f(*args, None, None, None, 0)
        os_, oe_, ob = np.empty(tot, st.dtype), np.empty(tot, st.dtype), np.empty(tot, np.int64)
        f(*args, _ptr(os_), _ptr(oe_), _ptr(ob), tot)
        return off, os_, oe_, ob

    def difference(self, m, a_s, a_e):
        """difference (hpp:1186-1211): CSR over the A intervals of uncovered
        pieces (start, end), single-contig map m."""
        st = m["starts"]
        a_s = np.ascontiguousarray(a_s, dtype=st.dtype)
        a_e = np.ascontiguousarray(a_e, dtype=st.dtype)
        f = getattr(self.lib, f"sio_difference_{self._sfx(st.dtype)}")
        off = np.zeros(a_s.shape[0] + 1, np.int64)
        args = (st.shape[0], _ptr(st), _ptr(m["ends"]), _ptr(m["branch"]), a_s.shape[0], _ptr(a_s), _ptr(a_e),
                _ptr(off))
        tot = f(*args, None, None, 0)
        os_, oe_ = np.empty(tot, st.dtype), np.empty(tot, st.dtype)
        f(*args, _ptr(os_), _ptr(oe_), tot)
        return off, os_, oe_

    def upper_bound_batch(self, m, qe, qc=None, nthreads=1):
        """upper_bound (hpp:501-516) of every query end within its contig's map:
        contig-local index of the last start <= qe, or -1."""
        qe = np.ascontiguousarray(qe, dtype=m["starts"].dtype)
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.int32)
        out = np.empty(qe.shape[0], dtype=np.int64)
        getattr(self.lib, f"sio_upper_bound_batch_{self._sfx(qe.dtype)}")(
            _ptr(m["seg"]), _ptr(m["starts"]), qe.shape[0], _ptr(qc), _ptr(qe), _ptr(out), nthreads)
        return out

    def has_overlaps_batch(self, m, qs, qe):
        """has_overlaps (hpp:865-871): true iff the interval at upper_bound(qe)
        reaches qs -- it looks at that one interval only, so it can be false
        while count() > 0 (a longer interval further back)."""
        st, en = m["starts"], m["ends"]
        ub = np.searchsorted(st, np.asarray(qe, st.dtype), side="right") - 1
        ok = ub >= 0
        res = np.zeros(len(qs), dtype=np.int32)
        res[ok] = (np.asarray(qs, st.dtype)[ok] <= en[ub[ok]]).astype(np.int32)
        return res

    def coverage(self, m, qs, qe):
        """Single-contig coverage (hpp:979-1006) per query: (count, covered)."""
        sfx = self._sfx(m["starts"].dtype)
        cnt = np.empty(len(qs), dtype=np.int64)
        cov = np.empty(len(qs), dtype=m["starts"].dtype)
        f = getattr(self.lib, f"sio_coverage_{sfx}")
        n = m["starts"].shape[0]
        c1 = C.c_int64(0)
        v1 = (C.c_int64 if sfx == "i64" else C.c_int32)(0)
        for k in range(len(qs)):
            f(n, _ptr(m["starts"]), _ptr(m["ends"]), _ptr(m["branch"]), int(qs[k]), int(qe[k]),
              C.byref(c1), C.byref(v1))
            cnt[k] = c1.value
            cov[k] = v1.value
        return cnt, cov


class Reference:
    """The reference's own header and C API, compiled into oracle/_ref (only
    where the reference checkout is present)."""

    def __init__(self, path=REF_SO):
        if not os.path.isfile(path):
            if not build_ref():
                raise FileNotFoundError("reference sources not available")
        self.lib = C.CDLL(path)
        for sfx in ("i32", "i64"):
            getattr(self.lib, f"ref_map_{sfx}_new").restype = _P
            getattr(self.lib, f"ref_map_{sfx}_new").argtypes = [_I64, _P, _P, _P]
            getattr(self.lib, f"ref_map_{sfx}_free").argtypes = [_P]
            getattr(self.lib, f"ref_map_{sfx}_size").restype = _I64
            getattr(self.lib, f"ref_map_{sfx}_size").argtypes = [_P]
            getattr(self.lib, f"ref_map_{sfx}_arrays").argtypes = [_P] * 5
            getattr(self.lib, f"ref_map_{sfx}_scalar").argtypes = [_P, C.c_int, _I64, _P, _P, _P]
            getattr(self.lib, f"ref_map_{sfx}_search").restype = _I64
            getattr(self.lib, f"ref_map_{sfx}_search").argtypes = [_P, C.c_int, _I64, _P, _P, _P, _P, _I64]
            getattr(self.lib, f"ref_map_{sfx}_coverage").argtypes = [_P, _I64, _P, _P, _P, _P]
            getattr(self.lib, f"ref_map_{sfx}_setop").restype = _I64
            getattr(self.lib, f"ref_map_{sfx}_setop").argtypes = [_P, _P, C.c_int, _P, _P, _P, _I64]
        self.lib.ref_c_setop.restype = _I64
        self.lib.ref_c_setop.argtypes = [_P, _P, C.c_int, _P, _P, _P, _I64]
        self.lib.ref_c_new.restype = _P
        self.lib.ref_c_new.argtypes = [_I64, _P, _P, _P]
        self.lib.ref_c_free.argtypes = [_P]
        self.lib.ref_c_arrays.argtypes = [_P] * 5
        self.lib.ref_c_search.restype = _I64
        self.lib.ref_c_search.argtypes = [_P, C.c_int, _I64, _P, _P, _P, _P, _I64]

    @staticmethod
    def _sfx(dtype):
        return "i64" if np.dtype(dtype) == np.int64 else "i32"

    def setops(self, a, b):
        """a.intersection(b) (keeping a's and, separately, b's data) and
        a.difference(b) through the reference's C++ class, and intersection /
        difference through its C API (int32 only).  a and b are (starts, ends,
        data) triples; A's arrays after its build() (the order the reference
        iterates) are returned too."""
        L = self.lib
        dt = np.asarray(a[0]).dtype
        sfx = self._sfx(dt)
        arr = [tuple(np.ascontiguousarray(x, dtype=t) for x, t in zip(m, (dt, dt, np.int32))) for m in (a, b)]
        res = {}
        hs = [getattr(L, f"ref_map_{sfx}_new")(m[0].shape[0], _ptr(m[0]), _ptr(m[1]), _ptr(m[2])) for m in arr]
        try:
            na = arr[0][0].shape[0]
            so, eo, do = np.empty(na, dt), np.empty(na, dt), np.empty(na, np.int32)
            if na:
                getattr(L, f"ref_map_{sfx}_arrays")(hs[0], _ptr(so), _ptr(eo), _ptr(do), None)
            res.update(a_sorted_starts=so, a_sorted_ends=eo, a_sorted_data=do)
            for op, key in ((0, "isect"), (1, "isect_bdata"), (2, "diff")):
                f = getattr(L, f"ref_map_{sfx}_setop")
                k = f(hs[0], hs[1], op, None, None, None, 0)
                os_, oe_, od = np.empty(k, dt), np.empty(k, dt), np.empty(k, np.int32)
                f(hs[0], hs[1], op, _ptr(os_), _ptr(oe_), _ptr(od), k)
                res.update({key + "_starts": os_, key + "_ends": oe_, key + "_data": od})
        finally:
            for h in hs:
                getattr(L, f"ref_map_{sfx}_free")(h)
        if sfx == "i32":
            hc = [L.ref_c_new(m[0].shape[0], _ptr(m[0]), _ptr(m[1]), _ptr(m[2])) for m in arr]
            try:
                for op, key in ((0, "c_isect"), (2, "c_diff")):
                    k = L.ref_c_setop(hc[0], hc[1], op, None, None, None, 0)
                    os_, oe_, od = np.empty(k, dt), np.empty(k, dt), np.empty(k, np.int32)
                    L.ref_c_setop(hc[0], hc[1], op, _ptr(os_), _ptr(oe_), _ptr(od), k)
                    res.update({key + "_starts": os_, key + "_ends": oe_, key + "_data": od})
            finally:
                for h in hc:
                    L.ref_c_free(h)
        return res

    def run(self, starts, ends, data, qs, qe):
        """Everything the fixtures need for one single-contig case."""
        starts = np.ascontiguousarray(starts)
        ends = np.ascontiguousarray(ends, dtype=starts.dtype)
        data = np.ascontiguousarray(data, dtype=np.int32)
        qs = np.ascontiguousarray(qs, dtype=starts.dtype)
        qe = np.ascontiguousarray(qe, dtype=starts.dtype)
        sfx = self._sfx(starts.dtype)
        L = self.lib
        n, nq = starts.shape[0], qs.shape[0]
        h = getattr(L, f"ref_map_{sfx}_new")(n, _ptr(starts), _ptr(ends), _ptr(data))
        res = {}
        try:
            so, eo = np.empty_like(starts), np.empty_like(ends)
            do, br = np.empty(n, np.int32), np.empty(n, np.int64)
            if n:
                getattr(L, f"ref_map_{sfx}_arrays")(h, _ptr(so), _ptr(eo), _ptr(do), _ptr(br))
            res.update(sorted_starts=so, sorted_ends=eo, sorted_data=do, branch=br)
            for mode, key in ((0, "count"), (1, "count_linear"), (2, "count_large"),
                              (3, "has_overlaps")):
                o = np.empty(nq, np.int64)
                getattr(L, f"ref_map_{sfx}_scalar")(h, mode, nq, _ptr(qs), _ptr(qe), _ptr(o))
                res[key] = o
            for mode, key in ((0, "search_idxs"), (1, "search_values"),
                              (2, "search_values_large")):
                off = np.empty(nq + 1, np.int64)
                tot = getattr(L, f"ref_map_{sfx}_search")(h, mode, nq, _ptr(qs), _ptr(qe),
                                                           _ptr(off), None, 0)
                out = np.empty(max(tot, 1), np.int64)
                getattr(L, f"ref_map_{sfx}_search")(h, mode, nq, _ptr(qs), _ptr(qe),
                                                     _ptr(off), _ptr(out), tot)
                res[key + "_off"] = off
                res[key] = out[:tot]
            cnt = np.empty(nq, np.int64)
            cov = np.empty(nq, starts.dtype)
            getattr(L, f"ref_map_{sfx}_coverage")(h, nq, _ptr(qs), _ptr(qe), _ptr(cnt), _ptr(cov))
            res["coverage_count"] = cnt
            res["coverage"] = cov
        finally:
            getattr(L, f"ref_map_{sfx}_free")(h)
        if sfx == "i32":
            hc = L.ref_c_new(n, _ptr(starts), _ptr(ends), _ptr(data))
            try:
                so, eo = np.empty_like(starts), np.empty_like(ends)
                do, br = np.empty(n, np.int32), np.empty(n, np.int64)
                if n:
                    L.ref_c_arrays(hc, _ptr(so), _ptr(eo), _ptr(do), _ptr(br))
                res.update(c_sorted_starts=so, c_sorted_ends=eo, c_sorted_data=do, c_branch=br)
                for mode, key in ((0, "c_search_idxs"), (1, "c_search_values"),
                                  (2, "c_count")):
                    off = np.empty(nq + 1, np.int64)
                    tot = L.ref_c_search(hc, mode, nq, _ptr(qs), _ptr(qe), _ptr(off), None, 0)
                    out = np.empty(max(tot, 1), np.int64)
                    L.ref_c_search(hc, mode, nq, _ptr(qs), _ptr(qe), _ptr(off), _ptr(out), tot)
                    res[key + "_off"] = off
                    if mode != 2:
                        res[key] = out[:tot]
            finally:
                L.ref_c_free(hc)
        return res
