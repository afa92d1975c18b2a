"""Python host side over the C-ABI.

* ``GpuIndex`` -- a device-resident set of per-contig interval maps with numpy
  batch queries in CSR form (the GPU-native surface).
* ``IntervalMap`` -- a drop-in mirror of the reference's Python class
  (src/superintervals/intervalmap.pyx:17-819, query/batch part): the same
  method names, argument meaning and errors, answered by the GPU.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import _capi
from ._capi import (ORDER_DESC, ORDER_IDXS_CPP, PATH_AUTO, PATH_BATCHED, PATH_PLAIN, UB_BINARY,
                    UB_EYTZINGER, UB_LEARNED, SIError, check)

__all__ = ["GpuIndex", "IntervalMap", "SIError", "ORDER_IDXS_CPP", "ORDER_DESC", "PATH_AUTO",
           "PATH_PLAIN", "PATH_BATCHED", "UB_BINARY", "UB_EYTZINGER", "UB_LEARNED"]


def _p(a: Optional[np.ndarray]):
    return None if a is None else C.c_void_p(a.ctypes.data)


class GpuIndex:
    """A set of per-contig interval maps resident on one GPU.

    ``coord_bits`` is 32 or 64 (the reference's S = int / int64_t).  Contig
    ``g`` holds the intervals ``[seg[g], seg[g+1])`` of the arrays passed to
    :meth:`add_arrays`; results carry contig-local positions, exactly as one
    reference IntervalMap per contig would return them.
    """

    def __init__(self, coord_bits: int = 32, device: int = 0):
        self.lib = _capi.load()
        self.bits = coord_bits
        self.dtype = np.dtype(np.int64 if coord_bits == 64 else np.int32)
        h = C.c_void_p()
        check(self.lib.createSuperIntervalsGpu(C.byref(h), coord_bits, device))
        self.h = h
        self._sfx = "_i64" if coord_bits == 64 else ""

    def close(self):
        if getattr(self, "h", None):
            self.lib.destroySuperIntervalsGpu(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- staging / build -----------------------------------------------------
    def _coords(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def add(self, start: int, end: int, value: int):
        f = self.lib.addIntervalGpu_i64 if self.bits == 64 else self.lib.addIntervalGpu
        check(f(self.h, int(start), int(end), int(value)))

    def add_arrays(self, starts, ends, values=None, seg=None):
        s, e = self._coords(starts), self._coords(ends)
        if s.shape != e.shape:
            raise ValueError("starts and ends must have the same length")
        v = None if values is None else np.ascontiguousarray(values, dtype=np.int32)
        if v is not None and v.shape != s.shape:
            raise ValueError("values length must match starts/ends length")
        f = getattr(self.lib, "addIntervalsGpu" + self._sfx)
        check(f(self.h, _p(s), _p(e), _p(v), s.shape[0]))
        if seg is not None:
            seg = np.ascontiguousarray(seg, dtype=np.int64)
            check(self.lib.setContigsGpu(self.h, seg.shape[0] - 1, _p(seg)))

    def set_contigs(self, seg):
        seg = np.ascontiguousarray(seg, dtype=np.int64)
        check(self.lib.setContigsGpu(self.h, seg.shape[0] - 1, _p(seg)))

    def build(self):
        check(self.lib.indexSuperIntervalsGpu(self.h))

    def clear(self):
        check(self.lib.clearSuperIntervalsGpu(self.h))

    def reserve(self, n: int):
        check(self.lib.reserveSuperIntervalsGpu(self.h, int(n)))

    def size(self) -> int:
        return int(self.lib.sizeSuperIntervalsGpu(self.h))

    def n_contigs(self) -> int:
        return int(self.lib.numContigsGpu(self.h))

    def arrays(self):
        """(starts, ends, data, branch) after build(); branch is contig-local, -1 = none."""
        n = self.size()
        s, e = np.empty(n, self.dtype), np.empty(n, self.dtype)
        d, b = np.empty(n, np.int32), np.empty(n, np.int64)
        check(self.lib.getIndexArraysGpu(self.h, _p(s), _p(e), _p(d), _p(b)))
        return s, e, d, b

    # -- BED ingest (examples/bed-intersect-si.rs:63-120), parsed on the GPU ---------
    @staticmethod
    def _stats(st):
        return {k: int(getattr(st, k)) for k, _ in _capi.cBedStats._fields_}

    def ingest_bed(self, text: bytes, half_open: bool = True) -> dict:
        """Stage the intervals of BED text (one contig per chrom, first-appearance
        order, payload = line number); call build() afterwards.  Returns line counts."""
        st = _capi.cBedStats()
        check(self.lib.ingestBedGpu(self.h, text, len(text), _capi.BED_HALF_OPEN if half_open else 0,
                                    C.byref(st)))
        return self._stats(st)

    def contig_names(self) -> list:
        out, n = [], C.c_size_t(0)
        for c in range(self.n_contigs()):
            if self.lib.contigNameGpu(self.h, c, None, 0, C.byref(n)) == _capi.SI_ERR_INVALID:
                return []
            buf = C.create_string_buffer(n.value + 1)
            check(self.lib.contigNameGpu(self.h, c, buf, n.value + 1, C.byref(n)))
            out.append(buf.value.decode("latin-1"))
        return out

    def bed_queries(self, text: bytes, half_open: bool = True):
        """Queries from BED text on this index's contigs: (qs, qe, qc, line, stats)."""
        st = _capi.cBedStats()
        n = C.c_size_t(0)
        flag = _capi.BED_HALF_OPEN if half_open else 0
        bufs = [np.empty(1, self.dtype), np.empty(1, self.dtype), np.empty(1, np.int32), np.empty(1, np.int64)]
        for cap in (0, None):
            if cap is None:
                cap = n.value
                bufs = [np.empty(cap, self.dtype), np.empty(cap, self.dtype), np.empty(cap, np.int32),
                        np.empty(cap, np.int64)]
            r = self.lib.bedQueriesGpu(self.h, text, len(text), flag, *[_p(b) for b in bufs], cap, C.byref(n),
                                       C.byref(st))
            if r == _capi.SI_ERR_CAPACITY:
                continue
            check(r)
            break
        k = n.value
        return bufs[0][:k], bufs[1][:k], bufs[2][:k], bufs[3][:k], self._stats(st)

    # -- index image (the Rust crate's serde counterpart, superintervals.rs:35-44) --
    def to_bytes(self) -> bytes:
        """The built index as one flat byte image."""
        size = C.c_size_t(0)
        self.lib.serializeIndexGpu(self.h, None, 0, C.byref(size))
        buf = C.create_string_buffer(max(size.value, 1))
        check(self.lib.serializeIndexGpu(self.h, buf, size.value, C.byref(size)))
        return buf.raw[: size.value]

    def from_bytes(self, image: bytes):
        """Replace this handle's intervals with an image's and index them (no sort)."""
        check(self.lib.deserializeIndexGpu(self.h, C.c_char_p(image), len(image)))

    def save(self, path: str):
        check(self.lib.saveIndexGpu(self.h, os.fsencode(path)))

    def load(self, path: str):
        check(self.lib.loadIndexGpu(self.h, os.fsencode(path)))

    # -- options ---------------------------------------------------------------
    def set_path(self, path: int):
        check(self.lib.setQueryPathGpu(self.h, int(path)))

    def set_upper_bound(self, mode: int):
        check(self.lib.setUpperBoundModeGpu(self.h, int(mode)))

    def set_output_budget(self, nbytes: int):
        check(self.lib.setOutputBudgetGpu(self.h, int(nbytes)))

    @property
    def stream(self):
        return self.lib.getStreamGpu(self.h)

    # -- queries (host buffers) ------------------------------------------------
    def _queries(self, qs, qe, qc):
        qs, qe = self._coords(qs), self._coords(qe)
        if qs.shape != qe.shape:
            raise ValueError("starts and ends must have the same length")
        qc = None if qc is None else np.ascontiguousarray(qc, dtype=np.int32)
        if qc is not None and qc.shape != qs.shape:
            raise ValueError("contig ids must match the query count")
        return qs, qe, qc

    def count(self, qs, qe, qc=None) -> np.ndarray:
        qs, qe, qc = self._queries(qs, qe, qc)
        out = np.empty(qs.shape[0], np.uint32)
        f = getattr(self.lib, "countOverlapsBatchGpu" + self._sfx)
        check(f(self.h, _p(qs), _p(qe), _p(qc), qs.shape[0], _p(out)))
        return out

    def has_overlaps(self, qs, qe, qc=None) -> np.ndarray:
        qs, qe, qc = self._queries(qs, qe, qc)
        out = np.empty(qs.shape[0], np.uint8)
        f = getattr(self.lib, "anyOverlapsBatchGpu" + self._sfx)
        check(f(self.h, _p(qs), _p(qe), _p(qc), qs.shape[0], _p(out)))
        return out.astype(bool)

    def search(self, qs, qe, qc=None, order=ORDER_IDXS_CPP, values=False):
        """CSR result: (offsets int64[nq+1], out int32[P]).  ``order`` selects
        the C++ search_idxs order or the fully descending order; ``values``
        returns payloads instead of contig-local positions."""
        qs, qe, qc = self._queries(qs, qe, qc)
        nq = qs.shape[0]
        off = np.empty(nq + 1, np.int64)
        total = C.c_size_t(0)
        cap = 0
        out = np.empty(1, np.int32)
        for _ in range(2):
            st = self.lib.searchBatchIntoGpu(self.h, _p(qs), _p(qe), _p(qc), nq, int(order),
                                             1 if values else 0, _p(off), _p(out), cap,
                                             C.byref(total))
            if st == _capi.SI_ERR_CAPACITY:
                cap = int(total.value)
                out = np.empty(max(cap, 1), np.int32)
                continue
            check(st)
            break
        return off, out[: int(off[-1])] if nq else out[:0]

    def _setop(self, fn, qs, qe, qc, extra, want_hits):
        qs, qe, qc = self._queries(qs, qe, qc)
        nq = qs.shape[0]
        off = np.empty(nq + 1, np.int64)
        total = C.c_size_t(0)
        cap = 0
        bufs = (np.empty(1, self.dtype), np.empty(1, self.dtype), np.empty(1, np.int32))
        for _ in range(2):
            args = [self.h, _p(qs), _p(qe), _p(qc), nq, *extra, _p(off), _p(bufs[0]), _p(bufs[1])]
            if want_hits:
                args.append(_p(bufs[2]))
            st = fn(*args, cap, C.byref(total))
            if st == _capi.SI_ERR_CAPACITY:
                cap = int(total.value)
                bufs = (np.empty(cap, self.dtype), np.empty(cap, self.dtype), np.empty(cap, np.int32))
                continue
            check(st)
            break
        k = int(total.value)
        return off, bufs[0][:k], bufs[1][:k], bufs[2][:k]

    def search_keys(self, qs, qe, qc=None, order=ORDER_DESC, with_data=False):
        """search_keys (superintervals.hpp:913-938) / search_items: CSR offsets, each
        hit's start and end (and payload with ``with_data``), in ``order``."""
        qs, qe, qc = self._queries(qs, qe, qc)
        nq = qs.shape[0]
        off = np.empty(nq + 1, np.int64)
        total = C.c_size_t(0)
        cap = 0
        bufs = (np.empty(1, self.dtype), np.empty(1, self.dtype), np.empty(1, np.int32))
        for _ in range(2):
            st = self.lib.searchKeysBatchGpu(self.h, _p(qs), _p(qe), _p(qc), nq, int(order), _p(off), _p(bufs[0]),
                                             _p(bufs[1]), _p(bufs[2]) if with_data else None, cap,
                                             C.byref(total))
            if st == _capi.SI_ERR_CAPACITY:
                cap = int(total.value)
                bufs = (np.empty(cap, self.dtype), np.empty(cap, self.dtype), np.empty(cap, np.int32))
                continue
            check(st)
            break
        k = int(total.value)
        return (off, bufs[0][:k], bufs[1][:k]) + ((bufs[2][:k],) if with_data else ())

    def coverage(self, qs, qe, qc=None):
        """coverage (superintervals.hpp:979-1006) per query: (count uint64, covered)."""
        qs, qe, qc = self._queries(qs, qe, qc)
        nq = qs.shape[0]
        cnt = np.empty(nq, np.uint64)
        cov = np.empty(nq, self.dtype)
        check(self.lib.coverageBatchGpu(self.h, _p(qs), _p(qe), _p(qc), nq, _p(cnt), _p(cov)))
        return cnt, cov

    def intersect(self, qs, qe, qc=None, order=ORDER_IDXS_CPP):
        """intersection (superintervals.hpp:1158-1177) of the query intervals (another
        map's) with this index: CSR offsets, piece starts, piece ends and the hit's
        contig-local position, in the search order ``order``."""
        return self._setop(self.lib.intersectBatchGpu, qs, qe, qc, [int(order)], True)

    def difference(self, qs, qe, qc=None):
        """difference (superintervals.hpp:1186-1211): the pieces of each query interval
        not covered by this index (CSR offsets, piece starts, piece ends)."""
        off, s, e, _ = self._setop(self.lib.differenceBatchGpu, qs, qe, qc, [], False)
        return off, s, e


class IntervalMap:
    """Drop-in mirror of the reference's Python ``IntervalMap``
    (src/superintervals/intervalmap.pyx): intervals are end-inclusive, values
    are arbitrary Python objects, ``build()`` must precede queries, results come
    in the reference's order.  Queries run on the GPU through the C-ABI."""

    def __init__(self, device: int = 0):
        self._device = device
        self._starts: list = []
        self._ends: list = []
        self._values: list = []
        self._idx: Optional[GpuIndex] = None
        self._sorted = None  # (starts, ends, perm) after build

    # construction (pyx:41-131)
    def add(self, start: int, end: int, value=None):
        self._starts.append(int(start))
        self._ends.append(int(end))
        self._values.append(value)
        self._sorted = None

    @classmethod
    def from_arrays(cls, starts, ends, values=None):
        inst = cls()
        s = np.asarray(starts).astype(np.int64).tolist()
        e = np.asarray(ends).astype(np.int64).tolist()
        if len(s) != len(e):
            raise ValueError("starts and ends must have the same length")
        if values is not None and len(values) != len(s):
            raise ValueError("values length must match starts/ends length")
        inst._starts, inst._ends = s, e
        inst._values = list(values) if values is not None else [None] * len(s)
        inst.build()
        return inst

    def build(self):
        idx = GpuIndex(32, self._device)
        n = len(self._starts)
        if n:
            idx.add_arrays(np.asarray(self._starts, np.int32), np.asarray(self._ends, np.int32),
                           np.arange(n, dtype=np.int32))
        idx.build()
        s, e, perm, _ = idx.arrays()
        self._idx = idx
        self._sorted = (s, e, perm)
        self._by_input = self._values  # the device payload of an interval is its index here
        self._values = [self._values[p] for p in perm.tolist()] if n else []
        self._starts, self._ends = s.tolist(), e.tolist()

    def _need(self):
        if self._sorted is None:
            # the reference leaves queries before build() undefined; here they raise
            raise SIError(_capi.SI_ERR_NOT_BUILT, "call build() before querying")

    # element access (pyx:133-218)
    def __len__(self):
        return self.size()

    def __getitem__(self, index: int):
        return self.at(index)

    def size(self) -> int:
        return len(self._starts)

    def at(self, index: int):
        if self.size() == 0 or index < 0 or index >= self.size():
            raise IndexError("Index out of range")
        return self._starts[index], self._ends[index], self._values[index]

    def starts_at(self, index: int):
        return self.at(index)[0]

    def ends_at(self, index: int):
        return self.at(index)[1]

    def data_at(self, index: int):
        return self.at(index)[2]

    def clear(self):
        self._starts, self._ends, self._values = [], [], []
        self._idx, self._sorted = None, None

    def reserve(self, n: int):
        pass

    # single queries (pyx:241-361), answered as one-query batches
    def has_overlaps(self, start: int, end: int) -> bool:
        return bool(self.has_overlaps_batch([start], [end])[0]) if self.size() else False

    def count(self, start: int, end: int) -> int:
        return int(self.count_batch([start], [end])[0]) if self.size() else 0

    def search_idxs(self, start: int, end: int) -> list:
        return self.search_idxs_batch([start], [end])[0] if self.size() else []

    def search_values(self, start: int, end: int) -> list:
        return self.search_values_batch([start], [end])[0] if self.size() else []

    def search_keys(self, start: int, end: int) -> list:
        self._need()
        if not self.size():
            return []
        _, s, e = self._idx.search_keys([start], [end], order=ORDER_IDXS_CPP)
        return list(zip(s.tolist(), e.tolist()))

    def search_items(self, start: int, end: int) -> list:
        self._need()
        if not self.size():
            return []
        _, s, e, d = self._idx.search_keys([start], [end], order=ORDER_IDXS_CPP, with_data=True)
        v = self._by_input
        return [(a, b, v[p]) for a, b, p in zip(s.tolist(), e.tolist(), d.tolist())]

    def coverage(self, start: int, end: int):
        """(count, covered) as pyx:347-361: the number of overlapping intervals and the sum
        of their overlapping lengths min(end) - max(start) (no +1)."""
        self._need()
        if not self.size():
            return 0, 0
        cnt, cov = self._idx.coverage([start], [end])
        return int(cnt[0]), int(cov[0])

    # batch queries (pyx:363-494)
    @staticmethod
    def _q(starts, ends):
        s = np.ascontiguousarray(starts, dtype=np.int32)
        e = np.ascontiguousarray(ends, dtype=np.int32)
        if s.shape[0] != e.shape[0]:
            raise ValueError("starts and ends must have the same length")
        return s, e

    def count_batch(self, starts, ends) -> list:
        s, e = self._q(starts, ends)
        self._need()
        if self.size() == 0:
            return [0] * s.shape[0]
        return self._idx.count(s, e).astype(np.int64).tolist()

    def has_overlaps_batch(self, starts, ends) -> list:
        s, e = self._q(starts, ends)
        self._need()
        if self.size() == 0:
            return [False] * s.shape[0]
        return self._idx.has_overlaps(s, e).tolist()

    def search_idxs_batch(self, starts, ends) -> list:
        s, e = self._q(starts, ends)
        self._need()
        if self.size() == 0:
            return [[] for _ in range(s.shape[0])]
        off, out = self._idx.search(s, e, order=ORDER_IDXS_CPP)
        vals = out.tolist()
        return [vals[off[i]:off[i + 1]] for i in range(s.shape[0])]

    # set operations (pyx:577-643); results are new, built maps
    def intersection(self, other: "IntervalMap", combine=None) -> "IntervalMap":
        """Regions covered by both maps: for each interval of this map (in its
        current order) and each hit in ``other`` (C++ search_idxs order), the
        overlapping piece; data = combine(a, b), by default the tuple (a, b)."""
        other._need()
        out = IntervalMap()
        if self.size() and other.size():
            off, s, e, h = other._idx.intersect(np.asarray(self._starts, np.int32),
                                                 np.asarray(self._ends, np.int32), order=ORDER_IDXS_CPP)
            owner = np.repeat(np.arange(self.size()), np.diff(off)).tolist()
            av, bv = self._values, other._values
            for k, (ps, pe, hh) in enumerate(zip(s.tolist(), e.tolist(), h.tolist())):
                a, b = av[owner[k]], bv[hh]
                out.add(ps, pe, combine(a, b) if combine is not None else (a, b))
        out.build()
        return out

    def difference(self, other: "IntervalMap") -> "IntervalMap":
        """Regions of this map not covered by ``other`` (A minus B); each piece
        keeps its source interval's value."""
        other._need()
        out = IntervalMap()
        if self.size():
            off, s, e = other._idx.difference(np.asarray(self._starts, np.int32),
                                              np.asarray(self._ends, np.int32))
            owner = np.repeat(np.arange(self.size()), np.diff(off)).tolist()
            for k, (ps, pe) in enumerate(zip(s.tolist(), e.tolist())):
                out.add(ps, pe, self._values[owner[k]])
        out.build()
        return out

    def search_values_batch(self, starts, ends) -> list:
        s, e = self._q(starts, ends)
        self._need()
        if self.size() == 0:
            return [[] for _ in range(s.shape[0])]
        off, out = self._idx.search(s, e, order=ORDER_DESC)
        v = self._values
        pos = out.tolist()
        return [[v[p] for p in pos[off[i]:off[i + 1]]] for i in range(s.shape[0])]
