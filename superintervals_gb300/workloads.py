"""Seeded synthetic interval workloads.

The reference publishes timings only on real BED files that are not
available here (test/benchmark.md:16-22), so every workload below is a seeded
synthetic stand-in with the shapes, sizes and length distributions of the
five configurations this library is measured on.  Intervals are
END-INCLUSIVE: a drawn length ``L`` gives ``end = start + L - 1``, as in the
reference (src/superintervals.hpp:38, test/bench.cpp:210).

Seeds: reference intervals use seed 1, queries seed 2, Zipf/Poisson draws
seed 3.  Generation uses numpy's PCG64 stream, so a workload is identical
from run to run on one machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

# GRCh38 primary assembly chromosome lengths (public assembly statistics).
HUMAN_CONTIGS = [
    ("chr1", 248956422), ("chr2", 242193529), ("chr3", 198295559),
    ("chr4", 190214555), ("chr5", 181538259), ("chr6", 170805979),
    ("chr7", 159345973), ("chr8", 145138636), ("chr9", 138394717),
    ("chr10", 133797422), ("chr11", 135086622), ("chr12", 133275309),
    ("chr13", 114364328), ("chr14", 107043718), ("chr15", 101991189),
    ("chr16", 90338345), ("chr17", 83257441), ("chr18", 80373285),
    ("chr19", 58617616), ("chr20", 64444167), ("chr21", 46709983),
    ("chr22", 50818468), ("chrX", 156040895), ("chrY", 57227415),
]

REF_SEED, QUERY_SEED, AUX_SEED = 1, 2, 3


@dataclass
class Workload:
    """Reference intervals grouped by contig plus a query batch.

    ``seg`` holds ``n_contigs + 1`` offsets: contig ``g``'s reference
    intervals are ``starts[seg[g]:seg[g+1]]`` (in insertion order, not
    sorted).  ``q_contig`` is None for single-contig workloads.
    """

    name: str
    starts: np.ndarray
    ends: np.ndarray
    data: np.ndarray
    seg: np.ndarray
    q_starts: np.ndarray
    q_ends: np.ndarray
    q_contig: Optional[np.ndarray] = None
    contigs: List[tuple] = field(default_factory=list)
    notes: str = ""

    @property
    def n(self) -> int:
        return int(self.starts.shape[0])

    @property
    def nq(self) -> int:
        return int(self.q_starts.shape[0])

    @property
    def dtype(self):
        return self.starts.dtype


def _lognormal_len(rng, n, median, sigma, lo, hi):
    z = rng.standard_normal(n)
    ln = np.exp(np.log(median) + sigma * z)
    return np.clip(np.rint(ln), lo, hi).astype(np.int64)


def _split_counts(total, weights):
    w = np.asarray(weights, dtype=np.float64)
    raw = total * w / w.sum()
    cnt = np.floor(raw).astype(np.int64)
    rem = total - int(cnt.sum())
    order = np.argsort(-(raw - cnt), kind="stable")
    cnt[order[:rem]] += 1
    return cnt


def config1(n=100_000, nq=100_000) -> Workload:
    """Plain small: one 248,956,422-bp contig, uniform starts, log-normal
    lengths (median 500, sigma 1.0, clipped to [1, 100k]); int32."""
    clen = HUMAN_CONTIGS[0][1]
    r = np.random.Generator(np.random.PCG64(REF_SEED))
    s = r.integers(0, clen, n, dtype=np.int64)
    ln = _lognormal_len(r, n, 500, 1.0, 1, 100_000)
    q = np.random.Generator(np.random.PCG64(QUERY_SEED))
    qs = q.integers(0, clen, nq, dtype=np.int64)
    qln = _lognormal_len(q, nq, 500, 1.0, 1, 100_000)
    return Workload(
        name=f"plain-small n={n} q={nq} int32 1 contig",
        starts=s.astype(np.int32), ends=(s + ln - 1).astype(np.int32),
        data=np.arange(n, dtype=np.int32), seg=np.array([0, n], dtype=np.int64),
        q_starts=qs.astype(np.int32), q_ends=(qs + qln - 1).astype(np.int32),
        contigs=[HUMAN_CONTIGS[0]],
    )


def _mixture_lengths(rng, n, short_len=150, long_lo=10_000, long_hi=50_000, p_long=0.10):
    is_long = rng.random(n) < p_long
    ln = np.full(n, short_len, dtype=np.int64)
    k = int(is_long.sum())
    ln[is_long] = rng.integers(long_lo, long_hi + 1, k, dtype=np.int64)
    return ln


def config2(n=10_000_000, nq=10_000_000) -> Workload:
    """Plain mid: one 248,956,422-bp contig; lengths 90% fixed 150 bp and
    10% uniform 10-50 kb; queries sorted by start; int32."""
    clen = HUMAN_CONTIGS[0][1]
    r = np.random.Generator(np.random.PCG64(REF_SEED))
    s = r.integers(0, clen, n, dtype=np.int64)
    ln = _mixture_lengths(r, n)
    q = np.random.Generator(np.random.PCG64(QUERY_SEED))
    qs = np.sort(q.integers(0, clen, nq, dtype=np.int64))
    qln = _mixture_lengths(q, nq)
    return Workload(
        name=f"plain-mid n={n} q={nq} int32 1 contig sorted queries",
        starts=s.astype(np.int32), ends=(s + ln - 1).astype(np.int32),
        data=np.arange(n, dtype=np.int32), seg=np.array([0, n], dtype=np.int64),
        q_starts=qs.astype(np.int32), q_ends=(qs + qln - 1).astype(np.int32),
        contigs=[HUMAN_CONTIGS[0]],
    )


def config3(n=50_000_000, nq=50_000_000, contigs=None, long_queries=False) -> Workload:
    """Batched uneven contigs: 24 human-like contigs; intervals and queries
    split in proportion to contig length; log-normal lengths (median 300,
    sigma 1.5, clipped to [1, 100k]) plus 1% long intervals of 1-5 Mb on the
    reference side.  Queries are unsorted and, unless ``long_queries``, use
    the short component only."""
    contigs = list(contigs or HUMAN_CONTIGS)
    lens = np.array([c[1] for c in contigs], dtype=np.int64)
    cnt = _split_counts(n, lens)
    qcnt = _split_counts(nq, lens)
    r = np.random.Generator(np.random.PCG64(REF_SEED))
    s_parts, l_parts = [], []
    for g, c in enumerate(cnt):
        s_parts.append(r.integers(0, lens[g], c, dtype=np.int64))
        ln = _lognormal_len(r, c, 300, 1.5, 1, 100_000)
        is_long = r.random(c) < 0.01
        k = int(is_long.sum())
        ln[is_long] = r.integers(1_000_000, 5_000_001, k, dtype=np.int64)
        l_parts.append(ln)
    s = np.concatenate(s_parts)
    ln = np.concatenate(l_parts)
    seg = np.zeros(len(contigs) + 1, dtype=np.int64)
    seg[1:] = np.cumsum(cnt)
    q = np.random.Generator(np.random.PCG64(QUERY_SEED))
    qc = np.repeat(np.arange(len(contigs), dtype=np.int32), qcnt)
    q.shuffle(qc)
    qs = (q.random(nq) * lens[qc]).astype(np.int64)
    qln = _lognormal_len(q, nq, 300, 1.5, 1, 100_000)
    if long_queries:
        is_long = q.random(nq) < 0.01
        qln[is_long] = q.integers(1_000_000, 5_000_001, int(is_long.sum()), dtype=np.int64)
    return Workload(
        name=f"batched-contigs n={n} q={nq} int32 {len(contigs)} contigs unsorted queries",
        starts=s.astype(np.int32), ends=(s + ln - 1).astype(np.int32),
        data=np.arange(n, dtype=np.int32), seg=seg,
        q_starts=qs.astype(np.int32), q_ends=(qs + qln - 1).astype(np.int32),
        q_contig=qc, contigs=contigs,
        notes="queries: short log-normal component only" if not long_queries else
              "queries: short component + 1% long 1-5 Mb",
    )


def config3_subset(names, scale=1.0, n_full=50_000_000, nq_full=50_000_000) -> Workload:
    """Configuration 3 on a subset of its contigs with the subset's share of the intervals and
    queries (contig length over the whole genome), so that intervals per bp and hits per query
    stay those of the full configuration (~500 hits per query from the 1% of 1-5 Mb
    intervals): a small case of the full-size regime for parity tests and profiles."""
    names = list(names)
    sub = [c for c in HUMAN_CONTIGS if c[0] in set(names)]
    if len(sub) != len(set(names)):
        raise ValueError(f"unknown contig in {names}")
    share = sum(c[1] for c in sub) / sum(c[1] for c in HUMAN_CONTIGS)
    n, nq = max(1000, int(n_full * scale * share)), max(1000, int(nq_full * scale * share))
    return config3(n=n, nq=nq, contigs=sub)


def _clustered_starts(rng, zrng, n, span, hotspots=10_000, zipf_s=1.1, jitter=5_000.0,
                      frac_hot=0.70):
    hot_pos = zrng.integers(0, span, hotspots, dtype=np.int64)
    ranks = np.arange(1, hotspots + 1, dtype=np.float64)
    p = ranks ** (-zipf_s)
    cdf = np.cumsum(p)
    cdf /= cdf[-1]
    is_hot = rng.random(n) < frac_hot
    k = int(is_hot.sum())
    pick = np.searchsorted(cdf, zrng.random(k), side="right")
    pick = np.minimum(pick, hotspots - 1)
    s = rng.integers(0, span, n, dtype=np.int64)
    s[is_hot] = hot_pos[pick] + np.rint(rng.standard_normal(k) * jitter).astype(np.int64)
    return np.clip(s, 0, span - 1)


def config4(n=100_000_000, nq=100_000_000, span=3_100_000_000) -> Workload:
    """Learned index: int64 coordinates over a 3.1e9-bp span; starts 70% from
    10k Zipf(1.1) hotspots with Gaussian jitter (sd 5 kb), 30% uniform;
    log-normal lengths (median 1 kb, sigma 1.0, clipped to [1, 1M])."""
    r = np.random.Generator(np.random.PCG64(REF_SEED))
    z = np.random.Generator(np.random.PCG64(AUX_SEED))
    s = _clustered_starts(r, z, n, span)
    ln = _lognormal_len(r, n, 1000, 1.0, 1, 1_000_000)
    q = np.random.Generator(np.random.PCG64(QUERY_SEED))
    z2 = np.random.Generator(np.random.PCG64(AUX_SEED))  # same hotspot set as the references
    qs = _clustered_starts(q, z2, nq, span)
    qln = _lognormal_len(q, nq, 1000, 1.0, 1, 1_000_000)
    return Workload(
        name=f"learned n={n} q={nq} int64 span={span}",
        starts=s, ends=s + ln - 1, data=np.arange(n, dtype=np.int32),
        seg=np.array([0, n], dtype=np.int64), q_starts=qs, q_ends=qs + qln - 1,
        contigs=[("span", span)],
    )


def config5_index(n=200_000_000, contigs=None) -> Workload:
    """Serving-loop resident index: ``n`` int32 intervals over the 24
    human-like contigs, log-normal lengths (median 500, sigma 1.0)."""
    contigs = list(contigs or HUMAN_CONTIGS)
    lens = np.array([c[1] for c in contigs], dtype=np.int64)
    cnt = _split_counts(n, lens)
    r = np.random.Generator(np.random.PCG64(REF_SEED))
    s = np.concatenate([r.integers(0, lens[g], c, dtype=np.int64) for g, c in enumerate(cnt)])
    ln = _lognormal_len(r, n, 500, 1.0, 1, 100_000)
    seg = np.zeros(len(contigs) + 1, dtype=np.int64)
    seg[1:] = np.cumsum(cnt)
    empty = np.zeros(0, dtype=np.int32)
    return Workload(
        name=f"serving n={n} int32 {len(contigs)} contigs",
        starts=s.astype(np.int32), ends=(s + ln - 1).astype(np.int32),
        data=np.arange(n, dtype=np.int32), seg=seg, q_starts=empty, q_ends=empty,
        q_contig=empty, contigs=contigs,
    )


def config5_requests(n_requests, contigs=None, rate_per_s=200.0, max_size=1_000_000):
    """Serving-loop request stream: Poisson arrivals (``rate_per_s``), request
    sizes log-uniform on [1, max_size] queries, query lengths log-normal
    (median 500, sigma 1.0).  Returns (arrival_s, sizes, qc, qs, qe) with the
    queries of all requests concatenated in arrival order."""
    contigs = list(contigs or HUMAN_CONTIGS)
    lens = np.array([c[1] for c in contigs], dtype=np.int64)
    z = np.random.Generator(np.random.PCG64(AUX_SEED))
    gaps = z.exponential(1.0 / rate_per_s, n_requests)
    arrival = np.cumsum(gaps)
    sizes = np.floor(np.exp(z.random(n_requests) * np.log(max_size + 1))).astype(np.int64)
    sizes = np.clip(sizes, 1, max_size)
    total = int(sizes.sum())
    q = np.random.Generator(np.random.PCG64(QUERY_SEED))
    p = lens / lens.sum()
    qc = q.choice(len(contigs), size=total, p=p).astype(np.int32)
    qs = (q.random(total) * lens[qc]).astype(np.int64)
    qln = _lognormal_len(q, total, 500, 1.0, 1, 100_000)
    return arrival, sizes, qc, qs.astype(np.int32), (qs + qln - 1).astype(np.int32)


def random_nested(seed, n, nq, dtype=np.int32, span=100_000, dup_frac=0.2,
                  max_len=5_000) -> Workload:
    """Small randomized differential case with nesting, shared endpoints and
    exact duplicates (the brute-force style check the reference lacks)."""
    r = np.random.Generator(np.random.PCG64(seed))
    s = r.integers(0, span, n, dtype=np.int64)
    ln = r.integers(1, max_len, n, dtype=np.int64)
    is_long = r.random(n) < 0.05          # a few long containers for deep nesting
    ln[is_long] = r.integers(max_len, span, int(is_long.sum()), dtype=np.int64)
    e = s + ln - 1
    nd = int(n * dup_frac)
    if nd and n > 1:
        src = r.integers(0, n, nd)
        dst = r.integers(0, n, nd)
        s[dst] = s[src]
        e[dst] = e[src]
    qs = r.integers(-10, span + 10, nq, dtype=np.int64)
    qe = qs + r.integers(-5, max_len, nq, dtype=np.int64)
    return Workload(
        name=f"random-nested seed={seed}", starts=s.astype(dtype), ends=e.astype(dtype),
        data=np.arange(n, dtype=np.int32), seg=np.array([0, n], dtype=np.int64),
        q_starts=qs.astype(dtype), q_ends=qe.astype(dtype),
    )


CONFIGS = {
    "config1": config1,
    "config2": config2,
    "config3": config3,
    "config4": config4,
}
