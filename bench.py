"""Benchmark of the batch overlap-query path (search_idxs) on one GB300.

One step = one search_idxs pass (count -> scan -> emit, exact per-query CSR
offsets, the reference's C++ order) over the whole query batch of the chosen
workload, against a device-resident index.  Inputs are seeded synthetic
intervals with the configuration's sizes and length distributions (the
reference's published timings use BED files that are not available here).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config config3]
                  [--path batched|plain] [--ub learned|eytzinger|binary]
  python bench.py --impl reference ...   # the reference algorithm on the host cores
  python bench.py --config config4       # --op upper_bound: learned vs Eytzinger vs binary
  python bench.py --config config5       # serving loop: Poisson requests, p50/p99 latency

Prints one JSON line.  `value` = queries/s with inputs resident in HBM;
`e2e` = the same through the C-ABI with pinned host buffers (H2D of the
queries and D2H of the CSR result inside the timed region).  Under torchrun
(N > 1) each rank holds its own replica of the index and processes its own
query batch of the configuration's size (weak scaling, no data-path
collective); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("overlap queries/s + result pairs/s on 1 GB300; % HBM peak; batched+learned vs plain")
METRIC_SERVE = "serving loop on 1 GB300: queries/s (saturated) and p50/p99 request latency at the offered rate"
ROW_OPS = ["intersect", "difference", "coverage", "keys", "count", "bed_ingest"]
ROW_DEFAULT_SCALE = 0.25   # full-size intersection pieces (25.5e9 x 12 B) would not fit in HBM
METRIC_UB = "upper-bound queries/s on 1 GB300: learned two-stage index vs binary search, bit-identical"
PEAK_FALLBACK_GBS = 6800.0
# DRAM traffic of the emit kernel per unit, from an ncu capture of dram__bytes_write.sum and
# dram__bytes_read.sum on configuration 3's density (profiles/k_tiles_config3_dram.md): writes
# scale with result pairs, reads with queries
EMIT_DRAM_WRITE_PER_PAIR = 3.972
EMIT_DRAM_READ_PER_QUERY = 182.1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="config3",
                    choices=["config1", "config2", "config3", "config4", "config5"])
    ap.add_argument("--requests", type=int, default=600, help="config5: requests in the stream")
    ap.add_argument("--rate", type=float, default=200.0, help="config5: offered requests/s (Poisson)")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink N and Q (tests only)")
    ap.add_argument("--contigs", default=None,
                    help="config3: only these contigs (comma-separated names), at the full "
                         "configuration's density (small profiling cases with the same hits per query)")
    ap.add_argument("--path", default="batched", choices=["batched", "plain", "auto"])
    ap.add_argument("--ub", default="learned", choices=["learned", "eytzinger", "binary"])
    ap.add_argument("--op", default=None, choices=["search_idxs", "upper_bound"] + ROW_OPS,
                    help="search_idxs (default); upper_bound (default for config4, whose full-size "
                         "result, ~2.9e13 pairs, cannot be materialised); or one of the operations "
                         "built on the path (intersect, difference, coverage, keys, count, bed_ingest)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default batched-path tunables")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--profile-only", action="store_true",
                    help="run warmup+steps without the extra legs (for ncu launch lists)")
    return ap.parse_args()


# ----------------------------------------------------------------------------- workload
def make_workload(cfg, scale, rank, contigs=None):
    from superintervals_gb300 import workloads as W
    sizes = {"config1": (100_000, 100_000), "config2": (10_000_000, 10_000_000),
             "config3": (50_000_000, 50_000_000), "config4": (100_000_000, 100_000_000)}
    n, nq = sizes[cfg]
    if cfg == "config3" and contigs:
        # a subset of the contigs with its share of the intervals and queries
        try:
            wl = W.config3_subset(contigs.split(","), scale, n, nq)
        except ValueError as e:
            raise SystemExit(f"--contigs {contigs}: {e}")
    else:
        n, nq = max(1000, int(n * scale)), max(1000, int(nq * scale))
        wl = getattr(W, cfg)(n=n, nq=nq)
    if rank:
        # weak scaling: every rank gets its own query batch of the same size
        rng = np.random.Generator(np.random.PCG64(1000 + rank))
        perm = rng.permutation(wl.nq)
        wl.q_starts, wl.q_ends = wl.q_starts[perm], wl.q_ends[perm]
        if wl.q_contig is not None:
            wl.q_contig = wl.q_contig[perm]
    return wl


def workload_desc(cfg, wl):
    d = {"workload": wl.name, "n_intervals": wl.n, "n_queries": wl.nq,
         "coord": str(wl.dtype), "contigs": int(len(wl.seg) - 1), "op": "search_idxs (C++ order)",
         "inputs": "larger than L2 (index + queries > 129 MB); L2 flushed between steps"}
    if wl.notes:
        d["notes"] = wl.notes
    return d


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, nm in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return PEAK_FALLBACK_GBS, "fallback"


# ----------------------------------------------------------------------------- GPU arm
def local_device() -> int:
    """This rank's GPU (one process per GPU under torchrun)."""
    return int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x: float, dist) -> float:
    """The slowest rank's time (the whole job ends when it does); x itself at N = 1."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args, rank, world, dist):
    from superintervals_gb300 import _capi
    from superintervals_gb300.interval_map import GpuIndex
    lib = _capi.load()
    wl = make_workload(args.config, args.scale, rank, args.contigs)
    s_bytes = wl.dtype.itemsize
    idx = GpuIndex(64 if s_bytes == 8 else 32, local_device())
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None)
    t0 = time.perf_counter()
    idx.build()
    build_s = time.perf_counter() - t0
    path = {"batched": _capi.PATH_BATCHED, "plain": _capi.PATH_PLAIN, "auto": _capi.PATH_AUTO}[args.path]
    ub = {"learned": _capi.UB_LEARNED, "eytzinger": _capi.UB_EYTZINGER, "binary": _capi.UB_BINARY}[args.ub]
    idx.set_path(path)
    idx.set_upper_bound(ub)
    st = idx.stream
    nq = wl.nq

    def dalloc(nbytes):
        p = C.c_void_p()
        _capi.check(lib.deviceMallocGpu(C.byref(p), max(int(nbytes), 1)))
        return p

    def h2d(dst, arr):
        _capi.check(lib.memcpyGpu(dst, C.c_void_p(arr.ctypes.data), arr.nbytes, st))

    d_qs, d_qe = dalloc(wl.q_starts.nbytes), dalloc(wl.q_ends.nbytes)
    h2d(d_qs, np.ascontiguousarray(wl.q_starts))
    h2d(d_qe, np.ascontiguousarray(wl.q_ends))
    d_qc = None
    if wl.q_contig is not None:
        d_qc = dalloc(wl.q_contig.nbytes)
        h2d(d_qc, np.ascontiguousarray(wl.q_contig))
    d_off = dalloc(8 * (nq + 1))
    total = C.c_size_t(0)
    st_ = lib.searchDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, 0, 0, d_off, None, 0, C.byref(total), st)
    if st_ not in (_capi.SI_OK, _capi.SI_ERR_CAPACITY):
        _capi.check(st_)
    P = int(total.value)
    tuned = None
    if path == _capi.PATH_BATCHED and not args.no_autotune:
        from superintervals_gb300 import autotune
        # timed on the whole batch: a prefix of unsorted queries is sparser along the genome and
        # favours smaller tiles.  The requested upper-bound provider stays fixed.
        tuned = autotune.tune(idx, d_qs, d_qe, d_qc, nq, sample=0, use_cache=False, keep_upper_bound=True)
    d_out = dalloc(4 * max(P, 1))

    def step():
        _capi.check(lib.searchDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, 0, 0, d_off, d_out, P,
                                        C.byref(total), st))

    ev = [C.c_void_p(), C.c_void_p()]
    for e in ev:
        _capi.check(lib.eventCreateGpu(C.byref(e)))

    def timed(k, w, fn, on_start=None):
        for _ in range(w):
            _capi.check(lib.flushL2Gpu(st))
            fn()
        _capi.check(lib.streamSynchronizeGpu(st))
        if dist:
            dist.barrier()
        if on_start:
            on_start()
        total_ms = 0.0
        for _ in range(k):
            _capi.check(lib.flushL2Gpu(st))
            _capi.check(lib.eventRecordGpu(ev[0], st))
            fn()
            _capi.check(lib.eventRecordGpu(ev[1], st))
            _capi.check(lib.streamSynchronizeGpu(st))
            ms = C.c_float()
            _capi.check(lib.eventElapsedMsGpu(ev[0], ev[1], C.byref(ms)))
            total_ms += ms.value
        if dist:
            dist.barrier()
        return total_ms

    launches = {}

    def counted():
        launches["before"] = lib.getLaunchCountGpu()

    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        total_ms = timed(args.steps, args.warmup, step, on_start=counted)
    launches_timed = lib.getLaunchCountGpu() - launches["before"]
    total_ms = max_over_ranks(total_ms, dist)
    ms_per_step = total_ms / args.steps
    res = {"wl": wl, "P": P, "nq": nq, "ms_per_step": ms_per_step, "build_s": build_s,
           "launches": launches_timed, "tuned": tuned,
           "clocks": clk.summary(), "s_bytes": s_bytes}
    if args.profile_only:
        return res
    # the timed step's own result for the first queries, for the comparison with the oracle
    if rank == 0 and not args.no_cpu:
        kq = min(nq, PARITY_QUERIES)
        h_off = np.empty(kq + 1, np.int64)
        _capi.check(lib.memcpyGpu(C.c_void_p(h_off.ctypes.data), d_off, h_off.nbytes, st))
        _capi.check(lib.streamSynchronizeGpu(st))
        h_val = np.empty(int(h_off[-1]), np.int32)
        if h_val.size:
            _capi.check(lib.memcpyGpu(C.c_void_p(h_val.ctypes.data), d_out, h_val.nbytes, st))
        _capi.check(lib.streamSynchronizeGpu(st))
        res["gpu_prefix"] = (h_off, h_val)

    # per-phase device times (count / scan / emit / prepare) for the roofline
    _capi.check(lib.setProfilingGpu(idx.h, 1))
    for _ in range(max(1, min(3, args.steps))):
        _capi.check(lib.flushL2Gpu(st))
        step()
    ms4 = (C.c_double * 4)()
    n4 = (C.c_int64 * 4)()
    _capi.check(lib.getPhaseTimesGpu(idx.h, ms4, n4))
    res["phase_ms"] = [ms4[k] / max(1, n4[k]) for k in range(4)]
    if path == _capi.PATH_BATCHED:
        # the emit in each of its two modes for the long-interval list's section of part B
        # (copied around its misses / filtered), the tuned mode restored afterwards
        cur = C.c_int64(1)
        _capi.check(lib.getBatchedOptionGpu(idx.h, _capi.OPT_EMIT_COPY, C.byref(cur)))
        res["emit_mode_ms"] = {}
        for mode, name in ((1, "copy"), (0, "filter")):
            _capi.check(lib.setProfilingGpu(idx.h, 0))
            _capi.check(lib.setProfilingGpu(idx.h, 1))
            _capi.check(lib.setBatchedOptionGpu(idx.h, _capi.OPT_EMIT_COPY, mode))
            for _ in range(max(1, min(3, args.steps))):
                _capi.check(lib.flushL2Gpu(st))
                step()
            _capi.check(lib.getPhaseTimesGpu(idx.h, ms4, n4))
            res["emit_mode_ms"][name] = ms4[2] / max(1, n4[2])
        _capi.check(lib.setBatchedOptionGpu(idx.h, _capi.OPT_EMIT_COPY, cur.value))
        res["emit_copy_tuned"] = int(cur.value)
    _capi.check(lib.setProfilingGpu(idx.h, 0))

    # the plain one-query-per-thread GPU path on the same inputs (the 1.0x baseline)
    if not args.no_plain and args.path != "plain":
        idx.set_path(_capi.PATH_PLAIN)
        idx.set_upper_bound(_capi.UB_BINARY)
        res["plain_ms"] = timed(max(1, args.steps // 2), 1, step) / max(1, args.steps // 2)
        idx.set_path(path)
        idx.set_upper_bound(ub)

    lib.deviceFreeGpu(d_out)       # the e2e leg below stages its own result buffer
    d_out = None
    # e2e through the C-ABI with pinned host buffers
    if not args.no_e2e:
        def pinned(nbytes):
            p = C.c_void_p()
            _capi.check(lib.hostMallocPinnedGpu(C.byref(p), max(int(nbytes), 1)))
            return p
        hq_s, hq_e = pinned(wl.q_starts.nbytes), pinned(wl.q_ends.nbytes)
        C.memmove(hq_s, wl.q_starts.ctypes.data, wl.q_starts.nbytes)
        C.memmove(hq_e, wl.q_ends.ctypes.data, wl.q_ends.nbytes)
        hq_c = None
        if wl.q_contig is not None:
            hq_c = pinned(wl.q_contig.nbytes)
            C.memmove(hq_c, wl.q_contig.ctypes.data, wl.q_contig.nbytes)
        h_off = pinned(8 * (nq + 1))
        h_out = pinned(4 * max(P, 1))
        # the library's default output budget: the result comes back in chunks, the emit of
        # one overlapping the device-to-host copy of the previous one

        def e2e_step():
            _capi.check(lib.searchBatchIntoGpu(idx.h, hq_s, hq_e, hq_c, nq, 0, 0, h_off, h_out, P,
                                               C.byref(total)))
        for _ in range(max(1, args.warmup)):
            e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        k = max(1, args.steps)
        for _ in range(k):
            e2e_step()
        e2e_s = (time.perf_counter() - t0) / k
        res["e2e_s"] = max_over_ranks(e2e_s, dist)
        free_b, tot_b = C.c_size_t(0), C.c_size_t(0)
        _capi.check(lib.deviceMemInfoGpu(local_device(), C.byref(free_b), C.byref(tot_b)))
        res["e2e_chunks"] = -(-4 * P // max(tot_b.value // 16, 4 << 30))   # the library's default chunk budget
        res["h2d_bytes"] = wl.q_starts.nbytes + wl.q_ends.nbytes + (wl.q_contig.nbytes if hq_c else 0)
        res["d2h_bytes"] = 8 * (nq + 1) + 4 * P
        # the host link this box gives, copied the way the e2e call copies its result: 4 GiB
        # device-to-host copies into the same pinned buffer, over the whole result span, best
        # of two repeats (the first also maps the fresh device buffer)
        chunk = min(4 * P, 4 << 30)
        if chunk >= (64 << 20):
            span = 4 * P
            d_tmp = dalloc(chunk)
            best = None
            for _ in range(2):
                t0 = time.perf_counter()
                for off_b in range(0, span - chunk + 1, chunk):
                    _capi.check(lib.memcpyGpu(C.c_void_p(h_out.value + off_b), d_tmp, chunk, st))
                _capi.check(lib.streamSynchronizeGpu(st))
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            res["d2h_link_GBps"] = (span // chunk) * chunk / best / 1e9
            lib.deviceFreeGpu(d_tmp)
        for p in (hq_s, hq_e, hq_c, h_off, h_out):
            if p:
                lib.hostFreePinnedGpu(p)
    # latency of single-query calls (the drop-in's per-query methods are one-query batches
    # through the host-buffer C-ABI): count and search_idxs of one query, median of 200 calls
    if rank == 0:
        one_s, one_e = wl.q_starts[:1].copy(), wl.q_ends[:1].copy()
        one_c = None if wl.q_contig is None else wl.q_contig[:1].copy()
        cnt1 = np.zeros(1, np.uint32)
        off1 = np.zeros(2, np.int64)
        val1 = np.zeros(1 << 16, np.int32)
        f_cnt = lib.countOverlapsBatchGpu_i64 if s_bytes == 8 else lib.countOverlapsBatchGpu
        lat = {"count": [], "search_idxs": []}
        saved = path
        idx.set_path(_capi.PATH_AUTO)     # one query takes the plain path
        for _ in range(220):
            t0 = time.perf_counter()
            _capi.check(f_cnt(idx.h, C.c_void_p(one_s.ctypes.data), C.c_void_p(one_e.ctypes.data),
                              None if one_c is None else C.c_void_p(one_c.ctypes.data), 1,
                              C.c_void_p(cnt1.ctypes.data)))
            t1 = time.perf_counter()
            _capi.check(lib.searchBatchIntoGpu(idx.h, C.c_void_p(one_s.ctypes.data), C.c_void_p(one_e.ctypes.data),
                                               None if one_c is None else C.c_void_p(one_c.ctypes.data), 1, 0, 0,
                                               C.c_void_p(off1.ctypes.data), C.c_void_p(val1.ctypes.data),
                                               val1.size, C.byref(total)))
            t2 = time.perf_counter()
            lat["count"].append(t1 - t0)
            lat["search_idxs"].append(t2 - t1)
        idx.set_path(saved)
        res["single_query_us"] = {k: 1e6 * statistics.median(v[20:]) for k, v in lat.items()}
    for p in (d_qs, d_qe, d_qc, d_off, d_out):
        if p:
            lib.deviceFreeGpu(p)
    idx.close()
    return res


# ----------------------------------------------------------------------------- upper bound
UB_MODES = (("binary", 0), ("eytzinger", 1), ("learned", 2))


def run_gpu_ub(args, rank, world, dist):
    """Upper bound of every query end (upperBoundDeviceGpu) with each provider over the
    same device-resident batch; every provider's output must equal binary search's."""
    from superintervals_gb300 import _capi
    from superintervals_gb300.interval_map import GpuIndex
    lib = _capi.load()
    wl = make_workload(args.config, args.scale, rank, args.contigs)
    s_bytes = wl.dtype.itemsize
    idx = GpuIndex(64 if s_bytes == 8 else 32, local_device())
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None)
    t0 = time.perf_counter()
    idx.build()
    build_s = time.perf_counter() - t0
    st = idx.stream
    nq = wl.nq

    def dalloc(nbytes):
        p = C.c_void_p()
        _capi.check(lib.deviceMallocGpu(C.byref(p), max(int(nbytes), 1)))
        return p

    qe = np.ascontiguousarray(wl.q_ends)
    qc = None if wl.q_contig is None else np.ascontiguousarray(wl.q_contig)
    d_qe, d_out = dalloc(qe.nbytes), dalloc(4 * nq)
    _capi.check(lib.memcpyGpu(d_qe, C.c_void_p(qe.ctypes.data), qe.nbytes, st))
    d_qc = None
    if qc is not None:
        d_qc = dalloc(qc.nbytes)
        _capi.check(lib.memcpyGpu(d_qc, C.c_void_p(qc.ctypes.data), qc.nbytes, st))
    ev = [C.c_void_p(), C.c_void_p()]
    for e in ev:
        _capi.check(lib.eventCreateGpu(C.byref(e)))
    host = np.empty(nq, dtype=np.int32)
    ref = None
    res = {"wl": wl, "nq": nq, "s_bytes": s_bytes, "build_s": build_s, "modes": {}}
    # each provider per query (plain path: one thread per query in the batch's order) and
    # through the sorted batch (batched path: the ends radix-sorted, two searches per 256
    # sorted ends, the rest resolved in a shared-memory window, answers scattered back)
    for path_name, path in (("per_query", _capi.PATH_PLAIN), ("sorted_batch", _capi.PATH_BATCHED)):
        idx.set_path(path)
        for name, mode in UB_MODES:
            t0 = time.perf_counter()
            idx.set_upper_bound(mode)          # builds the provider's structure (model / tree)
            prep_s = time.perf_counter() - t0

            def step():
                _capi.check(lib.upperBoundDeviceGpu(idx.h, d_qe, d_qc, nq, mode, d_out, st))
            for _ in range(args.warmup):
                _capi.check(lib.flushL2Gpu(st))
                step()
            _capi.check(lib.streamSynchronizeGpu(st))
            if dist:
                dist.barrier()
            k0 = lib.getLaunchCountGpu()
            total_ms = 0.0
            with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
                for _ in range(args.steps):
                    _capi.check(lib.flushL2Gpu(st))
                    _capi.check(lib.eventRecordGpu(ev[0], st))
                    step()
                    _capi.check(lib.eventRecordGpu(ev[1], st))
                    _capi.check(lib.streamSynchronizeGpu(st))
                    ms = C.c_float()
                    _capi.check(lib.eventElapsedMsGpu(ev[0], ev[1], C.byref(ms)))
                    total_ms += ms.value
            launches = lib.getLaunchCountGpu() - k0   # the L2 flush is a memset, not counted
            total_ms = max_over_ranks(total_ms, dist)
            _capi.check(lib.memcpyGpu(C.c_void_p(host.ctypes.data), d_out, host.nbytes, st))
            _capi.check(lib.streamSynchronizeGpu(st))
            if ref is None:
                ref = host.copy()
                same = True
            else:
                same = bool(np.array_equal(host, ref))
            key = name if path_name == "per_query" else f"{name}+sorted"
            res["modes"][key] = {"ms_per_step": total_ms / args.steps, "prepare_s": prep_s,
                                 "identical_to_binary": same, "launches": launches,
                                 "clocks": clk.summary(), "path": path_name}
    idx.set_path(_capi.PATH_AUTO)
    # the oracle's upper bound on a sample (sanity check of the binary result itself)
    from oracle.oracle import Oracle
    o = Oracle()
    m = o.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
    k = min(nq, 1_000_000)
    want = o.upper_bound_batch(m, qe[:k], None if qc is None else qc[:k], nthreads=host_threads())
    res["oracle_sample_ok"] = bool(np.array_equal(ref[:k].astype(np.int64), want))
    res["oracle_map"] = (o, m)
    # e2e: H2D of the query ends, the learned upper bound and D2H of the result, all
    # through the C-ABI from pinned host memory
    if not args.no_e2e:
        mode = dict(UB_MODES)[args.ub]
        idx.set_upper_bound(mode)
        idx.set_path(_capi.PATH_BATCHED)
        hp, ho = C.c_void_p(), C.c_void_p()
        _capi.check(lib.hostMallocPinnedGpu(C.byref(hp), qe.nbytes))
        _capi.check(lib.hostMallocPinnedGpu(C.byref(ho), 4 * nq))
        C.memmove(hp, qe.ctypes.data, qe.nbytes)

        def e2e_step():
            _capi.check(lib.memcpyGpu(d_qe, hp, qe.nbytes, st))
            _capi.check(lib.upperBoundDeviceGpu(idx.h, d_qe, d_qc, nq, mode, d_out, st))
            _capi.check(lib.memcpyGpu(ho, d_out, 4 * nq, st))
            _capi.check(lib.streamSynchronizeGpu(st))
        for _ in range(max(1, args.warmup)):
            e2e_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        res["e2e_s"] = max_over_ranks((time.perf_counter() - t0) / args.steps, dist)
        res["h2d_bytes"] = qe.nbytes
        res["d2h_bytes"] = 4 * nq
        lib.hostFreePinnedGpu(hp)
        lib.hostFreePinnedGpu(ho)
    for p in (d_qe, d_qc, d_out):
        if p:
            lib.deviceFreeGpu(p)
    idx.close()
    return res


def cpu_run_ub(o, m, wl, seconds, nthreads):
    """The reference's upper_bound (oracle port) over a bounded query sample."""
    qc = wl.q_contig
    probe = min(wl.nq, 200_000)
    t0 = time.perf_counter()
    o.upper_bound_batch(m, wl.q_ends[:probe], None if qc is None else qc[:probe], nthreads=nthreads)
    dt = max(time.perf_counter() - t0, 1e-6)
    k = int(min(wl.nq, max(probe, probe * seconds / dt)))
    t0 = time.perf_counter()
    o.upper_bound_batch(m, wl.q_ends[:k], None if qc is None else qc[:k], nthreads=nthreads)
    dt = time.perf_counter() - t0
    return {"q_per_s": k / dt, "sample_q": k, "seconds": dt}


def ub_line(args, res, world):
    wl, nq, s = res["wl"], res["nq"], res["s_bytes"]
    modes = res["modes"]
    main = modes[args.ub + "+sorted"]
    ms = main["ms_per_step"]
    peak, peak_kind = measured_peak()
    # algorithmic bytes: every query end read and its int32 result written, the starts array
    # read once (the sorted batch reads each block's window of starts once)
    algo = nq * (s + 4) + wl.n * s
    line = {"metric": METRIC_UB, "value": world * nq / (ms / 1e3), "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64" if s == 8 else "int32",
            "data": "synthetic (seeded)",
            "config": dict(workload_desc(args.config, wl), op="upper_bound", upper_bound=args.ub,
                           path="sorted batch (batched path)"),
            "build_s": res["build_s"], "clocks": main["clocks"],
            "providers": {k: {"queries_per_s": nq / (v["ms_per_step"] / 1e3), "ms_per_step": v["ms_per_step"],
                              "prepare_s": v["prepare_s"], "identical_to_binary": v["identical_to_binary"],
                              "path": v["path"]}
                          for k, v in modes.items()},
            "speedup_vs_binary": modes["binary"]["ms_per_step"] / ms,
            "speedup_vs_binary_note": "binary = the reference's halving search, one query per thread in "
                                      "the batch's order; value = the chosen provider on the sorted batch",
            "learned_vs_binary_per_query": modes["binary"]["ms_per_step"] / modes["learned"]["ms_per_step"],
            "oracle_sample_identical": res["oracle_sample_ok"],
            "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (ms / 1e3) / 1e9 / peak, "traffic": None,
                         "kernel": "sorted batch (radix sort + k_qprep + k_ub_scatter)",
                         "peak_kind": peak_kind, "algorithmic_bytes": algo},
            "gpu_launches": main["launches"]}
    line["config"]["inputs"] = "index > L2 (starts array alone 0.8 GB); L2 flushed between steps"
    if "e2e_s" in res:
        line["e2e"] = {"value": world * nq / res["e2e_s"], "unit": "queries/s",
                       "h2d_bytes_per_step": res["h2d_bytes"], "d2h_bytes_per_step": res["d2h_bytes"]}
    if not args.no_cpu:
        nth = host_threads()
        o, m = res["oracle_map"]
        c = cpu_run_ub(o, m, wl, args.cpu_seconds, nth)
        line["cpu_baseline"] = {"value": c["q_per_s"], "unit": "queries/s", "cores": nth, "kind": "port",
                                "sample": f"{c['sample_q']} of {nq} queries, upper_bound, {nth} threads"}
    return line


# ----------------------------------------------------------------------------- operations on the path
def run_gpu_rows(args, op, rank, world, dist):
    """intersection / difference / coverage / search_keys over a device-resident batch of the
    configuration-3 workload (scaled), through the device-buffer C-ABI calls."""
    from superintervals_gb300 import _capi
    from superintervals_gb300.interval_map import GpuIndex
    lib = _capi.load()
    scale = args.scale if args.scale != 1.0 else ROW_DEFAULT_SCALE
    wl = make_workload(args.config, scale, rank)
    s_bytes = wl.dtype.itemsize
    idx = GpuIndex(64 if s_bytes == 8 else 32, local_device())
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg if len(wl.seg) > 2 else None)
    idx.build()
    idx.set_path(_capi.PATH_AUTO)
    idx.set_upper_bound(_capi.UB_LEARNED)
    st = idx.stream
    nq = wl.nq

    def dalloc(nbytes):
        p = C.c_void_p()
        _capi.check(lib.deviceMallocGpu(C.byref(p), max(int(nbytes), 1)))
        return p
    bufs = []

    def upload(a):
        a = np.ascontiguousarray(a)
        p = dalloc(a.nbytes)
        _capi.check(lib.memcpyGpu(p, C.c_void_p(a.ctypes.data), a.nbytes, st))
        bufs.append(p)
        return p
    d_qs, d_qe = upload(wl.q_starts), upload(wl.q_ends)
    d_qc = upload(wl.q_contig) if wl.q_contig is not None else None
    d_off = dalloc(8 * (nq + 1))
    bufs.append(d_off)
    total = C.c_size_t(0)
    out = [None, None, None]

    def call(cap):
        if op == "intersect":
            return lib.intersectDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, 0, d_off, out[0], out[1], out[2], cap,
                                          C.byref(total), st)
        if op == "difference":
            return lib.differenceDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, d_off, out[0], out[1], cap, C.byref(total),
                                           st)
        if op == "keys":
            return lib.searchKeysDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, 1, d_off, out[0], out[1], out[2], cap,
                                           C.byref(total), st)
        if op == "count":
            return lib.countOverlapsDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, out[0], st)
        return lib.coverageDeviceGpu(idx.h, d_qs, d_qe, d_qc, nq, out[0], out[1], st)
    if op == "count":
        out[0] = dalloc(4 * nq)
        P = nq
    elif op == "coverage":
        out[0], out[1] = dalloc(8 * nq), dalloc(s_bytes * nq)
        P = nq
    else:
        r = call(0)
        if r not in (_capi.SI_OK, _capi.SI_ERR_CAPACITY):
            _capi.check(r)
        P = int(total.value)
        out[0], out[1], out[2] = dalloc(s_bytes * max(P, 1)), dalloc(s_bytes * max(P, 1)), dalloc(4 * max(P, 1))
    bufs += [b for b in out if b]
    hits = int(idx.count(wl.q_starts, wl.q_ends, wl.q_contig).astype(np.int64).sum())
    ev = [C.c_void_p(), C.c_void_p()]
    for e in ev:
        _capi.check(lib.eventCreateGpu(C.byref(e)))

    def step():
        _capi.check(call(P))
    for _ in range(args.warmup):
        _capi.check(lib.flushL2Gpu(st))
        step()
    k0 = lib.getLaunchCountGpu()
    total_ms = 0.0
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            _capi.check(lib.flushL2Gpu(st))
            _capi.check(lib.eventRecordGpu(ev[0], st))
            step()
            _capi.check(lib.eventRecordGpu(ev[1], st))
            _capi.check(lib.streamSynchronizeGpu(st))
            ms = C.c_float()
            _capi.check(lib.eventElapsedMsGpu(ev[0], ev[1], C.byref(ms)))
            total_ms += ms.value
    launches = lib.getLaunchCountGpu() - k0
    total_ms = max_over_ranks(total_ms, dist)
    for b in bufs:
        lib.deviceFreeGpu(b)
    idx.close()
    return {"wl": wl, "scale": scale, "nq": nq, "out": P, "hits": hits, "s_bytes": s_bytes,
            "ms_per_step": total_ms / args.steps, "launches": launches, "clocks": clk.summary()}


def rows_algorithmic_bytes(op, Q, H, P, s):
    """Bytes the operation must move: every query read once and, per hit, the hit interval
    read and the output written."""
    if op == "count":
        # the survey's count bytes: query read, count written, one end read per hit
        return Q * (2 * s + 4) + H * s, "Q(2s+4) + H*s"
    if op == "intersect":
        return Q * (2 * s + 8) + H * (2 * s) + P * (2 * s + 4), "Q(2s+8) + H(2s) + P(2s+4)"
    if op == "difference":
        return Q * (2 * s + 8) + H * (2 * s) + P * (2 * s), "Q(2s+8) + H(2s) + P(2s)"
    if op == "keys":
        return Q * (2 * s + 8) + H * (2 * s + 4) * 2, "Q(2s+8) + 2H(2s+4)"
    # coverage comes from ranks and prefix sums (no hit lists) when no interval and no query has
    # start > end: per query, its read and the count and coverage written
    return Q * (3 * s + 12), "Q(3s+12): query read, count and coverage written (no per-hit traffic)"


def rows_cpu(op, wl, seconds, nth):
    """The oracle's restatement of the operation on the host (contig 0's queries)."""
    from oracle.oracle import ORDER_IDXS_CPP, Oracle
    o = Oracle()
    lo, hi = int(wl.seg[0]), int(wl.seg[1])
    m = o.build(wl.starts[lo:hi], wl.ends[lo:hi], wl.data[lo:hi])
    qc = wl.q_contig if wl.q_contig is not None else np.zeros(wl.nq, np.int32)
    sel = np.nonzero(qc == 0)[0]
    qs, qe = wl.q_starts[sel], wl.q_ends[sel]

    def run(k):
        if op == "intersect":
            o.intersection(m, qs[:k], qe[:k], ORDER_IDXS_CPP)
        elif op == "difference":
            o.difference(m, qs[:k], qe[:k])
        elif op == "coverage":
            o.coverage(m, qs[:k], qe[:k])
        elif op == "count":
            o.count_batch(m, qs[:k], qe[:k], nthreads=nth)
        else:
            o.search_batch(m, qs[:k], qe[:k], order=1, values=True, nthreads=nth)
    probe = min(len(sel), 2000)
    t0 = time.perf_counter()
    run(probe)
    dt = max(time.perf_counter() - t0, 1e-6)
    k = int(min(len(sel), max(probe, probe * seconds / dt)))
    t0 = time.perf_counter()
    run(k)
    dt = time.perf_counter() - t0
    threads = nth if op in ("keys", "count") else 1
    return {"q_per_s": k / dt, "sample_q": k, "threads": threads}


def rows_line(args, op, res, world):
    Q, H, P, s = res["nq"], res["hits"], res["out"], res["s_bytes"]
    ms = res["ms_per_step"]
    peak, peak_kind = measured_peak()
    algo, formula = rows_algorithmic_bytes(op, Q, H, 0 if op in ("coverage", "count") else P, s)
    wl = res["wl"]
    line = {"metric": f"{op} queries/s on 1 GB300 (device-resident)", "value": world * Q / (ms / 1e3),
            "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64" if s == 8 else "int32", "data": "synthetic (seeded)",
            "config": dict(workload_desc(args.config, wl), op=op, scale=res["scale"],
                           hits=H, outputs=P if op not in ("coverage", "count") else Q),
            "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (ms / 1e3) / 1e9 / peak, "traffic": None, "peak_kind": peak_kind,
                         "algorithmic_bytes": algo, "formula": formula + " (Q queries, H hits, P outputs)"},
            "gpu_launches": res["launches"], "clocks": res["clocks"]}
    if not args.no_cpu:
        nth = host_threads()
        c = rows_cpu(op, wl, args.cpu_seconds, nth)
        line["cpu_baseline"] = {"value": c["q_per_s"], "unit": "queries/s", "cores": c["threads"], "kind": "port",
                                "sample": f"{c['sample_q']} queries of contig 0, {op}, {c['threads']} thread(s)"}
    return line


def bed_text(wl, seed=5):
    """BED text of the workload's intervals (chrom names of the contig table, half-open ends),
    in a seeded random line order."""
    r = np.random.Generator(np.random.PCG64(seed))
    order = r.permutation(wl.n)
    G = len(wl.seg) - 1
    cid = np.repeat(np.arange(G), np.diff(wl.seg))[order]
    names = np.array([c[0].encode() for c in wl.contigs], dtype=object)
    s = wl.starts[order].astype(np.int64)
    e = wl.ends[order].astype(np.int64) + 1
    cols = [names[cid], np.char.mod(b"%d", s).astype(object), np.char.mod(b"%d", e).astype(object)]
    return b"\n".join(b"\t".join(t) for t in zip(*cols)) + b"\n"


def run_bed(args, rank, world, dist):
    """BED text (pinned host memory) -> GPU parse + contig dictionary + bucketing -> built index."""
    from superintervals_gb300 import _capi
    from superintervals_gb300.interval_map import GpuIndex
    lib = _capi.load()
    scale = args.scale if args.scale != 1.0 else ROW_DEFAULT_SCALE
    wl = make_workload(args.config, scale, rank)
    text = bed_text(wl)
    hp = C.c_void_p()
    _capi.check(lib.hostMallocPinnedGpu(C.byref(hp), len(text)))
    C.memmove(hp, text, len(text))
    idx = GpuIndex(32, local_device())
    stats = _capi.cBedStats()

    def step():
        _capi.check(lib.ingestBedGpu(idx.h, C.cast(hp, C.c_char_p), len(text), _capi.BED_HALF_OPEN,
                                     C.byref(stats)))
        _capi.check(lib.indexSuperIntervalsGpu(idx.h))
    for _ in range(max(1, args.warmup)):
        step()
    k0 = lib.getLaunchCountGpu()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        dt = max_over_ranks((time.perf_counter() - t0) / args.steps, dist)
    res = {"wl": wl, "scale": scale, "bytes": len(text), "intervals": int(stats.intervals), "s": dt,
           "launches": lib.getLaunchCountGpu() - k0, "clocks": clk.summary(), "names": idx.contig_names(),
           "text": text}
    lib.hostFreePinnedGpu(hp)
    idx.close()
    return res


def bed_line(args, res, world):
    from oracle.bed import parse_bed
    wl = res["wl"]
    line = {"metric": "BED intervals ingested + indexed per second on 1 GB300 (text in pinned host memory)",
            "value": world * res["intervals"] / res["s"], "unit": "intervals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * res["s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded)",
            "config": {"workload": f"BED text of {wl.name}", "scale": res["scale"], "text_bytes": res["bytes"],
                       "contigs": len(res["names"]), "op": "ingestBedGpu + indexSuperIntervalsGpu"},
            "text_GB_per_s": res["bytes"] / res["s"] / 1e9, "gpu_launches": res["launches"], "clocks": res["clocks"],
            "e2e": {"value": world * res["intervals"] / res["s"], "unit": "intervals/s",
                    "h2d_bytes_per_step": res["bytes"], "d2h_bytes_per_step": 12 * res["intervals"]}}
    if not args.no_cpu:
        text = res["text"]
        cut = text.find(b"\n", min(len(text) - 1, 8_000_000)) + 1 or len(text)
        t0 = time.perf_counter()
        _, _, st = parse_bed(text[:cut])
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": st["intervals"] / dt, "unit": "intervals/s", "cores": 1, "kind": "port",
                                "sample": f"first {cut} bytes ({st['intervals']} lines) parsed by oracle/bed.py "
                                          "(parse only, no index build)"}
    return line


# ----------------------------------------------------------------------------- serving loop
def serving_workload(args):
    from superintervals_gb300 import workloads as W
    n = max(100_000, int(200_000_000 * args.scale))
    wl = W.config5_index(n=n)
    max_size = max(1000, int(1_000_000 * args.scale))
    nreq = max(20, int(args.requests * min(1.0, 10 * args.scale)))
    arrival, sizes, qc, qs, qe = W.config5_requests(nreq, rate_per_s=args.rate, max_size=max_size)
    return wl, arrival - arrival[0], sizes, qc, qs, qe


def run_serving(args, rank, world, dist):
    """A device-resident index answers a stream of requests.  Requests arrive by a seeded
    Poisson process; the loop takes every request that has arrived (up to a batch cap and
    the free device memory) as one batch through the host-buffer C-ABI call
    (searchBatchIntoGpu: H2D of the queries, count -> scan -> emit, D2H of the CSR result)
    and a request's latency runs from its arrival to its results in host memory."""
    from superintervals_gb300 import _capi
    from superintervals_gb300.interval_map import GpuIndex
    lib = _capi.load()
    wl, arrival, sizes, qc, qs, qe = serving_workload(args)
    idx = GpuIndex(32, local_device())
    idx.add_arrays(wl.starts, wl.ends, wl.data, seg=wl.seg)
    t0 = time.perf_counter()
    idx.build()
    build_s = time.perf_counter() - t0
    nreq = len(sizes)
    roff = np.zeros(nreq + 1, np.int64)
    np.cumsum(sizes, out=roff[1:])
    nq_all = int(roff[-1])

    def pinned(nbytes):
        p = C.c_void_p()
        _capi.check(lib.hostMallocPinnedGpu(C.byref(p), max(int(nbytes), 1)))
        return p
    hq = [pinned(a.nbytes) for a in (qs, qe, qc)]
    for p, a in zip(hq, (qs, qe, qc)):
        C.memmove(p, a.ctypes.data, a.nbytes)
    max_batch = max(1_000_000, int(8_000_000 * min(1.0, 10 * args.scale)))
    h_off = pinned(8 * (max_batch + 1 + int(sizes.max())))
    cap = [max(1 << 20, 120 * max_batch)]
    h_out = [pinned(4 * cap[0])]
    idx.set_output_budget(16 << 30)
    free_b, tot_b = C.c_size_t(0), C.c_size_t(0)
    total = C.c_size_t(0)

    def serve(path, ub, saturate):
        idx.set_path(path)
        idx.set_upper_bound(ub)
        lat = np.zeros(nreq)
        pairs = 0
        hits_per_q = 100.0
        batches = 0
        k0 = lib.getLaunchCountGpu()
        start = time.perf_counter()
        r = 0
        while r < nreq:
            now = time.perf_counter() - start
            if not saturate and arrival[r] > now:
                time.sleep(min(arrival[r] - now, 0.0005))
                continue
            # admission: arrived requests, at most max_batch queries, and no more than half of
            # the free device memory at the current hits-per-query estimate
            _capi.check(lib.deviceMemInfoGpu(local_device(), C.byref(free_b), C.byref(tot_b)))
            per_q = 48 + 4 * hits_per_q
            room = min(max_batch, int(0.5 * free_b.value / per_q))
            r1 = r + 1
            while r1 < nreq and (saturate or arrival[r1] <= now) and roff[r1 + 1] - roff[r] <= room:
                r1 += 1
            q0, nq = int(roff[r]), int(roff[r1] - roff[r])
            args_ = [idx.h] + [C.c_void_p(p.value + a.itemsize * q0) for p, a in zip(hq, (qs, qe, qc))] + \
                    [nq, 0, 0, h_off]
            st = lib.searchBatchIntoGpu(*args_, h_out[0], cap[0], C.byref(total))
            if st == _capi.SI_ERR_CAPACITY:
                lib.hostFreePinnedGpu(h_out[0])
                cap[0] = int(total.value * 1.25) + 1
                h_out[0] = pinned(4 * cap[0])
                st = lib.searchBatchIntoGpu(*args_, h_out[0], cap[0], C.byref(total))
            _capi.check(st)
            done = time.perf_counter() - start
            lat[r:r1] = done - (0.0 if saturate else arrival[r:r1])
            pairs += int(total.value)
            hits_per_q = max(1.0, 0.8 * hits_per_q + 0.2 * total.value / max(nq, 1))
            batches += 1
            r = r1
        wall = time.perf_counter() - start
        return {"queries_per_s": nq_all / wall, "pairs_per_s": pairs / wall, "wall_s": wall, "batches": batches,
                "p50_ms": 1e3 * float(np.percentile(lat, 50)), "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                "launches": lib.getLaunchCountGpu() - k0, "pairs": pairs}

    res = {"wl": wl, "build_s": build_s, "nreq": nreq, "nq": nq_all, "sizes": sizes, "qs": qs, "qe": qe, "qc": qc}
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        # the library picks the batched path for batches of 4096+ queries and the plain one below
        serve(_capi.PATH_AUTO, _capi.UB_LEARNED, True)               # warm-up
        res["batched_sat"] = serve(_capi.PATH_AUTO, _capi.UB_LEARNED, True)
        res["batched_rate"] = serve(_capi.PATH_AUTO, _capi.UB_LEARNED, False)
    res["clocks"] = clk.summary()
    if not args.no_plain:
        res["plain_sat"] = serve(_capi.PATH_PLAIN, _capi.UB_BINARY, True)
        res["plain_rate"] = serve(_capi.PATH_PLAIN, _capi.UB_BINARY, False)
    for p in hq + [h_off, h_out[0]]:
        lib.hostFreePinnedGpu(p)
    idx.close()
    return res


def serving_line(args, res, world):
    b, br = res["batched_sat"], res["batched_rate"]
    wl = res["wl"]
    line = {"metric": METRIC_SERVE, "value": world * b["queries_per_s"], "unit": "queries/s", "n_gpus": world,
            "steps": res["nreq"], "warmup": 1, "ms_per_step": 1e3 * b["wall_s"] / res["nreq"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (seeded)",
            "config": {"workload": f"serving n={wl.n} int32 24 contigs, {res['nreq']} Poisson requests "
                                   f"({res['nq']} queries, sizes log-uniform), offered {args.rate}/s",
                       "n_intervals": wl.n, "requests": res["nreq"], "queries": res["nq"],
                       "op": "search_idxs (C++ order) per request batch",
                       "path": "auto (batched for 4096+ queries, else plain) + learned upper bound",
                       "inputs": "queries from pinned host memory; results to pinned host memory"},
            "latency_ms": {"offered_rate_per_s": args.rate, "p50": br["p50_ms"], "p99": br["p99_ms"],
                           "queries_per_s": br["queries_per_s"], "batches": br["batches"]},
            "saturated": {"p50_ms": b["p50_ms"], "p99_ms": b["p99_ms"], "batches": b["batches"],
                          "pairs_per_s": b["pairs_per_s"]},
            "build_s": res["build_s"], "clocks": res["clocks"], "gpu_launches": b["launches"],
            "e2e": {"value": world * b["queries_per_s"], "unit": "queries/s",
                    "h2d_bytes_per_step": int(12 * res["nq"] / max(b["batches"], 1)),
                    "d2h_bytes_per_step": int((8 * res["nq"] + 4 * b["pairs"]) / max(b["batches"], 1))}}
    if "plain_sat" in res:
        p, pr = res["plain_sat"], res["plain_rate"]
        line["plain_gpu"] = {"queries_per_s": p["queries_per_s"], "p50_ms": pr["p50_ms"], "p99_ms": pr["p99_ms"],
                             "saturated_speedup": b["queries_per_s"] / p["queries_per_s"]}
    if not args.no_cpu:
        nth = host_threads()
        c = serving_cpu(wl, res["qs"], res["qe"], res["qc"], args.cpu_seconds, nth)
        line["cpu_baseline"] = {"value": c["q_per_s"], "unit": "queries/s", "cores": nth, "kind": "port",
                                "sample": c["sample"]}
    return line


def serving_cpu(wl, qs, qe, qc, seconds, nth):
    """The oracle port over the three smallest contigs of the resident index and the stream's
    queries on them (building the whole 200 M-interval index on the host takes minutes)."""
    from superintervals_gb300.workloads import Workload
    G = len(wl.seg) - 1
    lens = np.array([c[1] for c in wl.contigs])
    pick = np.sort(np.argsort(lens)[:3])
    parts = [np.arange(wl.seg[g], wl.seg[g + 1]) for g in pick]
    sel = np.concatenate(parts)
    seg = np.zeros(len(pick) + 1, np.int64)
    seg[1:] = np.cumsum([len(x) for x in parts])
    remap = np.full(G, -1, np.int32)
    remap[pick] = np.arange(len(pick), dtype=np.int32)
    qmask = remap[qc] >= 0
    sub = Workload(name="serving sample", starts=wl.starts[sel], ends=wl.ends[sel], data=wl.data[sel], seg=seg,
                   q_starts=qs[qmask][:2_000_000], q_ends=qe[qmask][:2_000_000],
                   q_contig=remap[qc[qmask]][:2_000_000], contigs=[wl.contigs[g] for g in pick])
    c = cpu_run(sub, seconds, nth, single=False)
    c["sample"] = (f"{c['sample_q']} queries of the request stream on {len(pick)} contigs "
                   f"({len(sel)} intervals), search_idxs C++ order ({c['pairs']} pairs), {nth} threads")
    return c


# ----------------------------------------------------------------------------- CPU arm
PARITY_QUERIES = 1 << 20   # headline queries whose GPU result is compared with the oracle's


def cpu_run(wl, seconds, nthreads, keep=0, single=True):
    """The reference algorithm (oracle port, oracle/si_oracle.c, pinned bit-exactly to the
    reference's outputs) on the host cores: search_idxs in the C++ order over a bounded
    prefix of the batch, one walk per query appending to per-chunk buffers and then copied
    into one CSR result (the form the reference's per-query search_idxs takes,
    superintervals.hpp:879-905).  The sample is sized to about `seconds` of work and holds at
    least the first `keep` queries, whose CSR is returned for the parity check.  With
    `single`, the same is also timed on one thread over a smaller prefix."""
    from oracle.oracle import ORDER_IDXS_CPP, Oracle
    o = Oracle()
    m = o.build(wl.starts, wl.ends, wl.data, seg=wl.seg)

    def qslice(k):
        qc = None if wl.q_contig is None else wl.q_contig[:k]
        return wl.q_starts[:k], wl.q_ends[:k], qc

    probe = min(wl.nq, 20_000)
    t0 = time.perf_counter()
    o.search_lists(m, *qslice(probe), order=ORDER_IDXS_CPP, nthreads=nthreads)
    dt = max(time.perf_counter() - t0, 1e-6)
    k = int(min(wl.nq, max(probe, keep, probe * seconds / dt)))
    t0 = time.perf_counter()
    off, out = o.search_lists(m, *qslice(k), order=ORDER_IDXS_CPP, nthreads=nthreads)
    dt = time.perf_counter() - t0
    res = {"q_per_s": k / dt, "pairs_per_s": float(off[-1]) / dt, "sample_q": k, "seconds": dt,
           "pairs": int(off[-1])}
    if keep:
        kk = min(keep, k)
        res["kept"] = (off[:kk + 1].copy(), out[:int(off[kk])].copy())
    del off, out
    if single:
        # one thread at about the per-thread rate just measured, for a quarter of `seconds`
        k1 = int(min(k, max(probe, k / dt / max(nthreads, 1) * seconds / 4)))
        t0 = time.perf_counter()
        o1, _ = o.search_lists(m, *qslice(k1), order=ORDER_IDXS_CPP, nthreads=1)
        d1 = time.perf_counter() - t0
        res["single_thread"] = {"q_per_s": k1 / d1, "pairs_per_s": float(o1[-1]) / d1, "sample_q": k1}
    return res


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------- main
def init_dist(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, world, dist
    return rank, world, None


def main():
    args = parse()
    rank, world, dist = init_dist(args)
    cfg = args.config
    op = args.op or ("upper_bound" if cfg == "config4" else "search_idxs")
    if args.impl == "reference" and op in ROW_OPS:
        if rank != 0:
            return
        scale = args.scale if args.scale != 1.0 else ROW_DEFAULT_SCALE
        wl = make_workload(cfg, scale, 0)
        nth = host_threads()
        if op == "bed_ingest":
            from oracle.bed import parse_bed
            text = bed_text(wl)
            cut = text.find(b"\n", min(len(text) - 1, 8_000_000)) + 1 or len(text)
            t0 = time.perf_counter()
            _, _, stt = parse_bed(text[:cut])
            dt = time.perf_counter() - t0
            val, unit, cores = stt["intervals"] / dt, "intervals/s", 1
            sample = f"first {cut} bytes parsed by oracle/bed.py"
        else:
            c = rows_cpu(op, wl, args.cpu_seconds, nth)
            val, unit, cores = c["q_per_s"], "queries/s", c["threads"]
            sample = f"{c['sample_q']} queries of contig 0, {op}"
            dt = c["sample_q"] / max(val, 1e-9)
        line = {"metric": f"{op} on the host (reference algorithm)", "value": val, "unit": unit,
                "impl": "reference", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * dt,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": str(wl.dtype),
                "data": "synthetic (seeded)", "config": dict(workload_desc(cfg, wl), op=op, scale=scale),
                "cpu_baseline": {"value": val, "unit": unit, "cores": cores, "kind": "port", "sample": sample},
                "e2e": {"value": val, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.impl == "reference" and cfg == "config5":
        if rank != 0:
            return
        wl, arrival, sizes, qc, qs, qe = serving_workload(args)
        nth = host_threads()
        runs = [serving_cpu(wl, qs, qe, qc, args.cpu_seconds / max(1, args.steps), nth) for _ in range(args.steps)]
        qps = statistics.median(r["q_per_s"] for r in runs)
        line = {"metric": METRIC_SERVE, "value": qps, "unit": "queries/s", "impl": "reference", "n_gpus": 1,
                "steps": args.steps, "warmup": 0,
                "ms_per_step": 1000.0 * statistics.median(r["seconds"] for r in runs),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
                "data": "synthetic (seeded)",
                "config": {"workload": f"serving n={wl.n} int32 24 contigs", "op": "search_idxs (C++ order)"},
                "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": nth, "kind": "port",
                                 "sample": runs[0]["sample"]},
                "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.impl == "reference" and op == "upper_bound":
        if rank != 0:
            return
        from oracle.oracle import Oracle
        wl = make_workload(cfg, args.scale, 0)
        nth = host_threads()
        o = Oracle()
        m = o.build(wl.starts, wl.ends, wl.data, seg=wl.seg)
        for _ in range(max(0, min(args.warmup, 1))):
            cpu_run_ub(o, m, wl, min(2.0, args.cpu_seconds / 4), nth)
        runs = [cpu_run_ub(o, m, wl, args.cpu_seconds / max(1, args.steps), nth) for _ in range(args.steps)]
        qps = statistics.median(r["q_per_s"] for r in runs)
        line = {"metric": METRIC_UB, "value": qps, "unit": "queries/s", "impl": "reference", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 * statistics.median(r["seconds"] for r in runs),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": str(wl.dtype),
                "data": "synthetic (seeded)",
                "config": dict(workload_desc(cfg, wl), op="upper_bound", upper_bound="binary (reference)"),
                "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": nth, "kind": "port",
                                 "sample": f"{runs[0]['sample_q']} of {wl.nq} queries per step, "
                                           f"upper_bound, {nth} threads"},
                "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    if args.impl == "reference":
        if rank != 0:
            return
        wl = make_workload(cfg, args.scale, 0)
        nth = host_threads()
        for _ in range(max(0, min(args.warmup, 1))):
            cpu_run(wl, min(2.0, args.cpu_seconds / 4), nth, single=False)
        runs = [cpu_run(wl, args.cpu_seconds / max(1, args.steps), nth, single=(i == 0))
                for i in range(args.steps)]
        qps = statistics.median(r["q_per_s"] for r in runs)
        pps = statistics.median(r["pairs_per_s"] for r in runs)
        sample = (f"first {runs[0]['sample_q']} of {wl.nq} queries per step "
                  f"({runs[0]['pairs']} result pairs), search_idxs C++ order, {nth} threads, "
                  "one walk per query")
        line = {"metric": METRIC, "value": qps, "unit": "queries/s", "impl": "reference",
                "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1000.0 * statistics.median(r["seconds"] for r in runs),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": str(wl.dtype),
                "data": "synthetic (seeded)", "config": workload_desc(cfg, wl),
                "pairs_per_s": pps,
                "cpu_baseline": {"value": qps, "unit": "queries/s", "cores": nth, "kind": "port",
                                 "sample": sample,
                                 "single_thread": {"value": runs[0]["single_thread"]["q_per_s"],
                                                   "pairs_per_s": runs[0]["single_thread"]["pairs_per_s"],
                                                   "sample": f"first {runs[0]['single_thread']['sample_q']} "
                                                             "queries, 1 thread"}},
                "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0},
                "note": "reference algorithm restated in C (oracle/si_oracle.c, pinned to the "
                        "reference's own outputs; 1.06x the reference header's speed on one x86 "
                        "thread, profiles/cpu_port_vs_reference.md); the reference header cannot be "
                        "compiled on this host: its sources are not present here"}
        print(json.dumps(line), flush=True)
        return

    if cfg == "config5":
        res = run_serving(args, rank, world, dist)
        if rank == 0:
            print(json.dumps(serving_line(args, res, world)), flush=True)
        return
    if op == "bed_ingest":
        res = run_bed(args, rank, world, dist)
        if rank == 0:
            print(json.dumps(bed_line(args, res, world)), flush=True)
        return
    if op in ROW_OPS:
        res = run_gpu_rows(args, op, rank, world, dist)
        if rank == 0:
            print(json.dumps(rows_line(args, op, res, world)), flush=True)
        return
    if op == "upper_bound":
        res = run_gpu_ub(args, rank, world, dist)
        if rank == 0:
            print(json.dumps(ub_line(args, res, world)), flush=True)
        return
    res = run_gpu(args, rank, world, dist)
    if rank != 0:
        return
    wl, P, nq = res["wl"], res["P"], res["nq"]
    s = res["s_bytes"]
    ms = res["ms_per_step"]
    qps = world * nq / (ms / 1000.0)
    pps = world * P / (ms / 1000.0)
    peak, peak_kind = measured_peak()
    line = {"metric": METRIC, "value": qps, "unit": "queries/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32" if s == 4 else "int64", "data": "synthetic (seeded)",
            "config": dict(workload_desc(cfg, wl), path=args.path, upper_bound=args.ub,
                           autotuned=res.get("tuned")),
            "pairs_per_s": pps, "result_pairs_per_step": P,
            "build_s": res["build_s"], "clocks": res["clocks"]}
    if args.profile_only:
        print(json.dumps(line), flush=True)
        return
    # roofline of the dominant kernel (emit) with the algorithmic bytes
    # B = Q*(2s+8) + P*(s+4): query read, offset read, one end read and one index
    # write per result pair
    ph = res.get("phase_ms", [0, 0, 0, 0])
    emit_ms = ph[2] if ph[2] > 0 else ms
    algo = nq * (2 * s + 8) + P * (s + 4)
    achieved = algo / (emit_ms / 1000.0) / 1e9
    traffic = (EMIT_DRAM_WRITE_PER_PAIR * P + EMIT_DRAM_READ_PER_QUERY * nq
               if cfg == "config3" and args.path == "batched" else None)
    line["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic, "kernel": "emit",
                        "traffic_source": "per-unit DRAM bytes of profiles/k_tiles_config3_dram.md x this run's "
                                          "P and Q" if traffic else None,
                        "traffic_frac": (traffic / (emit_ms / 1000.0) / 1e9 / peak) if traffic else None,
                        "peak_kind": peak_kind, "algorithmic_bytes": algo,
                        "phase_ms": {"count": ph[0], "scan": ph[1], "emit": ph[2], "prepare": ph[3]},
                        "emit_ms_by_mode": res.get("emit_mode_ms"),
                        "whole_step_frac": (algo / (ms / 1000.0) / 1e9) / peak}
    line["gpu_launches"] = res["launches"]
    if "single_query_us" in res:
        line["single_query_latency_us"] = dict(res["single_query_us"],
                                               note="one-query calls through the host-buffer C-ABI "
                                                    "(the drop-in's per-query methods), median of 200")
    if "plain_ms" in res:
        line["plain_gpu"] = {"ms_per_step": res["plain_ms"], "queries_per_s": nq / (res["plain_ms"] / 1e3),
                             "speedup_vs_plain": res["plain_ms"] / ms}
    if "e2e_s" in res:
        line["e2e"] = {"value": world * nq / res["e2e_s"], "unit": "queries/s",
                       "h2d_bytes_per_step": res["h2d_bytes"], "d2h_bytes_per_step": res["d2h_bytes"],
                       "pairs_per_s": world * P / res["e2e_s"], "d2h_link_GBps": res.get("d2h_link_GBps"),
                       "ms_per_step": 1e3 * res["e2e_s"], "result_chunks": res.get("e2e_chunks")}
    if not args.no_cpu:
        nth = host_threads()
        keep = len(res["gpu_prefix"][0]) - 1 if "gpu_prefix" in res else 0
        c = cpu_run(wl, args.cpu_seconds, nth, keep=keep)
        line["cpu_baseline"] = {"value": c["q_per_s"], "unit": "queries/s", "cores": nth, "kind": "port",
                                "sample": f"first {c['sample_q']} of {nq} queries, search_idxs C++ order "
                                          f"({c['pairs']} pairs), {nth} threads; oracle/si_oracle.c "
                                          "one walk per query (1.06x the reference header's speed on "
                                          "one x86 thread, profiles/cpu_port_vs_reference.md)",
                                "pairs_per_s": c["pairs_per_s"]}
        if "single_thread" in c:
            st1 = c["single_thread"]
            line["cpu_baseline"]["single_thread"] = {"value": st1["q_per_s"], "pairs_per_s": st1["pairs_per_s"],
                                                     "sample": f"first {st1['sample_q']} queries, 1 thread"}
        if "gpu_prefix" in res and "kept" in c:
            g_off, g_val = res.pop("gpu_prefix")
            o_off, o_val = c.pop("kept")
            k = min(len(g_off), len(o_off)) - 1
            ok = bool(np.array_equal(g_off[:k + 1], o_off[:k + 1]) and
                      np.array_equal(g_val[:int(g_off[k])], o_val[:int(o_off[k])]))
            line["parity_sample_ok"] = ok
            line["parity_sample"] = (f"the timed step's CSR result for the first {k} queries "
                                     f"({int(o_off[k])} pairs) against the oracle, bit for bit")
            if not ok:
                print(json.dumps(line), flush=True)
                raise SystemExit("parity check failed: the GPU result differs from the oracle's")
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
