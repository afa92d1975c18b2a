// si_query.cu -- the PLAIN query path: one thread per query.
//
// Each thread runs the reference's own per-query algorithm:
//   upper_bound (src/superintervals.hpp:501-516): branch-free halving search for
//     the last k with starts[k] <= qe;
//   then the backward walk (hpp:551-579 / 623-649 / 879-905): while
//     ends[i] >= qs report i and step to i-1, otherwise jump to branch[i].
// count -> exclusive scan -> emit gives exact per-query CSR offsets.  The emit
// order follows the reference exactly:
//   kOrderIdxsCpp  C++ search_idxs (hpp:879-905): the head run i0+1..idx is
//                  written ASCENDING, the rest of the walk descending;
//   kOrderDesc     search_values (hpp:551-579) and the C API searchIdxs
//                  (c_superintervals.h:610-643): fully descending.
// This path is the 1.0x GPU baseline that the batched path is measured against.
#include <algorithm>
#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
// batches up to this many queries take one warp per query (lower latency per query); larger ones
// one thread per query (more queries in flight per warp)
constexpr int64_t kWarpQueries = 32768;

// last k in [0, n) with starts[k] <= v, else -1 (hpp:501-516)
template <typename S>
__device__ __forceinline__ int64_t ub_halving(const S* __restrict__ starts, int64_t n, S v) {
    int64_t length = n, idx = 0;
    while (length > 1) {
        const int64_t half = length >> 1;
        idx += (starts[idx + half] <= v) ? (length - half) : 0;
        length = half;
    }
    return (starts[idx] > v) ? idx - 1 : idx;
}

// Resolve the contig of query q: [lo, lo+len) in the concatenated arrays.
template <typename S>
__device__ __forceinline__ bool query_range(const MapView<S>& m, const int32_t* qc, int64_t q,
                                            int64_t& lo, int64_t& len, int* d_err) {
    int32_t g = qc ? qc[q] : 0;
    if (g < 0 || g >= m.G) {
        if (d_err) atomicCAS(d_err, kDevOk, kDevBadContig);
        return false;
    }
    lo = m.seg[g];
    len = m.seg[g + 1] - lo;
    return len > 0;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_count_plain(MapView<S> m, const S* __restrict__ qs,
                                                          const S* __restrict__ qe,
                                                          const int32_t* __restrict__ qc,
                                                          int64_t nq, uint32_t* __restrict__ counts,
                                                          int* d_err) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int64_t lo, len;
    uint32_t c = 0;
    if (query_range(m, qc, q, lo, len, d_err)) {
        const S s = qs[q];
        const int64_t u = ub_halving(m.starts + lo, len, qe[q]);
        if (u >= 0) {
            int64_t i = lo + u;
            const int64_t top = i;
            while (i >= lo && s <= m.ends[i]) --i;
            c = (uint32_t)(top - i);
            if (i >= lo) {
                i = m.branch[i];
                while (i >= 0) {
                    if (s <= m.ends[i]) {
                        ++c;
                        --i;
                        if (i < lo) break;
                    } else {
                        i = m.branch[i];
                    }
                }
            }
        }
    }
    counts[q] = c;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_emit_plain(MapView<S> m, const S* __restrict__ qs,
                                                         const S* __restrict__ qe,
                                                         const int32_t* __restrict__ qc,
                                                         int64_t nq,
                                                         const int64_t* __restrict__ offsets,
                                                         int64_t out_base, int order, bool values,
                                                         int32_t* __restrict__ out, int* d_err,
                                                         int64_t total_cap) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int64_t lo, len;
    if (!query_range(m, qc, q, lo, len, nullptr)) return;
    const S s = qs[q];
    const int64_t u = ub_halving(m.starts + lo, len, qe[q]);
    if (u < 0) return;
    if (offsets[q + 1] - out_base > total_cap) {  // the caller's buffer ends before this query's list
        atomicCAS(d_err, kDevOk, kDevOverflow);
        return;
    }
    int32_t* dst = out + (offsets[q] - out_base);
    const int64_t cap = offsets[q + 1] - offsets[q];
    int64_t w = 0;
    int64_t i = lo + u;
    const int64_t top = i;
    while (i >= lo && s <= m.ends[i]) --i;
    const int64_t h = top - i;
    if (h > cap) {
        atomicCAS(d_err, kDevOk, kDevOverflow);
        return;
    }
    if (order == kOrderIdxsCpp) {
        for (int64_t k = i + 1; k <= top; ++k) dst[w++] = values ? m.data[k] : (int32_t)(k - lo);
    } else {
        for (int64_t k = top; k > i; --k) dst[w++] = values ? m.data[k] : (int32_t)(k - lo);
    }
    if (i < lo) return;
    i = m.branch[i];
    while (i >= 0) {
        if (s <= m.ends[i]) {
            if (w >= cap) {
                atomicCAS(d_err, kDevOk, kDevOverflow);
                return;
            }
            dst[w++] = values ? m.data[i] : (int32_t)(i - lo);
            --i;
            if (i < lo) break;
        } else {
            i = m.branch[i];
        }
    }
}

// ---- one WARP per query: small batches, where latency matters more than throughput -----------
// The same results as the thread-per-query kernels above, with the scans done 32 positions at a
// time (the GPU form of the reference's block count, hpp:651-825: a ballot over 32 ends against
// qs and a popcount in place of the SIMD compare and lane sum).

// Entries of the ascending arr[a, b) that are <= key (strict: < key): a 32-ary search, one
// round trip per step (32 probes, one per lane, and a ballot).
template <typename S>
__device__ __forceinline__ int64_t warp_rank(const S* __restrict__ arr, int64_t a, int64_t b, S key, bool strict,
                                             int lane) {
    const int64_t a0 = a;
    while (b - a > 32) {
        const int64_t step = (b - a + 31) >> 5;
        const int64_t p = a + (int64_t)(lane + 1) * step - 1;
        bool in = false;
        if (p < b) {
            const S x = arr[p];
            in = strict ? (x < key) : (x <= key);
        }
        a += (int64_t)__popc(__ballot_sync(kFull, in)) * step;  // probes below the answer: a prefix
        b = b < a + step ? b : a + step;
    }
    bool in = false;
    if (a + lane < b) {
        const S x = arr[a + lane];
        in = strict ? (x < key) : (x <= key);
    }
    return a + __popc(__ballot_sync(kFull, in)) - a0;
}

// From a miss at p the walk goes on at branch[p] (hpp:551-579): every position strictly between
// branch[p] and p ends before ends[p] < qs.  For a 32-position chunk ending at i (lane l is position i - l), the
// next position to look at: below the chunk, and below the branch of every miss in it (each
// miss's skipped range reaches into the chunk, so together they cover everything from the
// smallest branch up).  br is the lane's branch entry, loaded beside its end.
__device__ __forceinline__ int64_t warp_next(int64_t i, bool miss, int32_t br) {
    const int b = __reduce_min_sync(kFull, miss ? br : INT32_MAX);
    return (int64_t)b < i - 32 ? (int64_t)b : i - 32;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_count_warp(MapView<S> m, const S* __restrict__ qs,
                                                         const S* __restrict__ qe,
                                                         const int32_t* __restrict__ qc, int64_t nq,
                                                         uint32_t* __restrict__ counts, int* d_err) {
    const int lane = threadIdx.x & 31;
    const int64_t q = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    if (q >= nq) return;  // whole warps
    int64_t lo, len;
    uint32_t c = 0;
    if (query_range(m, qc, q, lo, len, lane == 0 ? d_err : nullptr)) {
        const S s = qs[q], e = qe[q];
        const int64_t nle = warp_rank(m.starts, lo, lo + len, e, false, lane);  // upper bound + 1
        if (nle > 0) {
            if (m.end_sorted && s <= e) {
                // no interval has start > end: an interval ending before qs starts before qe, so
                // count = #(start <= qe) - #(end < qs)
                const int64_t below = warp_rank(m.end_sorted, lo, lo + len, s, true, lane);
                c = nle > below ? (uint32_t)(nle - below) : 0u;
            } else {
                int64_t i = lo + nle - 1;
                while (i >= lo) {
                    const int64_t k = i - lane;
                    const bool valid = k >= lo;
                    S e_k = 0;
                    int32_t br = 0;
                    if (valid) {
                        e_k = m.ends[k];
                        br = m.branch[k];
                    }
                    const bool hit = valid && s <= e_k;
                    c += (uint32_t)__popc(__ballot_sync(kFull, hit));
                    i = warp_next(i, valid && !hit, br);
                }
            }
        }
    }
    if (lane == 0) counts[q] = c;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_emit_warp(MapView<S> m, const S* __restrict__ qs,
                                                        const S* __restrict__ qe,
                                                        const int32_t* __restrict__ qc, int64_t nq,
                                                        const int64_t* __restrict__ offsets, int64_t out_base,
                                                        int order, bool values, int32_t* __restrict__ out,
                                                        int* d_err, int64_t total_cap) {
    const int lane = threadIdx.x & 31;
    const int64_t q = ((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5;
    if (q >= nq) return;
    int64_t lo, len;
    if (!query_range(m, qc, q, lo, len, nullptr)) return;
    const S s = qs[q], e = qe[q];
    const int64_t nle = warp_rank(m.starts, lo, lo + len, e, false, lane);
    if (nle == 0) return;
    if (offsets[q + 1] - out_base > total_cap) {  // the caller's buffer ends before this query's list
        if (lane == 0) atomicCAS(d_err, kDevOk, kDevOverflow);
        return;
    }
    int32_t* dst = out + (offsets[q] - out_base);
    const int64_t cap = offsets[q + 1] - offsets[q];
    const int64_t top = lo + nle - 1;
    // the head run: positions top, top - 1, ... that hit, found 32 at a time
    int64_t h = 0;
    while (true) {
        const int64_t k = top - h - lane;
        const unsigned stop = __ballot_sync(kFull, !(k >= lo && s <= m.ends[k]));
        if (stop) {
            h += __ffs(stop) - 1;
            break;
        }
        h += 32;
    }
    if (h > cap) {
        if (lane == 0) atomicCAS(d_err, kDevOk, kDevOverflow);
        return;
    }
    // ascending for the C++ search_idxs (hpp:892-895), else descending
    for (int64_t r = lane; r < h; r += 32) {
        const int64_t pos = (order == kOrderIdxsCpp) ? (top - h + 1 + r) : (top - r);
        dst[r] = values ? m.data[pos] : (int32_t)(pos - lo);
    }
    const int64_t p = top - h;  // a miss, or before the contig
    if (p < lo) return;
    int64_t w = h;
    int64_t i = m.branch[p];
    const unsigned lt = (1u << lane) - 1u;
    while (i >= lo) {
        const int64_t k = i - lane;
        const bool valid = k >= lo;
        S e_k = 0;
        int32_t br = 0;
        if (valid) {
            e_k = m.ends[k];
            br = m.branch[k];
        }
        const bool hit = valid && s <= e_k;
        const unsigned hm = __ballot_sync(kFull, hit);
        if (w + __popc(hm) > cap) {
            if (lane == 0) atomicCAS(d_err, kDevOk, kDevOverflow);
            return;
        }
        if (hit) dst[w + __popc(hm & lt)] = values ? m.data[k] : (int32_t)(k - lo);
        w += __popc(hm);
        i = warp_next(i, valid && !hit, br);
    }
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_any_plain(MapView<S> m, const S* __restrict__ qs,
                                                        const S* __restrict__ qe,
                                                        const int32_t* __restrict__ qc, int64_t nq,
                                                        uint8_t* __restrict__ out, int* d_err) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int64_t lo, len;
    uint8_t r = 0;
    if (query_range(m, qc, q, lo, len, d_err)) {
        // has_overlaps (hpp:865-871) inspects the interval at upper_bound(qe) only
        const int64_t u = ub_halving(m.starts + lo, len, qe[q]);
        r = (u >= 0 && qs[q] <= m.ends[lo + u]) ? 1 : 0;
    }
    out[q] = r;
}

inline unsigned blocks_for(int64_t n) {
    return (unsigned)std::max<int64_t>(1, ceil_div(n, kThreads));
}

__global__ void k_check_contigs(const int32_t* __restrict__ qc, int64_t nq, int G, int* d_err) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q < nq && (qc[q] < 0 || qc[q] >= G)) atomicCAS(d_err, kDevOk, kDevBadContig);
}

}  // namespace

cudaError_t launch_check_contigs(const int32_t* qc, int64_t nq, int G, int* d_err, cudaStream_t st) {
    if (!qc || nq <= 0) return cudaSuccess;
    k_check_contigs<<<blocks_for(nq), kThreads, 0, st>>>(qc, nq, G, d_err);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_count_plain(MapView<S> m, QueryBatch q, uint32_t* counts, int* d_err,
                               cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    if (q.nq <= kWarpQueries)
        k_count_warp<S><<<blocks_for(q.nq * 32), kThreads, 0, st>>>(
            m, static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, q.nq, counts, d_err);
    else
        k_count_plain<S><<<blocks_for(q.nq), kThreads, 0, st>>>(
            m, static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, q.nq, counts, d_err);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_emit_plain(MapView<S> m, QueryBatch q, const int64_t* offsets, int64_t out_base,
                              int order, bool values, int32_t* out, int* d_err, cudaStream_t st,
                              int64_t total_cap) {
    if (q.nq <= 0) return cudaSuccess;
    if (q.nq <= kWarpQueries)
        k_emit_warp<S><<<blocks_for(q.nq * 32), kThreads, 0, st>>>(
            m, static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, q.nq, offsets, out_base,
            order, values, out, d_err, total_cap);
    else
        k_emit_plain<S><<<blocks_for(q.nq), kThreads, 0, st>>>(
            m, static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, q.nq, offsets, out_base,
            order, values, out, d_err, total_cap);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_any_plain(MapView<S> m, QueryBatch q, uint8_t* out, int* d_err,
                             cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    k_any_plain<S><<<blocks_for(q.nq), kThreads, 0, st>>>(
        m, static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, q.nq, out, d_err);
    note_launch();
    return cudaGetLastError();
}

#define SIG_QINST(S)                                                                              \
    template cudaError_t launch_count_plain<S>(MapView<S>, QueryBatch, uint32_t*, int*,          \
                                               cudaStream_t);                                   \
    template cudaError_t launch_emit_plain<S>(MapView<S>, QueryBatch, const int64_t*, int64_t,   \
                                              int, bool, int32_t*, int*, cudaStream_t, int64_t); \
    template cudaError_t launch_any_plain<S>(MapView<S>, QueryBatch, uint8_t*, int*, cudaStream_t);
SIG_QINST(int32_t)
SIG_QINST(int64_t)

}  // namespace sig
