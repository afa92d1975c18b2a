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
