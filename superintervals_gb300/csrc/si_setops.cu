// si_setops.cu -- operations over the hit lists of the search path (CSR of contig-local
// positions): batch set operations of a list of intervals (map A, given as queries) against the
// index (map B), key gathers and coverage.
//
//   intersection (src/superintervals.hpp:1158-1177, src/c_superintervals.h:921-940): for query
//     interval [qs, qe] and each hit h in the search order, the piece
//     [max(qs, starts[h]), min(qe, ends[h])], kept when start <= end.
//   difference (hpp:1186-1211, c:951-974): the hits' (start, end) keys sorted ascending and
//     swept with a cursor from qs; every uncovered piece [cursor, cs - 1] and the trailing
//     [cursor, qe] are emitted.
//
// Both run count -> scan -> emit over the hit lists (CSR of contig-local positions), one warp
// per query.  Intersection compacts kept pieces with a ballot.  Difference walks the hits in
// ascending position order (the reverse of the fully descending list): with start <= end for
// every hit and qs <= qe, the order inside a run of equal starts does not change the pieces, so
// the cursor before each hit is a warp max-scan of (ce + 1) and the gaps are a ballot.  When B
// holds intervals with start > end the order inside equal-start runs matters (the reference
// sorts by (start, end) ascending), and lane 0 sweeps the query sequentially in exactly that
// order.  A covered piece reaching the type's maximum ends the sweep (the reference's
// cursor = end + 1 overflows there).
#include <algorithm>
#include <type_traits>
#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerBlock = kThreads / kWarp;

template <typename S>
__device__ __forceinline__ S smax(S a, S b) { return a > b ? a : b; }
template <typename S>
__device__ __forceinline__ S smin(S a, S b) { return a < b ? a : b; }

template <typename S>
__device__ __forceinline__ S warp_incl_max(S v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const S o = __shfl_up_sync(kFull, v, d);
        if (lane >= d) v = smax(v, o);
    }
    return v;
}

// One warp per query, grid-stride over queries.
template <typename S, bool EMIT>
__global__ void __launch_bounds__(kThreads) k_isect(MapView<S> m, const S* __restrict__ qs,
                                                    const S* __restrict__ qe, const int32_t* __restrict__ qc,
                                                    int64_t nq, const int64_t* __restrict__ hoff,
                                                    const int32_t* __restrict__ hits, uint32_t* __restrict__ cnt,
                                                    const int64_t* __restrict__ ooff, S* __restrict__ os,
                                                    S* __restrict__ oe, int32_t* __restrict__ ob, int* d_err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t q = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); q < nq; q += warps) {
        const int g = qc ? qc[q] : 0;
        if (g < 0 || g >= m.G) {  // reported; such a query has no piece
            if (lane == 0) {
                atomicCAS(d_err, kDevOk, kDevBadContig);
                if (!EMIT) cnt[q] = 0;
            }
            continue;
        }
        const int64_t a = hoff[q], b = hoff[q + 1];
        const S s0 = qs[q], e0 = qe[q];
        const int64_t lo = m.seg[g];
        int64_t w = EMIT ? ooff[q] : 0;
        uint32_t c = 0;
        for (int64_t p0 = a; p0 < b; p0 += 32) {
            const int64_t p = p0 + lane;
            bool keep = false;
            S s = 0, e = 0;
            int32_t h = 0;
            if (p < b) {
                h = hits[p];
                S hs, he;
                if (m.rec) {
                    const IvRec<S> r = m.rec[lo + h];
                    hs = r.s;
                    he = r.e;
                } else {
                    hs = m.starts[lo + h];
                    he = m.ends[lo + h];
                }
                s = smax(s0, hs);
                e = smin(e0, he);
                keep = s <= e;
            }
            const uint32_t bal = __ballot_sync(kFull, keep);
            if (EMIT && keep) {
                const int64_t at = w + __popc(bal & lanemask_lt());
                os[at] = s;
                oe[at] = e;
                ob[at] = h;
            }
            w += __popc(bal);
            c += __popc(bal);
        }
        if (!EMIT && lane == 0) cnt[q] = c;
    }
}

// Exact sequential sweep of one query (lane 0): runs of equal start in ascending start order,
// each run in ascending end order.  The hit list is fully descending in position, i.e. start
// descending and, inside an equal-start run, end ascending.
template <typename S, bool EMIT>
__device__ uint32_t diff_sequential(const S* __restrict__ st, const S* __restrict__ en,
                                    const int32_t* __restrict__ list, int64_t m, S s0, S e0, S* os, S* oe,
                                    int64_t w) {
    uint32_t c = 0;
    S cursor = s0;
    bool closed = false;
    int64_t j = m - 1;
    while (j >= 0) {
        const S rs = st[list[j]];
        int64_t r = j;
        while (r > 0 && st[list[r - 1]] == rs) --r;
        for (int64_t k = r; k <= j; ++k) {
            const int32_t h = list[k];
            const S cs = smax(st[h], s0), ce = smin(en[h], e0);
            if (!closed && cs > cursor) {
                if (EMIT) {
                    os[w + c] = cursor;
                    oe[w + c] = cs - 1;
                }
                ++c;
            }
            if (ce == Lim<S>::hi) closed = true;
            else if (ce + 1 > cursor) cursor = ce + 1;
        }
        j = r - 1;
    }
    if (!closed && cursor <= e0) {
        if (EMIT) {
            os[w + c] = cursor;
            oe[w + c] = e0;
        }
        ++c;
    }
    return c;
}

template <typename S, bool EMIT>
__global__ void __launch_bounds__(kThreads) k_diff(MapView<S> m, const S* __restrict__ qs,
                                                   const S* __restrict__ qe, const int32_t* __restrict__ qc,
                                                   int64_t nq, const int64_t* __restrict__ hoff,
                                                   const int32_t* __restrict__ hits, int sequential,
                                                   uint32_t* __restrict__ cnt, const int64_t* __restrict__ ooff,
                                                   S* __restrict__ os, S* __restrict__ oe, int* d_err) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t q = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); q < nq; q += warps) {
        const int g = qc ? qc[q] : 0;
        if (g < 0 || g >= m.G) {  // reported; such a query has no piece
            if (lane == 0) {
                atomicCAS(d_err, kDevOk, kDevBadContig);
                if (!EMIT) cnt[q] = 0;
            }
            continue;
        }
        // the writing pass skips the queries without a piece (often nearly all of them)
        if (EMIT && ooff[q + 1] == ooff[q]) continue;
        const int64_t a = hoff[q], b = hoff[q + 1], mq = b - a;
        const S s0 = qs[q], e0 = qe[q];
        const int64_t lo = m.seg[g];
        const S* st = m.starts + lo;
        const S* en = m.ends + lo;
        const int64_t w0 = EMIT ? ooff[q] : 0;
        if (sequential) {
            if (lane == 0) {
                const uint32_t c = diff_sequential<S, EMIT>(st, en, hits + a, mq, s0, e0, os, oe, w0);
                if (!EMIT) cnt[q] = c;
            }
            continue;
        }
        // qs > qe: every hit starts at or before qe < qs, so no gap opens before the cursor qs,
        // and the trailing piece needs cursor <= qe: no piece at all
        if (s0 > e0) {
            if (!EMIT && lane == 0) cnt[q] = 0;
            continue;
        }
        S cursor = s0;
        bool closed = false;
        int64_t w = w0;
        uint32_t c = 0;
        for (int64_t t0 = 0; t0 < mq; t0 += 32) {
            const int64_t t = t0 + lane;
            const bool valid = t < mq;
            S cs = 0, nxt = Lim<S>::lo;
            bool cl = false;
            if (valid) {
                const int32_t h = hits[b - 1 - t];  // ascending position order
                S hs, he;
                if (m.rec) {
                    const IvRec<S> r = m.rec[lo + h];
                    hs = r.s;
                    he = r.e;
                } else {
                    hs = st[h];
                    he = en[h];
                }
                cs = smax(hs, s0);
                const S ce = smin(he, e0);
                cl = ce == Lim<S>::hi;
                nxt = cl ? Lim<S>::lo : ce + 1;
            }
            const S incl = warp_incl_max(nxt);
            S excl = __shfl_up_sync(kFull, incl, 1);
            if (lane == 0) excl = Lim<S>::lo;
            const uint32_t clb = __ballot_sync(kFull, cl);
            const S cur = smax(cursor, excl);
            const bool closed_here = closed || (clb & lanemask_lt()) != 0;
            const bool gap = valid && !closed_here && cs > cur;
            const uint32_t gb = __ballot_sync(kFull, gap);
            if (EMIT && gap) {
                const int64_t at = w + __popc(gb & lanemask_lt());
                os[at] = cur;
                oe[at] = cs - 1;
            }
            w += __popc(gb);
            c += __popc(gb);
            cursor = smax(cursor, __shfl_sync(kFull, incl, 31));
            closed = closed || clb != 0;
            // covered up to qe: the later hits (starting at or before qe) open no gap
            if (closed || cursor > e0) break;
        }
        if (!closed && cursor <= e0) {
            if (EMIT && lane == 0) {
                os[w] = cursor;
                oe[w] = e0;
            }
            ++c;
        }
        if (!EMIT && lane == 0) cnt[q] = c;
    }
}

// search_keys / search_items (hpp:913-938, pyx:302-345): the hits' (start, end[, data]) in
// hit-list order.  One warp per query.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_keys(MapView<S> m, const int32_t* __restrict__ qc, int64_t nq,
                                                   const int64_t* __restrict__ hoff,
                                                   const int32_t* __restrict__ hits, S* __restrict__ os,
                                                   S* __restrict__ oe, int32_t* __restrict__ od) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t q = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); q < nq; q += warps) {
        const int g = qc ? qc[q] : 0;  // reported by the search that made the lists
        if (g < 0 || g >= m.G) continue;
        const int64_t lo = m.seg[g];
        for (int64_t p = hoff[q] + lane; p < hoff[q + 1]; p += 32) {
            const int64_t k = lo + hits[p];
            if (m.rec) {
                const IvRec<S> r = m.rec[k];
                os[p] = r.s;
                oe[p] = r.e;
                if (od) od[p] = r.d;
            } else {
                os[p] = m.starts[k];
                oe[p] = m.ends[k];
                if (od) od[p] = m.data[k];
            }
        }
    }
}

// coverage (hpp:979-1006, pyx:347-361): per query the number of hits and the sum of
// min(end, qe) - max(start, qs) over them (no +1), accumulated in the coordinate type with
// two's-complement wrap.  One warp per query.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_coverage(MapView<S> m, const S* __restrict__ qs,
                                                       const S* __restrict__ qe, const int32_t* __restrict__ qc,
                                                       int64_t nq, const int64_t* __restrict__ hoff,
                                                       const int32_t* __restrict__ hits,
                                                       uint64_t* __restrict__ count, S* __restrict__ cov) {
    using U = typename std::make_unsigned<S>::type;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * kWarpsPerBlock;
    for (int64_t q = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); q < nq; q += warps) {
        const int g = qc ? qc[q] : 0;
        if (g < 0 || g >= m.G) {  // reported by the search that made the lists (no hits)
            if (lane == 0) {
                count[q] = 0;
                cov[q] = 0;
            }
            continue;
        }
        const int64_t lo = m.seg[g];
        const S s0 = qs[q], e0 = qe[q];
        U acc = 0;
        for (int64_t p = hoff[q] + lane; p < hoff[q + 1]; p += 32) {
            const int64_t k = lo + hits[p];
            S hs, he;
            if (m.rec) {
                const IvRec<S> r = m.rec[k];
                hs = r.s;
                he = r.e;
            } else {
                hs = m.starts[k];
                he = m.ends[k];
            }
            acc += (U)smin(he, e0) - (U)smax(hs, s0);
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) acc += __shfl_xor_sync(kFull, acc, d);
        if (lane == 0) {
            count[q] = (uint64_t)(hoff[q + 1] - hoff[q]);
            cov[q] = (S)acc;
        }
    }
}

template <typename S>
__global__ void k_any_inverted(const S* __restrict__ starts, const S* __restrict__ ends, int64_t n,
                               int* __restrict__ flag) {
    bool inv = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        inv = inv || starts[i] > ends[i];
    if (__any_sync(kFull, inv) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

inline unsigned warp_blocks(int64_t nq) {
    // one warp per query, at most 16 resident blocks of 8 warps per SM on 152 SMs
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(nq, kWarpsPerBlock), 152 * 16 * 8));
}

}  // namespace

template <typename S>
cudaError_t launch_isect(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits,
                         uint32_t* counts, const int64_t* ooff, S* os, S* oe, int32_t* ob, int* d_err,
                         cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    const S* qs = static_cast<const S*>(q.qs);
    const S* qe = static_cast<const S*>(q.qe);
    if (ooff)
        k_isect<S, true><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, qs, qe, q.qc, q.nq, hoff, hits, nullptr, ooff,
                                                                 os, oe, ob, d_err);
    else
        k_isect<S, false><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, qs, qe, q.qc, q.nq, hoff, hits, counts,
                                                                  nullptr, nullptr, nullptr, nullptr, d_err);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_diff(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits, bool sequential,
                        uint32_t* counts, const int64_t* ooff, S* os, S* oe, int* d_err, cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    const S* qs = static_cast<const S*>(q.qs);
    const S* qe = static_cast<const S*>(q.qe);
    if (ooff)
        k_diff<S, true><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, qs, qe, q.qc, q.nq, hoff, hits, sequential ? 1 : 0,
                                                                nullptr, ooff, os, oe, d_err);
    else
        k_diff<S, false><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, qs, qe, q.qc, q.nq, hoff, hits,
                                                                 sequential ? 1 : 0, counts, nullptr, nullptr,
                                                                 nullptr, d_err);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_keys(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits, S* os, S* oe,
                        int32_t* od, cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    k_keys<S><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, q.qc, q.nq, hoff, hits, os, oe, od);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_coverage(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits,
                            uint64_t* count, S* cov, cudaStream_t st) {
    if (q.nq <= 0) return cudaSuccess;
    k_coverage<S><<<warp_blocks(q.nq), kThreads, 0, st>>>(m, static_cast<const S*>(q.qs),
                                                           static_cast<const S*>(q.qe), q.qc, q.nq, hoff, hits,
                                                           count, cov);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_records(const S* __restrict__ starts, const S* __restrict__ ends,
                                                      const int32_t* __restrict__ data, int64_t n,
                                                      IvRec<S>* __restrict__ rec) {
    const int64_t stride = (int64_t)gridDim.x * kThreads;
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) {
        IvRec<S> r{};
        r.s = starts[i];
        r.e = ends[i];
        r.d = data[i];
        rec[i] = r;
    }
}

template <typename S>
cudaError_t launch_records(const S* starts, const S* ends, const int32_t* data, int64_t n, IvRec<S>* rec,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_records<S><<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kThreads), 152 * 8)), kThreads, 0,
                   st>>>(starts, ends, data, n, rec);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_any_inverted(MapView<S> m, int* flag, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess || m.n <= 0) return e;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(m.n, kThreads), 152 * 8));
    k_any_inverted<S><<<blocks, kThreads, 0, st>>>(m.starts, m.ends, m.n, flag);
    note_launch();
    return cudaGetLastError();
}

#define SIG_SINST(S)                                                                                          \
    template cudaError_t launch_isect<S>(MapView<S>, QueryBatch, const int64_t*, const int32_t*, uint32_t*,   \
                                         const int64_t*, S*, S*, int32_t*, int*, cudaStream_t);               \
    template cudaError_t launch_diff<S>(MapView<S>, QueryBatch, const int64_t*, const int32_t*, bool,         \
                                        uint32_t*, const int64_t*, S*, S*, int*, cudaStream_t);               \
    template cudaError_t launch_any_inverted<S>(MapView<S>, int*, cudaStream_t);                          \
    template cudaError_t launch_keys<S>(MapView<S>, QueryBatch, const int64_t*, const int32_t*, S*, S*,        \
                                        int32_t*, cudaStream_t);                                              \
    template cudaError_t launch_coverage<S>(MapView<S>, QueryBatch, const int64_t*, const int32_t*,            \
                                            uint64_t*, S*, cudaStream_t);                                     \
    template cudaError_t launch_records<S>(const S*, const S*, const int32_t*, int64_t, IvRec<S>*, cudaStream_t);
SIG_SINST(int32_t)
SIG_SINST(int64_t)

}  // namespace sig
