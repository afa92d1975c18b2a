// si_batched.cu -- the BATCHED query path.
//
// The reference answers a batch one query at a time (src/superintervals/intervalmap.pyx:363-494
// loop over IntervalMap::search_idxs, hpp:879-905).  Queries that lie close together on a contig
// hit nearly the same intervals, so here they are answered together:
//
//  1. prepare: queries are radix-sorted by one packed key (class, contig, end offset);
//     each sorted query gets its upper bound (binary / Eytzinger / learned, si_ubound.cuh)
//     through a block-cooperative search.  "class" puts queries longer than a threshold
//     after the short ones.
//  2. tiles: a CTA takes `tile_q` consecutive sorted short queries of one contig.  Their
//     candidate set C = { k <= max ub : ends[k] >= min qs } holds every hit of every query of
//     the tile; it is gathered into shared memory, in descending position order, by a
//     block-wide top-down BFS over the max-of-32 pyramid of ends for the positions near the
//     tile, and over the pyramid of the long-interval list (intervals at least 32768 long)
//     for the positions further back.  C is split by interval length: near-start candidates
//     are filtered per query, long ones are nearly all hits.  The count pass counts (one
//     query per thread) and records the query's head-run length (the run of consecutive hits
//     ending at ub); the emit pass writes the head run arithmetically (ascending for the
//     C++ search_idxs order, hpp:892-895; descending for search_values / the C API) and then
//     the remaining hits in descending order (one query per warp, ballot compaction) --
//     exactly the reference's output.
//  3. long queries share the tile's long-interval candidates and scan their own window
//     directly; tiles whose C overflows shared memory take the per-query walk over the
//     pyramid (one warp per query, 32 positions per step).
// Tiles and long queries are handed out by an atomic work counter (persistent CTAs), so uneven
// per-query result counts do not leave SMs idle.
#include <algorithm>
#include <vector>

#include "si_batched.cuh"
#include "si_gpu/c_api.h"
#include "si_ubound.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
constexpr int kWarpsPerCta = kThreads / kWarp;

template <typename S>
struct Pyr {
    const S* ends;
    const S* m[kMaxLevels];
    int H;
};

// Highest chunk index <= cmax whose max end is >= L (or -1), by climbing the pyramid and
// descending into the nearest qualifying node.  Warp-uniform.
template <typename S>
__device__ __forceinline__ int64_t highest_chunk(const Pyr<S>& P, int64_t cmax, S L, int lane) {
    if (cmax < 0) return -1;
    if (P.H == 0) return 0;
    int64_t node = cmax;
    int h = 1;
    int64_t found = -1;
    while (true) {
        const int64_t grp = node >> 5;
        const int pos = (int)(node & 31);
        const S v = P.m[h - 1][(grp << 5) + lane];
        const unsigned mask = __ballot_sync(kFull, lane <= pos && v >= L);
        if (mask) {
            found = (grp << 5) + (31 - __clz(mask));
            break;
        }
        if (h == P.H || grp == 0) return -1;
        node = grp - 1;
        ++h;
    }
    while (h > 1) {
        const S v = P.m[h - 2][(found << 5) + lane];
        const unsigned mask = __ballot_sync(kFull, v >= L);
        if (!mask) return -1;  // cannot happen: the parent's max is >= L
        found = (found << 5) + (31 - __clz(mask));
        --h;
    }
    return found;
}

// Visit in descending position order every position k in [lo, u] with ends[k] >= L.
// f(chunk, hitmask, value) is called per 32-position chunk holding hits (bit l = position
// chunk*32+l); it returns false to stop.  Warp-uniform.
template <typename S, typename F>
__device__ __forceinline__ void scan_desc(const Pyr<S>& P, int64_t lo, int64_t u, S L, int lane, F&& f) {
    int64_t cur = u;
    while (cur >= lo) {
        const int64_t c = highest_chunk(P, cur >> 5, L, lane);
        if (c < 0 || ((c << 5) + 31) < lo) return;
        if (c < (cur >> 5)) cur = (c << 5) + 31;
        const int64_t grp = c >> 5;
        unsigned gm;
        if (P.H == 0) {
            gm = 1u;
        } else {
            const S v1 = P.m[0][(grp << 5) + lane];
            gm = __ballot_sync(kFull, lane <= (int)(c & 31) && v1 >= L);
        }
        while (gm) {
            int64_t ch[4];
            S val[4];
            bool ok[4];
            int cnt = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                ok[k] = false;
                if (gm) {
                    const int b = 31 - __clz(gm);
                    gm &= ~(1u << b);
                    ch[k] = (grp << 5) + b;
                    const int64_t p = (ch[k] << 5) + lane;
                    ok[k] = p <= cur && p >= lo;
                    val[k] = ok[k] ? P.ends[p] : Lim<S>::lo;
                    cnt = k + 1;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (k < cnt) {
                    const unsigned hm = __ballot_sync(kFull, ok[k] && val[k] >= L);
                    if (hm && !f(ch[k], hm, val[k])) return;
                }
            }
        }
        cur = (grp << 10) - 1;
    }
}

// Query class codes (the sort key's top bits): g for a short query of contig g, G + g for a
// long one, 2G + g for one with start > end (long-query path, counted by the count pass),
// 3G for a contig id outside [0, G).
__device__ __forceinline__ bool code_is_long(uint32_t c, int G) {
    return c >= (uint32_t)G && c < 3u * (uint32_t)G;
}
__device__ __forceinline__ bool code_is_inverted(uint32_t c, int G) {
    return c >= 2u * (uint32_t)G && c < 3u * (uint32_t)G;
}
__device__ __forceinline__ int code_contig(uint32_t c, int G) {
    const uint32_t u = (uint32_t)G;
    return (int)(c < u ? c : c < 2u * u ? c - u : c < 3u * u ? c - 2u * u : 0u);
}

__device__ __forceinline__ unsigned above_mask(int lane) {
    // bits strictly above `lane`
    return lane == 31 ? 0u : ~((2u << lane) - 1u);
}

template <typename S>
struct TileArgs {
    Pyr<S> P;
    Pyr<S> PL;               // pyramid over the long-interval list (intervals >= long_split long)
    const int32_t* long_pos; // its global positions, in position order
    const int64_t* blk_cut;  // per tile of 256 queries: (p_cut, long-list end) or -1; null: none
    const int64_t* long_seg; // first list index of each contig
    int64_t long_split;
    const S* end_sorted;     // each contig's ends ascending (no interval has start > end), or null
    const S* starts;
    int64_t split_len;
    const int32_t* data;
    const int64_t* seg;
    int32_t G;
    const S* sq_s;
    const int32_t* sq_u;
    const uint32_t* sq_c;
    const int32_t* sq_id;
    int64_t nq;
    int tile_q;
    int cap;
    int n_tiles;
    int* tile_counter;
    // count pass
    uint32_t* counts;
    int32_t* heads;
    // emit pass
    const int32_t* heads_in;
    const int64_t* offsets;
    int64_t id_lo, id_hi;    // emit only the queries with ids in [id_lo, id_hi)
    int64_t out_cap;         // values the output holds: queries whose lists end past it are skipped
    int64_t out_base;
    int order;
    bool values;
    bool emit_copy;          // copy the long-interval list's section of part B (else filter it)
    int32_t* out;
    int* d_err;
    // per-tile candidate lists stored by the count pass and reloaded by the emit pass
    unsigned char* cache;
    int64_t cache_stride;
};

// ---- per-query walk (long queries, overflowing tiles): one warp, direct output ----
template <typename S, bool EMIT>
__device__ void walk_query(const TileArgs<S>& a, S qs, int64_t u, int64_t lo, int32_t id, int lane) {
    if (!EMIT) {
        uint32_t cnt = 0;
        int64_t head = 0;
        bool open = true;
        int64_t expect = u;
        if (u >= lo) {
            scan_desc(a.P, lo, u, qs, lane, [&](int64_t ch, unsigned hm, S) {
                cnt += __popc(hm);
                if (open) {
                    if (ch != (expect >> 5)) {
                        open = false;
                    } else {
                        const int le = (int)(expect & 31);
                        const unsigned low = (le == 31) ? ~0u : ((1u << (le + 1)) - 1u);
                        const unsigned zeros = ~hm & low;
                        if (!zeros) {
                            head += le + 1;
                            expect = (ch << 5) - 1;
                        } else {
                            head += le - (31 - __clz(zeros));
                            open = false;
                        }
                    }
                }
                return true;
            });
        }
        if (lane == 0) {
            a.counts[id] = cnt;
            a.heads[id] = (int32_t)head;
        }
        return;
    }
    int64_t h = 0;
    if (a.end_sorted) {
        // short queries were counted from ranks, without their head run: find it here
        for (int64_t top = u; top >= lo; top -= 32) {
            const int64_t p = top - lane;
            const unsigned m = __ballot_sync(kFull, p >= lo && a.P.ends[p] >= qs);
            const int run = (m == kFull) ? 32 : __ffs(~m) - 1;
            h += run;
            if (run < 32) break;
        }
    } else {
        h = a.heads_in[id];
    }
    const int64_t base = a.offsets[id] - a.out_base;
    const int64_t capq = a.offsets[id + 1] - a.offsets[id];
    if (h > capq) {
        if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
        return;
    }
    int32_t* dst = a.out + base;
    for (int64_t r = lane; r < h; r += 32) {
        const int64_t pos = (a.order == kOrderIdxsCpp) ? (u - h + 1 + r) : (u - r);
        dst[r] = a.values ? a.data[pos] : (int32_t)(pos - lo);
    }
    int64_t w = h;
    const int64_t start = u - h;
    if (start >= lo) {
        scan_desc(a.P, lo, start, qs, lane, [&](int64_t ch, unsigned hm, S) {
            const int k = __popc(hm);
            if (w + k > capq) {
                if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
                return false;
            }
            if ((hm >> lane) & 1u) {
                const int64_t pos = (ch << 5) + lane;
                dst[w + __popc(hm & above_mask(lane))] = a.values ? a.data[pos] : (int32_t)(pos - lo);
            }
            w += k;
            return true;
        });
    }
}

// Block-wide exclusive scan of v[0, n) in place; the total goes to *s_sum.  Ends synchronized.
__device__ void block_excl_scan(int32_t* v, int n, int* s_wsum, int* s_sum) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int per = (n + kThreads - 1) / kThreads;
    const int beg = tid * per;
    const int end = min(beg + per, n);
    int local = 0;
    for (int i = beg; i < end; ++i) local += v[i];
    int inc = local;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(kFull, inc, d);
        if (lane >= d) inc += y;
    }
    if (lane == 31) s_wsum[warp] = inc;
    __syncthreads();
    int woff = 0;
    for (int w = 0; w < warp; ++w) woff += s_wsum[w];
    int run = woff + inc - local;
    for (int i = beg; i < end; ++i) {
        const int t = v[i];
        v[i] = run;
        run += t;
    }
    if (tid == kThreads - 1) *s_sum = woff + inc;
    __syncthreads();
}

// Block-wide top-down gather of C = { k in [lo, umax] : ends[k] >= L } in DESCENDING position
// order into (cpos, cend), one level of the max pyramid per round: every warp expands frontier
// nodes (one coalesced 32-child load + ballot each), a block scan places the surviving children
// in order.  Frontier lists ping-pong between cpos and lst.  Returns |C|, or -1 when a frontier
// or C would exceed `cap`.  Block-uniform.
template <typename S>
__device__ int gather_bfs(const Pyr<S>& P, int64_t lo, int64_t umax, S L, int cap, int32_t* cpos, S* cend,
                          int32_t* lst, int32_t* cnt, uint32_t* msk, int* s_wsum, int* s_n, int* s_sum,
                          const int32_t* remap = nullptr) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (umax < lo) return 0;
    // start at the lowest level whose nodes covering [lo, umax] are at most 32 (the top level
    // always is): the levels above it hold no extra information for this range
    int H = 0;
    while (H < P.H && (umax >> (5 * H)) - (lo >> (5 * H)) >= 32) ++H;
    if (warp == 0) {
        const int64_t nlo = lo >> (5 * H), nhi = umax >> (5 * H);
        const int64_t node = nlo + lane;
        bool ok = node <= nhi;
        S v = Lim<S>::lo;
        if (ok) v = (H == 0) ? P.ends[node] : P.m[H - 1][node];
        ok = ok && v >= L;
        const unsigned m = __ballot_sync(kFull, ok);
        const bool fits = __popc(m) <= cap;  // nothing is written past `cap`
        if (ok && fits) {
            const int idx = __popc(m & above_mask(lane));
            ((H & 1) ? lst : cpos)[idx] = (H == 0 && remap) ? remap[node] : (int32_t)node;
            if (H == 0) cend[idx] = v;
        }
        if (lane == 0) *s_n = fits ? __popc(m) : -1;
    }
    __syncthreads();
    int nf = *s_n;
    if (nf < 0) return -1;
    for (int h = H; h >= 1; --h) {
        const S* A = (h == 1) ? P.ends : P.m[h - 2];
        const int sh = 5 * (h - 1);
        const int64_t clo = lo >> sh, chi = umax >> sh;
        const int32_t* in = (h & 1) ? lst : cpos;
        int32_t* out = (h & 1) ? cpos : lst;
        for (int f0 = warp; f0 < nf; f0 += 4 * kWarpsPerCta) {
            // up to 4 frontier nodes per warp per round: the loads are independent
            bool ok[4];
            S v[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int f = f0 + k * kWarpsPerCta;
                ok[k] = false;
                if (f < nf) {
                    const int64_t c = ((int64_t)in[f] << 5) + lane;
                    ok[k] = c >= clo && c <= chi;
                    v[k] = ok[k] ? A[c] : Lim<S>::lo;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int f = f0 + k * kWarpsPerCta;
                const unsigned m = __ballot_sync(kFull, ok[k] && v[k] >= L);
                if (f < nf && lane == 0) {
                    msk[f] = m;
                    cnt[f] = __popc(m);
                }
            }
        }
        __syncthreads();
        block_excl_scan(cnt, nf, s_wsum, s_sum);
        const int total = *s_sum;
        if (total > cap) return -1;
        for (int f = warp; f < nf; f += kWarpsPerCta) {
            const unsigned m = msk[f];
            if ((m >> lane) & 1u) {
                const int64_t c = ((int64_t)in[f] << 5) + lane;
                const int idx = cnt[f] + __popc(m & above_mask(lane));
                out[idx] = (h == 1 && remap) ? remap[c] : (int32_t)c;
                if (h == 1) cend[idx] = A[c];
            }
        }
        __syncthreads();
        nf = total;
    }
    return nf;
}

// start >= qs - X, without overflow
template <typename S>
__device__ __forceinline__ bool near_start(S start, S qs, int64_t X) {
    return start >= qs || (uint64_t)qs - (uint64_t)start <= (uint64_t)X;
}

// The smallest start that near_start accepts: qs - X clamped to the coordinate range, so that
// near_start(start, qs, X) == (start >= near_threshold(qs, X)).
template <typename S>
__device__ __forceinline__ S near_threshold(S qs, int64_t X) {
    const uint64_t room = (uint64_t)qs - (uint64_t)Lim<S>::lo;  // qs - S_MIN >= 0
    return (uint64_t)X >= room ? Lim<S>::lo : (S)((uint64_t)qs - (uint64_t)X);
}

// end - start >= X, without overflow
template <typename S>
__device__ __forceinline__ bool is_long_iv(S start, S end, int64_t X) {
    return end >= start && (uint64_t)end - (uint64_t)start >= (uint64_t)X;
}

constexpr int kLnu = 128;        // long-list candidates ending before the tile's max qs
constexpr int kCacheHeader = 32; // bytes before a tile's cached lists
constexpr int kMaxBlocks = 8192 / 32 + 1;

// First position p in [a, b] with start[p] >= qs - X (starts ascending; b means none).
// Warp-cooperative 32-ary search over global memory.  Warp-uniform.
template <typename S>
__device__ __forceinline__ int64_t warp_first_near(const S* __restrict__ starts, int64_t a, int64_t b, S qs,
                                                   int64_t X, int lane) {
    while (b - a > 32) {
        const int64_t step = (b - a + 31) >> 5;
        const int64_t idx = a + lane * step;
        const unsigned m = __ballot_sync(kFull, idx < b && near_start<S>(starts[idx], qs, X));
        if (!m) {
            const int64_t last = min((int64_t)31, (b - 1 - a) / step);  // every valid sample is below
            a = a + last * step + 1;
        } else {
            const int k = __ffs(m) - 1;
            if (k == 0) return a;
            const int64_t na = a + (int64_t)(k - 1) * step + 1, nb = a + (int64_t)k * step;
            a = na;
            b = nb;
        }
    }
    const int64_t idx = a + lane;
    const unsigned m = __ballot_sync(kFull, idx < b && near_start<S>(starts[idx], qs, X));
    return m ? a + __ffs(m) - 1 : b;
}

// First index in [a, b) of an ascending array whose element is >= key (b when none).
// Warp-cooperative 32-ary search over global memory.  Warp-uniform.
template <typename T, typename K>
__device__ __forceinline__ int64_t warp_first_geq(const T* __restrict__ arr, int64_t a, int64_t b, K key,
                                                  int lane) {
    while (b - a > 32) {
        const int64_t step = (b - a + 31) >> 5;
        const int64_t idx = a + lane * step;
        const unsigned m = __ballot_sync(kFull, idx < b && (K)arr[idx] >= key);
        if (!m) {
            const int64_t last = min((int64_t)31, (b - 1 - a) / step);
            a = a + last * step + 1;
        } else {
            const int k = __ffs(m) - 1;
            if (k == 0) return a;
            const int64_t na = a + (int64_t)(k - 1) * step + 1, nb = a + (int64_t)k * step;
            a = na;
            b = nb;
        }
    }
    const int64_t idx = a + lane;
    const unsigned m = __ballot_sync(kFull, idx < b && (K)arr[idx] >= key);
    return m ? a + __ffs(m) - 1 : b;
}

// Upper bound of v inside one contig (last k with starts[k] <= v, else -1) by one warp: 32-ary
// steps over the contig's starts.  With the learned provider, the leaf (32-ary steps over the
// leaves' first keys) and the leaf model's error window narrow the range first; the answer is
// checked against its neighbours and the whole leaf is searched when the window missed (exact
// either way, as ub_search).  Warp-uniform.
template <typename S>
__device__ int64_t warp_ub(const UbView<S>& U, int g, const S* __restrict__ starts, int64_t n, S v, int lane) {
    if (n <= 0 || v < starts[0]) return -1;
    if (v == Lim<S>::hi) return n - 1;
    const S v1 = (S)(v + 1);  // first index whose start is >= v1, minus one
    if (U.mode == 2 && U.leaves) {
        const int base = U.leaf_base[g];
        const int nl = U.leaf_base[g + 1] - base;
        const int l0 = (int)warp_first_geq<S, S>(U.leaf_key + base, 0, nl, v1, lane) - 1;  // >= 0
        const int64_t pa = U.leaf_pos[base + l0];
        const int64_t pb = (l0 + 1 < nl ? (int64_t)U.leaf_pos[base + l0 + 1] : n) - 1;
        const LeafModel M = U.leaves[base + l0];
        const double pred = M.y0 + M.slope * ((double)v - U.key_mean[g] - M.x0);
        const double plo = pred - (double)M.err_lo - 1.0, phi = pred + (double)M.err_hi + 1.0;
        const int64_t a = plo <= (double)pa ? pa : (plo >= (double)pb ? pb : (int64_t)plo);
        int64_t b = phi >= (double)pb ? pb : (phi <= (double)pa ? pa : (int64_t)phi + 1);
        if (b > pb) b = pb;
        const int64_t r = warp_first_geq<S, S>(starts, a, b + 1, v1, lane) - 1;
        const bool ok = r >= pa && starts[r] <= v && (r + 1 >= n || starts[r + 1] > v);
        if (ok) return r;
        return warp_first_geq<S, S>(starts, pa, pb + 1, v1, lane) - 1;
    }
    return warp_first_geq<S, S>(starts, 0, n, v1, lane) - 1;
}

// First index in [a, b) of an ascending position list whose position is >= key (b when none).
__device__ __forceinline__ int64_t warp_first_pos_geq(const int32_t* __restrict__ pos, int64_t a, int64_t b,
                                                      int64_t key, int lane) {
    return warp_first_geq<int32_t, int64_t>(pos, a, b, key, lane);
}

// First index of a DESCENDING position list whose position is < key (n when none).
__device__ __forceinline__ int first_below(const int32_t* __restrict__ pos, int n, int64_t key) {
    int b0 = 0, b1 = n;
    while (b0 < b1) {
        const int mid = (b0 + b1) >> 1;
        if ((int64_t)pos[mid] >= key) b0 = mid + 1;
        else b1 = mid;
    }
    return b0;
}

// One long query, one warp.  Hits are the window [plo, u] of intervals starting at or after
// qs - X (read directly, 32 positions per step) plus, below the window, the tile's shared
// long candidates (intervals at least X long; shorter ones below the window cannot reach qs).
template <typename S, bool EMIT>
__device__ void long_query(const TileArgs<S>& a, S qs, int64_t u, int64_t lo, int32_t id,
                           const int32_t* __restrict__ cpos, const S* __restrict__ cend, int nc, int64_t h_in,
                           int64_t out_off, int64_t capq, int lane) {
    if (u < lo) {
        if (!EMIT && lane == 0) {
            a.counts[id] = 0;
            a.heads[id] = 0;
        }
        return;
    }
    const int64_t X = a.long_split;
    const S* __restrict__ ends = a.P.ends;
    const int64_t plo = warp_first_near<S>(a.starts, lo, u + 1, qs, X, lane);
    if (!EMIT) {
        uint32_t cnt = 0;
        int64_t head = 0;
        bool open = true;
        for (int64_t top = u; top >= plo; top -= 32) {
            const int64_t p = top - lane;
            const unsigned m = __ballot_sync(kFull, p >= plo && ends[p] >= qs);
            cnt += __popc(m);
            if (open) {
                const int run = (m == kFull) ? 32 : __ffs(~m) - 1;
                head += run;
                if (run < 32 && top - run >= plo) open = false;  // a miss inside the window ends it
            }
        }
        // a head run covering the whole window may continue into longer intervals below it
        for (int64_t top = plo - 1; open && top >= lo; top -= 32) {
            const int64_t p = top - lane;
            const unsigned m = __ballot_sync(kFull, p >= lo && ends[p] >= qs);
            const int run = (m == kFull) ? 32 : __ffs(~m) - 1;
            head += run;
            if (run < 32) open = false;
        }
        for (int kk = first_below(cpos, nc, plo); kk < nc; kk += 32) {
            const int tt = kk + lane;
            cnt += __popc(__ballot_sync(kFull, tt < nc && cend[tt] >= qs));
        }
        if (lane == 0) {
            a.counts[id] = cnt;
            a.heads[id] = (int32_t)head;
        }
        return;
    }
    int64_t h = h_in;
    if (h < 0) {
        // counted from ranks, without its head run: find it here (positions u, u - 1, ... hit)
        h = 0;
        for (int64_t top = u; top >= lo; top -= 32) {
            const int64_t p = top - lane;
            const unsigned m = __ballot_sync(kFull, p >= lo && ends[p] >= qs);
            const int run = (m == kFull) ? 32 : __ffs(~m) - 1;
            h += run;
            if (run < 32) break;
        }
    }
    if (h > capq) {
        if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
        return;
    }
    int32_t* dst = a.out + out_off;
    for (int64_t r = lane; r < h; r += 32) {
        const int64_t pos = (a.order == kOrderIdxsCpp) ? (u - h + 1 + r) : (u - r);
        dst[r] = a.values ? a.data[pos] : (int32_t)(pos - lo);
    }
    int64_t w = h;
    const unsigned lt = lanemask_lt();
    for (int64_t top = u - h; top >= plo; top -= 32) {  // the window below the head run
        const int64_t p = top - lane;
        const bool hit = p >= plo && ends[p] >= qs;
        const unsigned m = __ballot_sync(kFull, hit);
        const int k = __popc(m);
        if (w + k > capq) {
            if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
            return;
        }
        if (hit) dst[w + __popc(m & lt)] = a.values ? a.data[p] : (int32_t)(p - lo);
        w += k;
    }
    const int64_t below = plo < u - h + 1 ? plo : u - h + 1;  // long candidates under both
    for (int kk = first_below(cpos, nc, below); kk < nc; kk += 32) {
        const int tt = kk + lane;
        const bool hit = tt < nc && cend[tt] >= qs;
        const unsigned m = __ballot_sync(kFull, hit);
        const int k = __popc(m);
        if (w + k > capq) {
            if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
            return;
        }
        if (hit) {
            const int32_t pos = cpos[tt];
            dst[w + __popc(m & lt)] = a.values ? a.data[pos] : pos - (int32_t)lo;
        }
        w += k;
    }
}

// One warp copies src[0, len) (shared memory) to dst[0, len) (global memory): 4-byte stores,
// 128 values per round in four independent 32-wide slices.
__device__ __forceinline__ void warp_copy4(int32_t* __restrict__ dst, const int32_t* __restrict__ src, int len,
                                           int lane) {
    int k = lane;
    for (; k + 96 < len; k += 128) {
        const int32_t v0 = src[k], v1 = src[k + 32], v2 = src[k + 64], v3 = src[k + 96];
        dst[k] = v0;
        dst[k + 32] = v1;
        dst[k + 64] = v2;
        dst[k + 96] = v3;
    }
    for (; k < len; k += 32) dst[k] = src[k];
}

template <typename S, bool EMIT>
__global__ void __launch_bounds__(kThreads, 4) k_tiles(TileArgs<S> a) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int cap = a.cap, T = a.tile_q;
    S* cend = reinterpret_cast<S*>(smem);
    int32_t* cpos = reinterpret_cast<int32_t*>(cend + cap);
    S* q_s = reinterpret_cast<S*>(cpos + cap);
    int32_t* q_u = reinterpret_cast<int32_t*>(q_s + T);
    uint32_t* q_c = reinterpret_cast<uint32_t*>(q_u + T);
    int32_t* q_id = reinterpret_cast<int32_t*>(q_c + T);
    int64_t* q_off = reinterpret_cast<int64_t*>(q_id + T);    // emit: output offset of the query
    int32_t* q_cap = reinterpret_cast<int32_t*>(q_off + T);   // emit: its result count
    int32_t* q_h = q_cap + T;                                  // emit: its head-run length
    int32_t* q_ta = q_h + T;                                   // emit: first candidate after the head
    int32_t* q_tsplit = q_ta + T;                              // emit: end of the near-qs candidates
    int32_t* q_lb = q_tsplit + T;                              // emit: first long candidate (-1-x: misses)
    int32_t* lst = q_lb + T;                                    // BFS frontier, then long positions
    int32_t* cnt = lst + cap;                                  // BFS counts  } then long ends
    uint32_t* msk = reinterpret_cast<uint32_t*>(cnt + cap);   // BFS masks   } (+ starts, 32-bit S)
    int32_t* lpos = lst;
    S* lend = reinterpret_cast<S*>(cnt);
    S* cstart = (sizeof(S) == 4) ? reinterpret_cast<S*>(msk) : reinterpret_cast<S*>(msk + cap);
    __shared__ int s_tile, s_n, s_sum, s_nlnu, s_nlm, s_next;
    __shared__ int64_t s_cut[2];
    __shared__ int s_wsum[kWarpsPerCta];
    __shared__ S s_red[kWarpsPerCta], s_red2[kWarpsPerCta];
    __shared__ int32_t s_red3[kWarpsPerCta];
    __shared__ uint32_t s_bmask[kMaxBlocks];
    __shared__ int32_t s_boff[kMaxBlocks];
    __shared__ int32_t s_lnu_idx[kLnu];  // long candidates ending before the run's max qs: their
    __shared__ S s_lnu_end[kLnu];        // indices in the long list (ascending) and their ends

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t X = a.split_len;
    while (true) {
        if (tid == 0) s_tile = atomicAdd(a.tile_counter, 1);
        __syncthreads();
        const int tc = s_tile;
        if (tc >= a.n_tiles) return;
        // heaviest first: long queries sort to the end of the batch, so tiles are handed
        // out from the end and the per-query walks overlap the shared-candidate tiles
        const int t = a.n_tiles - 1 - tc;
        const int64_t j0 = (int64_t)t * T;
        const int nt = (int)((a.nq - j0) < (int64_t)T ? (a.nq - j0) : (int64_t)T);
        if (!EMIT && a.end_sorted && a.sq_c[j0 + nt - 1] < 2u * (uint32_t)a.G) {
            // classes are sorted and tiles are handed out from the end: this tile and every
            // later one hold short and long queries only, counted by the prepare pass
            return;
        }
        for (int i = tid; i < nt; i += kThreads) {
            q_s[i] = a.sq_s[j0 + i];
            q_u[i] = a.sq_u[j0 + i];
            q_c[i] = a.sq_c[j0 + i];
            q_id[i] = a.sq_id[j0 + i];
            if (EMIT) {
                // the tile's random per-query reads, issued together instead of per query
                const int32_t id = q_id[i];
                if (id < a.id_lo || id >= a.id_hi) {
                    q_off[i] = 0;
                    q_cap[i] = -1;  // outside the emitted window: skipped
                    q_h[i] = 0;
                } else {
                    const int64_t o = a.offsets[id], o1 = a.offsets[id + 1];
                    q_off[i] = o - a.out_base;
                    // a list ending past the output (a replayed graph with too small a capacity,
                    // reported by the caller) is not written
                    q_cap[i] = (o1 - a.out_base <= a.out_cap) ? (int32_t)(o1 - o) : -1;
                    // queries counted from ranks have no head run from the count pass: the emit
                    // finds it (-1)
                    const bool counted_by_rank = a.end_sorted && !code_is_inverted(q_c[i], a.G);
                    q_h[i] = counted_by_rank ? -1 : a.heads_in[id];
                }
            }
        }
        __syncthreads();
        int r0 = 0;
        while (r0 < nt) {
            // run of equal class/contig words [r0, r1): sorted, so binary search the end
            const uint32_t cw = q_c[r0];
            int lo_i = r0 + 1, hi_i = nt;
            while (lo_i < hi_i) {
                const int mid = (lo_i + hi_i) >> 1;
                if (q_c[mid] == cw) lo_i = mid + 1;
                else hi_i = mid;
            }
            const int r1 = lo_i;
            const bool is_long = code_is_long(cw, a.G);
            const int g = code_contig(cw, a.G);  // invalid contigs are reported by the prepare kernel
            const int64_t lo = a.seg[g];
            bool per_query = is_long && a.PL.ends == nullptr;
            const bool long_run = is_long && !per_query;
            // nc candidates; nl of them long, the first nlm of which come from the tile's own
            // gather (positions >= p_cut), the rest from the long-interval list; nlnu lnu entries
            int nc = 0, nl = 0, nlnu = 0, nlm = 0;
            // count pass over an index without inverted intervals: the prepare pass counted every
            // query but those with start > end (from ranks)
            const bool rank_run = !EMIT && a.end_sorted != nullptr && !code_is_inverted(cw, a.G);
            if (!is_long && !rank_run) {
                // a tile that is one run can reuse the candidate lists the count pass stored
                const bool whole = (r0 == 0 && r1 == nt);
                unsigned char* rec = (whole && a.cache) ? a.cache + (size_t)t * a.cache_stride : nullptr;
                int32_t* g_cpos = reinterpret_cast<int32_t*>(rec + kCacheHeader);
                S* g_cend = reinterpret_cast<S*>(g_cpos + cap);
                S* g_cstart = g_cend + cap;
                int32_t* g_lpos = reinterpret_cast<int32_t*>(g_cstart + cap);
                S* g_lend = reinterpret_cast<S*>(g_lpos + cap);
                int32_t* g_lnu_idx = reinterpret_cast<int32_t*>(g_lend + cap);
                S* g_lnu_end = reinterpret_cast<S*>(g_lnu_idx + kLnu);
                bool cached = false;
                if (EMIT && rec) {
                    if (tid == 0) {
                        const int32_t* hdr = reinterpret_cast<const int32_t*>(rec);
                        s_n = hdr[3] == 1 ? hdr[0] : -1;
                        s_sum = hdr[1];
                        s_nlnu = hdr[2];
                        s_nlm = hdr[4];
                    }
                    __syncthreads();
                    if (s_n >= 0) {
                        nc = s_n;
                        nl = s_sum;
                        nlnu = s_nlnu;
                        nlm = s_nlm;
                        for (int k = tid; k < nc; k += kThreads) {
                            cpos[k] = g_cpos[k];
                            cend[k] = g_cend[k];
                            cstart[k] = g_cstart[k];
                        }
                        for (int k = tid; k < nl; k += kThreads) {
                            lpos[k] = g_lpos[k];
                            lend[k] = g_lend[k];
                        }
                        for (int k = tid; k < nlnu && k < kLnu; k += kThreads) {
                            s_lnu_idx[k] = g_lnu_idx[k];
                            s_lnu_end[k] = g_lnu_end[k];
                        }
                        __syncthreads();
                        cached = true;
                    }
                }
                if (!cached) {
                    // L = min qs, Q = max qs over the run; umax = ub of the run's last query
                    // queries are only roughly ordered inside a run: reduce max ub as well
                    S mn = Lim<S>::hi, mx = Lim<S>::lo;
                    int32_t um = INT32_MIN;
                    for (int i = r0 + tid; i < r1; i += kThreads) {
                        mn = q_s[i] < mn ? q_s[i] : mn;
                        mx = q_s[i] > mx ? q_s[i] : mx;
                        um = q_u[i] > um ? q_u[i] : um;
                    }
    #pragma unroll
                    for (int d = 16; d > 0; d >>= 1) {
                        const S o = __shfl_xor_sync(kFull, mn, d);
                        mn = o < mn ? o : mn;
                        const S p = __shfl_xor_sync(kFull, mx, d);
                        mx = p > mx ? p : mx;
                        um = max(um, __shfl_xor_sync(kFull, um, d));
                    }
                    if (lane == 0) {
                        s_red[warp] = mn;
                        s_red2[warp] = mx;
                        s_red3[warp] = um;
                    }
                    if (tid == 0) s_nlnu = 0;
                    __syncthreads();
                    S L = s_red[0], Q = s_red2[0];
                    int32_t umx = s_red3[0];
    #pragma unroll
                    for (int w = 1; w < kWarpsPerCta; ++w) {
                        L = s_red[w] < L ? s_red[w] : L;
                        Q = s_red2[w] > Q ? s_red2[w] : Q;
                        umx = max(umx, s_red3[w]);
                    }
                    const int64_t umax = umx;
                    // positions below p_cut hold intervals starting more than long_split before L;
                    // those that reach L are at least long_split long, so they are gathered from
                    // the long-interval list instead of the whole position range
                    // precomputed by the prepare pass for a tile that is one block of sorted queries
                    // of one contig (valid when it lies inside [lo, umax + 1])
                    int64_t pre_pc = -1, pre_ch = -1;
                    if (a.blk_cut && r0 == 0 && r1 == nt) {
                        pre_pc = a.blk_cut[2 * t];
                        pre_ch = a.blk_cut[2 * t + 1];
                        if (pre_pc < lo || pre_pc > umax + 1) pre_pc = -1;
                    }
                    if (pre_pc >= 0) {
                        if (tid == 0) {
                            s_cut[0] = pre_pc;
                            s_cut[1] = pre_ch;
                        }
                    } else if (warp == 0) {
                        const int64_t pc =
                            umax < lo ? lo : warp_first_near<S>(a.starts, lo, umax + 1, L, a.long_split, lane);
                        const int64_t ch = warp_first_pos_geq(a.long_pos, a.long_seg[g], a.long_seg[g + 1], pc, lane);
                        if (lane == 0) {
                            s_cut[0] = pc;
                            s_cut[1] = ch;
                        }
                    }
                    __syncthreads();
                    const int64_t pcut = s_cut[0], c_lo = a.long_seg[g], c_hi = s_cut[1];
                    nc = gather_bfs<S>(a.P, pcut, umax, L, cap, cpos, cend, lst, cnt, msk, s_wsum, &s_n, &s_sum);
                    if (nc >= 0 && c_hi > c_lo) {  // then the long ones below p_cut, still descending
                        const int nlong = gather_bfs<S>(a.PL, c_lo, c_hi - 1, L, cap - nc, cpos + nc, cend + nc,
                                                        lst + nc, cnt, msk, s_wsum, &s_n, &s_sum, a.long_pos);
                        nc = nlong < 0 ? -1 : nc + nlong;
                    }
                    per_query = nc < 0;
                    if (!per_query && nc > 0) {
                        // long candidates (end - start >= X) into (lpos, lend), in order
                        const int nb = (nc + 31) >> 5;
                        for (int b = warp; b < nb; b += kWarpsPerCta) {
                            const int tt = (b << 5) + lane;
                            bool isl = false;
                            if (tt < nc) {
                                const S st = a.starts[cpos[tt]];
                                cstart[tt] = st;
                                isl = is_long_iv<S>(st, cend[tt], X);
                            }
                            const unsigned m = __ballot_sync(kFull, isl);
                            if (lane == 0) {
                                s_bmask[b] = m;
                                s_boff[b] = __popc(m);
                            }
                        }
                        __syncthreads();
                        block_excl_scan(s_boff, nb, s_wsum, &s_sum);
                        nl = s_sum;
                        for (int b = warp; b < nb; b += kWarpsPerCta) {
                            const unsigned m = s_bmask[b];
                            if ((m >> lane) & 1u) {
                                const int tt = (b << 5) + lane;
                                const int idx = s_boff[b] + __popc(m & lanemask_lt());
                                lpos[idx] = cpos[tt];
                                lend[idx] = cend[tt];
                            }
                        }
                        __syncthreads();
                        // nlm: long candidates from the tile's own gather (positions >= p_cut).  The
                        // lnu list: the others (from the long-interval list, at least 32768 long)
                        // that end before Q, i.e. possible misses for some query, in long-list order
                        // as their long-list indices (at most kLnu kept; a larger count makes every
                        // query filter them)
                        if (warp == 0) {
                            int w = 0, nm = 0;
                            for (int b0 = 0; b0 < nl; b0 += 32) {
                                const int k = b0 + lane;
                                const bool own = k < nl && (int64_t)lpos[k] >= pcut;
                                const bool f = k < nl && !own && lend[k] < Q;
                                const unsigned m = __ballot_sync(kFull, f);
                                const int slot = w + __popc(m & lanemask_lt());
                                if (f && slot < kLnu) {
                                    s_lnu_idx[slot] = k;
                                    s_lnu_end[slot] = lend[k];
                                }
                                w += __popc(m);
                                nm += __popc(__ballot_sync(kFull, own));
                            }
                            if (lane == 0) {
                                s_nlnu = w;
                                s_nlm = nm;
                            }
                        }
                        __syncthreads();
                        nlnu = s_nlnu;
                        nlm = s_nlm;
                    }
                    if (!EMIT && rec) {
                        // store the lists for the emit pass (header last field: 1 = usable)
                        for (int k = tid; k < nc; k += kThreads) {
                            g_cpos[k] = cpos[k];
                            g_cend[k] = cend[k];
                            g_cstart[k] = cstart[k];
                        }
                        for (int k = tid; k < nl; k += kThreads) {
                            g_lpos[k] = lpos[k];
                            g_lend[k] = lend[k];
                        }
                        for (int k = tid; k < nlnu && k < kLnu; k += kThreads) {
                            g_lnu_idx[k] = s_lnu_idx[k];
                            g_lnu_end[k] = s_lnu_end[k];
                        }
                        if (tid == 0) {
                            int32_t* hdr = reinterpret_cast<int32_t*>(rec);
                            hdr[0] = per_query ? -1 : nc;
                            hdr[1] = nl;
                            hdr[2] = nlnu;
                            hdr[3] = per_query ? 0 : 1;
                            hdr[4] = nlm;
                        }
                    }
                }
                if (per_query) nc = 0;
            }
            if (long_run && !rank_run) {
                // long queries share the tile's long-interval candidates (long pyramid)
                S mn = Lim<S>::hi;
                int32_t um = INT32_MIN;
                for (int i = r0 + tid; i < r1; i += kThreads) {
                    mn = q_s[i] < mn ? q_s[i] : mn;
                    um = q_u[i] > um ? q_u[i] : um;
                }
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) {
                    const S o = __shfl_xor_sync(kFull, mn, d);
                    mn = o < mn ? o : mn;
                    um = max(um, __shfl_xor_sync(kFull, um, d));
                }
                if (lane == 0) {
                    s_red[warp] = mn;
                    s_red3[warp] = um;
                }
                __syncthreads();
                S L = s_red[0];
                int32_t umx = s_red3[0];
#pragma unroll
                for (int w = 1; w < kWarpsPerCta; ++w) {
                    L = s_red[w] < L ? s_red[w] : L;
                    umx = max(umx, s_red3[w]);
                }
                if (warp == 0) {
                    const int64_t ch =
                        warp_first_pos_geq(a.long_pos, a.long_seg[g], a.long_seg[g + 1], (int64_t)umx + 1, lane);
                    if (lane == 0) s_cut[1] = ch;
                }
                __syncthreads();
                const int64_t c_lo = a.long_seg[g], c_hi = s_cut[1];
                nc = c_hi > c_lo ? gather_bfs<S>(a.PL, c_lo, c_hi - 1, L, cap, cpos, cend, lst, cnt, msk, s_wsum,
                                                 &s_n, &s_sum, a.long_pos)
                                 : 0;
                if (nc < 0) {
                    per_query = true;
                    nc = 0;
                }
            }
            if ((per_query || long_run) && !rank_run) {
                // per-query work differs widely in length: warps claim queries one at a time
                if (tid == 0) s_next = r0;
                __syncthreads();
                while (true) {
                    int i = 0;
                    if (lane == 0) i = atomicAdd(&s_next, 1);
                    i = __shfl_sync(kFull, i, 0);
                    if (i >= r1) break;
                    if (EMIT && q_cap[i] < 0) continue;  // outside the emitted window
                    if (per_query)
                        walk_query<S, EMIT>(a, q_s[i], (int64_t)q_u[i], lo, q_id[i], lane);
                    else
                        long_query<S, EMIT>(a, q_s[i], (int64_t)q_u[i], lo, q_id[i], cpos, cend, nc,
                                            EMIT ? (int64_t)q_h[i] : 0, EMIT ? q_off[i] : 0,
                                            EMIT ? (int64_t)q_cap[i] : 0, lane);
                }
            }
            if (!EMIT && !per_query && !long_run && !rank_run) {
                // count pass: one query per THREAD over the shared-memory lists
                for (int i = r0 + tid; i < r1; i += kThreads) {
                    const S qs = q_s[i];
                    const int32_t u = q_u[i];
                    uint32_t c = 0;
                    int head = 0;
                    if (u >= lo && nc > 0) {
                        int b0 = 0, b1 = nc;  // first candidate at or below u
                        while (b0 < b1) {
                            const int mid = (b0 + b1) >> 1;
                            if (cpos[mid] > u) b0 = mid + 1;
                            else b1 = mid;
                        }
                        const int t0 = b0;
                        // part A and the head run: candidates whose start is within X of qs, i.e.
                        // start >= thr (thr = qs - X, clamped to the coordinate range)
                        const S thr = near_threshold<S>(qs, X);
                        int t = t0;
                        // the head run: consecutive positions u, u-1, ... that are hits
                        while (t < nc && cstart[t] >= thr && cend[t] >= qs && cpos[t] == u - (t - t0)) ++t;
                        head = t - t0;
                        c = (uint32_t)head;
                        bool open = t == nc || cstart[t] < thr;  // the head may go on below the split
                        for (; t < nc && cstart[t] >= thr; ++t) c += cend[t] >= qs ? 1u : 0u;
                        const int tsplit = t;
                        for (; open && t < nc; ++t) {  // a head run reaching into the long candidates
                            if (cpos[t] == u - (t - t0) && cend[t] >= qs) ++head;
                            else open = false;
                        }
                        // part B: long candidates below the split are hits unless they end before qs:
                        // the tile's own ones are checked one by one, those from the long-interval
                        // list are all hits but the lnu entries that end before qs
                        if (tsplit < nc && nl > 0) {
                            const int32_t psplit = cpos[tsplit];
                            int l0 = 0, l1 = nl;
                            while (l0 < l1) {
                                const int mid = (l0 + l1) >> 1;
                                if (lpos[mid] > psplit) l0 = mid + 1;
                                else l1 = mid;
                            }
                            const int b2 = max(l0, nlm);
                            for (int k = l0; k < b2; ++k) c += lend[k] >= qs ? 1u : 0u;
                            if (nlnu <= kLnu) {
                                int miss = 0;  // lnu entries at or after b2
                                for (int k = 0; k < nlnu; ++k)
                                    miss += (s_lnu_idx[k] >= b2 && s_lnu_end[k] < qs) ? 1 : 0;
                                c += (uint32_t)(nl - b2 - miss);
                            } else {
                                for (int k = b2; k < nl; ++k) c += lend[k] >= qs ? 1u : 0u;
                            }
                        }
                    }
                    a.counts[q_id[i]] = c;
                    a.heads[q_id[i]] = head;
                }
            }
            if (EMIT && !per_query && !long_run) {
                // emit, step 1: one query per THREAD finds where its hits lie in the lists
                for (int i = r0 + tid; i < r1; i += kThreads) {
                    const S qs = q_s[i];
                    const int32_t u = q_u[i];
                    int ta = nc, tsplit = nc, lb = nl;
                    if (a.end_sorted) q_h[i] = 0;  // no candidate: no head (set below otherwise)
                    if (u >= lo && nc > 0) {
                        int b0 = 0, b1 = nc;  // first candidate at or below u
                        while (b0 < b1) {
                            const int mid = (b0 + b1) >> 1;
                            if (cpos[mid] > u) b0 = mid + 1;
                            else b1 = mid;
                        }
                        const int t0 = b0;
                        const S thr = near_threshold<S>(qs, X);
                        // starts do not increase along the list: first t in [from, nc) whose start
                        // is below key
                        auto first_start_below = [&](int from, S key) {
                            int l0 = from, l1 = nc;
                            while (l0 < l1) {
                                const int mid = (l0 + l1) >> 1;
                                if (cstart[mid] >= key) l0 = mid + 1;
                                else l1 = mid;
                            }
                            return l0;
                        };
                        int h = q_h[i];
                        if (a.end_sorted) {
                            // counted from ranks: the head run (consecutive positions u, u - 1, ...
                            // that are hits) is found here.  Positions from u down to the last start
                            // >= qs end at or after qs (no interval has start > end), so they are all
                            // in the list and all hits; the run then goes on while positions stay
                            // consecutive and hit.
                            int t = first_start_below(t0, qs);
                            while (t < nc && cpos[t] == u - (t - t0) && cend[t] >= qs) ++t;
                            h = t - t0;
                            q_h[i] = h;
                        }
                        ta = t0 + (h < nc - t0 ? h : nc - t0);
                        tsplit = first_start_below(ta, thr);
                        const int tb = max(tsplit, ta);
                        if (tb < nc && nl > 0) {
                            const int32_t pb = cpos[tb];
                            int l0 = 0, l1 = nl;
                            while (l0 < l1) {
                                const int mid = (l0 + l1) >> 1;
                                if (lpos[mid] > pb) l0 = mid + 1;
                                else l1 = mid;
                            }
                            lb = l0;
                        }
                    }
                    q_ta[i] = ta;
                    q_tsplit[i] = tsplit;
                    q_lb[i] = lb;
                }
                __syncthreads();
                // the lists now only feed the writes: turn positions into the values written
                // (contig-local positions, or payloads), once per run instead of once per hit
                for (int k = tid; k < nc; k += kThreads) {
                    const int32_t p = cpos[k];
                    cpos[k] = a.values ? a.data[p] : p - (int32_t)lo;
                }
                for (int k = tid; k < nl; k += kThreads) {
                    const int32_t p = lpos[k];
                    lpos[k] = a.values ? a.data[p] : p - (int32_t)lo;
                }
                __syncthreads();
            }
            for (int i = r0 + warp; EMIT && !per_query && !long_run && i < r1; i += kWarpsPerCta) {
                // emit, step 2: one query per WARP writes its hits, coalesced
                const S qs = q_s[i];
                const int64_t u = q_u[i];
                const int64_t h = q_h[i];
                const int64_t capq = q_cap[i];
                if (capq < 0) continue;  // outside the emitted window
                int32_t* dst = a.out + q_off[i];
                if (h > capq) {
                    if (lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
                    continue;
                }
                for (int64_t r = lane; r < h; r += 32) {
                    const int64_t pos = (a.order == kOrderIdxsCpp) ? (u - h + 1 + r) : (u - r);
                    dst[r] = a.values ? a.data[pos] : (int32_t)(pos - lo);
                }
                const unsigned lt = lanemask_lt();
                int32_t* d = dst + h;            // next write
                int64_t room = capq - h;         // writes left for this query
                bool bad = false;
                // part A: candidates near qs after the head, two 32-wide slices per round
                {
                    const int ta = q_ta[i], tsplit = q_tsplit[i];
                    for (int kk = ta; kk < tsplit; kk += 64) {
                        const int t0 = kk + lane, t1 = t0 + 32;
                        const bool h0 = t0 < tsplit && cend[t0] >= qs;
                        const bool h1 = t1 < tsplit && cend[t1] >= qs;
                        const int32_t v0 = h0 ? cpos[t0] : 0, v1 = h1 ? cpos[t1] : 0;
                        const unsigned m0 = __ballot_sync(kFull, h0), m1 = __ballot_sync(kFull, h1);
                        const int c0 = __popc(m0), c = c0 + __popc(m1);
                        if (c > room) {
                            bad = true;
                            break;
                        }
                        if (h0) d[__popc(m0 & lt)] = v0;
                        if (h1) d[c0 + __popc(m1 & lt)] = v1;
                        d += c;
                        room -= c;
                    }
                }
                // part B: the long candidates from lb on.  Those of the tile's own gather ([lb, b2))
                // are filtered one by one.  Those from the long-interval list ([b2, nl)) are all
                // hits but the few lnu entries (ending before the run's largest qs) that end
                // before this query's start: with the copy mode on, that section is copied as runs
                // between those entries, else it is filtered too
                const int lb = q_lb[i];
                const int b2 = max(lb, nlm);
                int fend = a.emit_copy && nlnu <= kLnu ? b2 : nl;  // filtered: [lb, fend)
                for (int kk = lb; !bad && kk < fend; kk += 128) {
                    // 128 candidates per round as four independent 32-wide slices, so their
                    // shared-memory reads and ballots overlap instead of chaining; only the last
                    // round checks the range end
                    bool hit[4];
                    int32_t pv[4];
                    unsigned m[4];
                    if (kk + 128 <= fend) {
#pragma unroll
                        for (int s2 = 0; s2 < 4; ++s2) {
                            const int tt = kk + 32 * s2 + lane;
                            hit[s2] = lend[tt] >= qs;
                            pv[s2] = lpos[tt];
                        }
                    } else {
#pragma unroll
                        for (int s2 = 0; s2 < 4; ++s2) {
                            const int tt = kk + 32 * s2 + lane;
                            const bool in = tt < fend;
                            hit[s2] = in && lend[tt] >= qs;
                            pv[s2] = in ? lpos[tt] : 0;
                        }
                    }
#pragma unroll
                    for (int s2 = 0; s2 < 4; ++s2) m[s2] = __ballot_sync(kFull, hit[s2]);
                    const int c0 = __popc(m[0]), c1 = c0 + __popc(m[1]), c2 = c1 + __popc(m[2]);
                    const int c = c2 + __popc(m[3]);
                    if (c > room) {
                        bad = true;
                        break;
                    }
                    if (hit[0]) d[__popc(m[0] & lt)] = pv[0];
                    if (hit[1]) d[c0 + __popc(m[1] & lt)] = pv[1];
                    if (hit[2]) d[c1 + __popc(m[2] & lt)] = pv[2];
                    if (hit[3]) d[c2 + __popc(m[3] & lt)] = pv[3];
                    d += c;
                    room -= c;
                }
                if (!bad && fend < nl) {
                    // the long-interval list's section: misses are the lnu entries at or after b2
                    // that end before qs, in long-list order
                    unsigned mm[kLnu / 32];
                    int nmiss = 0;
#pragma unroll
                    for (int j = 0; j < kLnu / 32; ++j) {
                        mm[j] = 0u;
                        if (32 * j < nlnu) {  // warp-uniform
                            const int k = 32 * j + lane;
                            const bool ms = k < nlnu && s_lnu_idx[k] >= b2 && s_lnu_end[k] < qs;
                            mm[j] = __ballot_sync(kFull, ms);
                            nmiss += __popc(mm[j]);
                        }
                    }
                    const int len = nl - b2 - nmiss;
                    if (len > room) {
                        bad = true;
                    } else {
                        // runs between the misses, 4-byte warp stores
                        int at = b2;
#pragma unroll
                        for (int j = 0; j < kLnu / 32; ++j) {
                            unsigned mj = mm[j];
                            while (mj) {
                                const int mi = s_lnu_idx[32 * j + __ffs(mj) - 1];
                                mj &= mj - 1;
                                warp_copy4(d, lpos + at, mi - at, lane);
                                d += mi - at;
                                at = mi + 1;
                            }
                        }
                        warp_copy4(d, lpos + at, nl - at, lane);
                        d += nl - at;
                        room -= len;
                    }
                }
                if (bad && lane == 0) atomicCAS(a.d_err, kDevOk, kDevOverflow);
            }
            __syncthreads();
            r0 = r1;
        }
    }
}

// ---- query keys: (class|contig, end) -------------------------------------------------
// Smallest and largest query end as offset-binary (unsigned order = signed order).
template <typename S>
__global__ void k_qend_minmax(const S* __restrict__ qe, int64_t nq, unsigned long long* __restrict__ mm) {
    unsigned long long lo = ~0ull, hi = 0ull;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long v = (unsigned long long)(int64_t)qe[q] ^ 0x8000000000000000ull;
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long a = __shfl_xor_sync(kFull, lo, d), b = __shfl_xor_sync(kFull, hi, d);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(&mm[0], lo);
        atomicMax(&mm[1], hi);
    }
}

// Class code of a query (see code_is_long): a query with start > end takes the long-query path,
// which does not need start <= end.
__device__ __forceinline__ uint32_t query_code(int32_t g, int G, bool inverted, bool is_long) {
    if (g < 0 || g >= G) return 3u * (uint32_t)G;
    return (uint32_t)g + (inverted ? 2u * (uint32_t)G : is_long ? (uint32_t)G : 0u);
}

// The packed key's layout from the batch's smallest and largest end (offset-binary): the end
// offset loses `shift` low bits so that code and end fit 24 bits; out = {shift, end bits}.
__global__ void k_pack_params(const unsigned long long* __restrict__ mm, int code_bits, int* __restrict__ out) {
    if (threadIdx.x != 0) return;
    const unsigned long long span = mm[1] - mm[0];
    int span_bits = 0;
    while (span_bits < 64 && (span >> span_bits) != 0) ++span_bits;
    const int shift = max(8, span_bits + code_bits - 24);
    out[0] = shift;
    out[1] = max(0, span_bits - shift);
}

// One 32-bit key per query: class code above the end's offset from the batch's smallest end,
// shifted right by `shift` (tiles need queries grouped by class and contig and close in
// position, not exactly ordered).  Also writes (start, end) interleaved for the prepare pass
// and, with ghist, the counts of the key's three low bytes for the radix sort (the key has at
// most 24 bits; byte 3 is counted by the caller).  Grid-stride, four queries per thread in
// flight so that enough loads are outstanding to cover memory latency.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_qkeys_packed(const S* __restrict__ qs, const S* __restrict__ qe,
                                                           const int32_t* __restrict__ qc, int64_t nq,
                                                           int64_t long_len, int G,
                                                           const unsigned long long* __restrict__ mm, int shift,
                                                           int ebits, const int* __restrict__ d_pack,
                                                           uint32_t* __restrict__ key, uint32_t* __restrict__ pay,
                                                           S* __restrict__ qpair, uint32_t* __restrict__ ghist) {
    constexpr int U = 4;
    __shared__ uint32_t h[3 * 256];
    const int tid = threadIdx.x;
    if (ghist) {
        for (int i = tid; i < 3 * 256; i += kThreads) h[i] = 0;
        __syncthreads();
    }
    if (d_pack) {  // worked out on the device
        shift = d_pack[0];
        ebits = d_pack[1];
    }
    const unsigned long long m0 = mm[0];
    const int64_t stride = (int64_t)gridDim.x * kThreads * U;
    for (int64_t q0 = (int64_t)blockIdx.x * kThreads * U + tid; q0 < nq; q0 += stride) {
        S s[U], e[U];
        int32_t g[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t q = q0 + u * kThreads;
            g[u] = 0;
            s[u] = 0;
            e[u] = 0;
            if (q < nq) {
                g[u] = qc ? qc[q] : 0;
                s[u] = qs[q];
                e[u] = qe[q];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t q = q0 + u * kThreads;
            if (q >= nq) continue;
            const bool is_long = ((double)e[u] - (double)s[u] + 1.0) > (double)long_len;
            const uint32_t code = query_code(g[u], G, s[u] > e[u], is_long);
            const unsigned long long rel = ((unsigned long long)(int64_t)e[u] ^ 0x8000000000000000ull) - m0;
            const uint32_t k = (code << ebits) | (uint32_t)(rel >> shift);
            key[q] = k;
            pay[q] = (uint32_t)q;
            if constexpr (sizeof(S) == 4) {
                reinterpret_cast<int2*>(qpair)[q] = make_int2((int)s[u], (int)e[u]);
            } else {
                reinterpret_cast<longlong2*>(qpair)[q] = make_longlong2((long long)s[u], (long long)e[u]);
            }
            if (ghist) {
                atomicAdd(&h[k & 255u], 1u);
                atomicAdd(&h[256 + ((k >> 8) & 255u)], 1u);
                atomicAdd(&h[512 + ((k >> 16) & 255u)], 1u);
            }
        }
    }
    if (ghist) {
        __syncthreads();
        for (int i = tid; i < 3 * 256; i += kThreads)
            if (h[i]) atomicAdd(&ghist[i], h[i]);
        if (blockIdx.x == 0 && tid == 0) atomicAdd(&ghist[3 * 256], (uint32_t)nq);  // byte 3: all zero
    }
}

template <typename S>
__global__ void k_qkeys(const S* __restrict__ qs, const S* __restrict__ qe, const int32_t* __restrict__ qc,
                        int64_t nq, int64_t long_len, int G, uint32_t* w0, uint32_t* w1, uint32_t* wc,
                        uint32_t* __restrict__ pay) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    const int32_t g = qc ? qc[q] : 0;
    const bool is_long = ((double)qe[q] - (double)qs[q] + 1.0) > (double)long_len;
    // The end key drops its lowest byte: tiles need queries grouped by class and contig and
    // close in position, not exactly ordered, and a constant digit costs no sort pass.
    if constexpr (sizeof(S) == 4) {
        w0[q] = ((uint32_t)qe[q] ^ 0x80000000u) & ~0xffu;
    } else {
        const uint64_t b = (uint64_t)qe[q] ^ 0x8000000000000000ull;
        w0[q] = (uint32_t)b & ~0xffu;
        w1[q] = (uint32_t)(b >> 32);
    }
    wc[q] = query_code(g, G, qs[q] > qe[q], is_long);
    pay[q] = (uint32_t)q;
}

constexpr int kPrepWindow = 2048;  // starts staged per block by the cooperative search

// Prepare the sorted batch: gather each query's record and find its upper bound.  A block
// holds 256 consecutive sorted queries; when they share one class/contig code (the usual
// case) the block searches only its smallest and largest end with the index's accelerator,
// stages the starts between the two answers in shared memory and resolves every query
// there.  Otherwise each query searches on its own.
template <typename S>
__global__ void __launch_bounds__(kThreads, 6) k_qprep(const uint32_t* __restrict__ pay,
                                                    const uint32_t* __restrict__ wc, int code_shift,
                                                    const int* __restrict__ d_pack,
                                                    const S* __restrict__ qs, const S* __restrict__ qe,
                                                    const S* __restrict__ qpair,
                                                    int64_t nq, MapView<S> m, UbView<S> U,
                                                    S* __restrict__ sq_s, int32_t* __restrict__ sq_u,
                                                    uint32_t* __restrict__ sq_c, int32_t* __restrict__ sq_id,
                                                    int* d_err, int64_t long_split,
                                                    const int32_t* __restrict__ long_pos,
                                                    const int64_t* __restrict__ long_seg,
                                                    int64_t* __restrict__ blk_cut, const S* __restrict__ end_sorted,
                                                    uint32_t* __restrict__ counts) {
    __shared__ S win[kPrepWindow];
    __shared__ S win2[kPrepWindow];  // the sorted ends between the block's two ranks
    __shared__ S s_mn[kWarpsPerCta], s_mx[kWarpsPerCta], s_mq[kWarpsPerCta], s_xq[kWarpsPerCta];
    __shared__ int64_t s_a, s_b, s_ra, s_rb;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (d_pack) code_shift = d_pack[1];  // the packed key's end bits, worked out on the device
    const int64_t jb = (int64_t)blockIdx.x * kThreads;
    const int64_t j = jb + tid;
    const int64_t jl = (jb + kThreads < nq ? jb + kThreads : nq) - 1;  // last query of the block
    const bool valid = j < nq;
    // the class code is the key word itself, or its top bits when the key is packed
    uint32_t orig = 0, cw = 0;
    S v = 0, vs = 0;
    if (valid) {
        orig = pay[j];
        cw = wc[j] >> code_shift;
        if (qpair) {  // one 8- or 16-byte load of the record
            if constexpr (sizeof(S) == 4) {
                const int2 r = reinterpret_cast<const int2*>(qpair)[orig];
                vs = r.x;
                v = r.y;
            } else {
                const longlong2 r = reinterpret_cast<const longlong2*>(qpair)[orig];
                vs = r.x;
                v = r.y;
            }
        } else {
            v = qe[orig];
            vs = qs[orig];
        }
    }
    const uint32_t cfirst = wc[jb] >> code_shift, clast = wc[jl] >> code_shift;
    const bool uniform = cfirst == clast && cfirst < 3u * (uint32_t)m.G;  // sorted: one code
    int g = code_contig(valid ? cw : cfirst, m.G);
    bool bad = false;
    if (valid && cw >= 3u * (uint32_t)m.G) {
        atomicCAS(d_err, kDevOk, kDevBadContig);
        bad = true;
    }
    const int64_t lo = m.seg[g];
    const int64_t n = m.seg[g + 1] - lo;
    int64_t u = -1;
    bool done = false;
    if (blk_cut && tid == 0 && !uniform) blk_cut[2 * blockIdx.x] = -1;
    // queries with start <= end (short and long classes) are counted here from two ranks when
    // the index keeps its sorted ends: count = #(start <= qe) - #(end < qs), as no interval
    // has start > end
    const bool rank_count = counts != nullptr && end_sorted != nullptr;
    const bool rank_block = rank_count && uniform && cfirst < 2u * (uint32_t)m.G && n > 0;
    if (uniform) {
        S mn = valid ? v : Lim<S>::hi, mx = valid ? v : Lim<S>::lo, mq = valid ? vs : Lim<S>::hi;
        S xq = valid ? vs : Lim<S>::lo;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const S o = __shfl_xor_sync(kFull, mn, d);
            mn = o < mn ? o : mn;
            const S p = __shfl_xor_sync(kFull, mx, d);
            mx = p > mx ? p : mx;
            const S r = __shfl_xor_sync(kFull, mq, d);
            mq = r < mq ? r : mq;
            const S x = __shfl_xor_sync(kFull, xq, d);
            xq = x > xq ? x : xq;
        }
        if (lane == 0) {
            s_mn[warp] = mn;
            s_mx[warp] = mx;
            s_mq[warp] = mq;
            s_xq[warp] = xq;
        }
        __syncthreads();
        if (rank_block && (warp == 2 || warp == 3)) {
            // the block's ranks lie between those of its smallest (warp 2) and largest (warp 3) qs
            S key = warp == 2 ? s_mq[0] : s_xq[0];
            for (int w = 1; w < kWarpsPerCta; ++w)
                key = warp == 2 ? (s_mq[w] < key ? s_mq[w] : key) : (s_xq[w] > key ? s_xq[w] : key);
            const int64_t r = warp_first_geq<S, S>(end_sorted, lo, lo + n, key, lane);
            if (lane == 0) {
                if (warp == 2) s_ra = r;
                else s_rb = r;
            }
        }
        if (blk_cut && warp == 1) {
            // for the tile of these queries (warp 1, beside warp 0's searches): p_cut = first
            // position whose start is within long_split of the smallest qs, and the first
            // long-list index at or after it
            int64_t pc = -1, ch = -1;
            if (cfirst < (uint32_t)m.G && n > 0) {
                S L = s_mq[0];
                for (int w = 1; w < kWarpsPerCta; ++w) L = s_mq[w] < L ? s_mq[w] : L;
                pc = warp_first_near<S>(m.starts, lo, lo + n, L, long_split, lane);
                ch = warp_first_pos_geq(long_pos, long_seg[g], long_seg[g + 1], pc, lane);
            }
            if (lane == 0) {
                blk_cut[2 * blockIdx.x] = pc;
                blk_cut[2 * blockIdx.x + 1] = ch;
            }
        }
        if ((warp == 4 || warp == 5) && n > 0) {
            // warp 4: upper bound of the block's smallest end, warp 5: of its largest
            S x = warp == 4 ? s_mn[0] : s_mx[0];
            for (int w = 1; w < kWarpsPerCta; ++w)
                x = warp == 4 ? (s_mn[w] < x ? s_mn[w] : x) : (s_mx[w] > x ? s_mx[w] : x);
            const int64_t r = warp_ub(U, g, m.starts + lo, n, x, lane);
            if (lane == 0) {
                if (warp == 4) s_a = r;
                else s_b = r;
            }
        }
        __syncthreads();
        // both windows (the starts between the two upper bounds, the sorted ends between the two
        // ranks) are staged together, behind one barrier
        const int64_t a0 = s_a < 0 ? 0 : s_a, b0 = s_b;
        const bool win_ok = n > 0 && b0 >= a0 && b0 - a0 + 1 <= kPrepWindow;
        const int64_t A = rank_block ? s_ra : 0, B = rank_block ? s_rb : 0;
        const bool staged = rank_block && B - A <= kPrepWindow;
        if (win_ok)
            for (int64_t k = a0 + tid; k <= b0; k += kThreads) win[k - a0] = m.starts[lo + k];
        if (staged)
            for (int64_t k = tid; k < B - A; k += kThreads) win2[k] = end_sorted[A + k];
        if (win_ok || staged) __syncthreads();
        if (n > 0) {
            if (b0 < a0) {
                done = true;  // every end of the block precedes the contig's first start
                u = -1;
            } else if (win_ok) {
                if (valid && !bad) u = a0 + ub_range(win, (int64_t)0, b0 - a0, v);
                done = true;
            } else if (valid && !bad) {
                u = ub_range(m.starts + lo, a0, b0, v);  // answer lies between the block's two
                done = true;
            }
        } else {
            done = true;
        }
        if (rank_block) {
            if (valid) {
                int64_t b0 = 0, b1 = B - A;  // first index of the window whose end is >= qs
                while (b0 < b1) {
                    const int64_t mid = (b0 + b1) >> 1;
                    const S e = staged ? win2[mid] : end_sorted[A + mid];
                    if (e < vs) b0 = mid + 1;
                    else b1 = mid;
                }
                const int64_t below = A + b0 - lo;  // ends before qs
                counts[orig] = (!bad && u + 1 > below) ? (uint32_t)(u + 1 - below) : 0u;
            }
        }
    }
    if (!valid) return;
    if (!done && !bad && n > 0) {
        const S* tr = (U.mode == 1) ? U.eytz_keys + (int64_t)g * U.eytz_n : nullptr;
        u = ub_search(U, g, m.starts + lo, n, v, tr);
    }
    if (rank_count && !rank_block && (bad || cw < 2u * (uint32_t)m.G)) {
        // a block of mixed classes: each query searches its rank on its own
        int64_t b0 = 0, b1 = bad ? 0 : n;
        while (b0 < b1) {
            const int64_t mid = (b0 + b1) >> 1;
            if (end_sorted[lo + mid] < vs) b0 = mid + 1;
            else b1 = mid;
        }
        counts[orig] = (!bad && u + 1 > b0) ? (uint32_t)(u + 1 - b0) : 0u;
    }
    sq_s[j] = vs;
    sq_u[j] = (int32_t)(lo + u);
    sq_c[j] = cw;
    sq_id[j] = (int32_t)orig;
}

// First index k in [lo, hi) of the ascending array arr with arr[k] >= key (strict: > key), for
// every thread's key of a block of 256 sorted queries.  A uniform block (one contig, keys
// close together) finds the ranks of its smallest and largest key with one warp each, stages
// the entries between them in shared memory (win, kPrepWindow slots) when they fit and
// resolves each key there; otherwise each key searches [lo, hi) on its own.  Block-wide.
template <typename S>
__device__ int64_t block_rank(const S* __restrict__ arr, int64_t lo, int64_t hi, S key, bool strict, bool valid,
                              bool uniform, S* win, S* s_kmin, S* s_kmax, int64_t* s_r, int tid, int lane,
                              int warp) {
    // strict: arr > key, i.e. arr >= key + 1 (no key + 1 above the largest value)
    const bool none = strict && key == Lim<S>::hi;
    const S k2 = (strict && !none) ? (S)(key + 1) : key;
    if (!uniform) {
        if (!valid || none) return hi;
        int64_t b0 = lo, b1 = hi;
        while (b0 < b1) {
            const int64_t mid = (b0 + b1) >> 1;
            if (arr[mid] < k2) b0 = mid + 1;
            else b1 = mid;
        }
        return b0;
    }
    S mn = (valid && !none) ? k2 : Lim<S>::hi, mx = (valid && !none) ? k2 : Lim<S>::lo;
    const bool any_none = __syncthreads_or(valid && none);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        const S o = __shfl_xor_sync(kFull, mn, d);
        mn = o < mn ? o : mn;
        const S p = __shfl_xor_sync(kFull, mx, d);
        mx = p > mx ? p : mx;
    }
    if (lane == 0) {
        s_kmin[warp] = mn;
        s_kmax[warp] = mx;
    }
    __syncthreads();
    if (warp < 2) {
        S k = warp == 0 ? s_kmin[0] : s_kmax[0];
        for (int w = 1; w < kWarpsPerCta; ++w)
            k = warp == 0 ? (s_kmin[w] < k ? s_kmin[w] : k) : (s_kmax[w] > k ? s_kmax[w] : k);
        const int64_t r = warp_first_geq<S, S>(arr, lo, hi, k, lane);
        if (lane == 0) s_r[warp] = r;
    }
    __syncthreads();
    const int64_t A = s_r[0], B = any_none ? hi : s_r[1];
    const bool staged = B - A <= kPrepWindow;
    if (staged)
        for (int64_t k = tid; k < B - A; k += kThreads) win[k] = arr[A + k];
    __syncthreads();
    int64_t r = hi;
    if (valid && !none) {
        int64_t b0 = 0, b1 = B - A;
        while (b0 < b1) {
            const int64_t mid = (b0 + b1) >> 1;
            const S e = staged ? win[mid] : arr[A + mid];
            if (e < k2) b0 = mid + 1;
            else b1 = mid;
        }
        r = A + b0;
    }
    __syncthreads();  // win and the reductions are reused by the next call
    return r;
}

// coverage of sorted queries from ranks and prefix sums, for an index without intervals with
// start > end and queries with start <= end.  Over the hits {start <= qe} minus {end < qs}:
//   count = a_u - r_qs
//   sum min(end, qe) = PE[r_qe] - PE[r_qs] + qe * (a_u - r_qe)
//   sum max(start, qs) = PS[a_u] - PS[ls] + qs * (ls - r_qs)
// with a_u = 1 + the upper bound of qe, r_qs / r_qe the first sorted ends >= qs / > qe, ls the
// first start >= qs, and PS / PE the exclusive prefix sums (mod 2^64) of the starts and of
// the sorted ends.  The coverage, sum min - sum max, wraps as the coordinate type does.
template <typename S>
__global__ void __launch_bounds__(kThreads) k_cov_ranks(const S* __restrict__ sq_s, const int32_t* __restrict__ sq_u,
                                                        const uint32_t* __restrict__ sq_c,
                                                        const int32_t* __restrict__ sq_id, const S* __restrict__ qe,
                                                        int64_t nq, MapView<S> m, const S* __restrict__ end_sorted,
                                                        const uint64_t* __restrict__ ps_start,
                                                        const uint64_t* __restrict__ ps_end,
                                                        uint64_t* __restrict__ count, S* __restrict__ cov) {
    __shared__ S win[kPrepWindow];
    __shared__ S s_kmin[kWarpsPerCta], s_kmax[kWarpsPerCta];
    __shared__ int64_t s_r[2];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t jb = (int64_t)blockIdx.x * kThreads, j = jb + tid;
    const int64_t jl = (jb + kThreads < nq ? jb + kThreads : nq) - 1;
    const bool valid = j < nq;
    const uint32_t cfirst = sq_c[jb], clast = sq_c[jl];
    const bool uniform = cfirst == clast && cfirst < 2u * (uint32_t)m.G;  // one contig, start <= end
    const uint32_t cw = valid ? sq_c[j] : cfirst;
    const bool bad = cw >= 2u * (uint32_t)m.G;  // bad contig (reported by the prepare pass)
    const int g = code_contig(cw, m.G);
    const int64_t lo = m.seg[g], hi = m.seg[g + 1];
    S s0 = 0, e0 = 0;
    int64_t u = lo - 1;
    int32_t id = 0;
    if (valid) {
        s0 = sq_s[j];
        u = sq_u[j];
        id = sq_id[j];
        e0 = qe[id];
    }
    const bool live = valid && !bad;
    const int64_t r_qs = block_rank<S>(end_sorted, lo, hi, s0, false, live, uniform, win, s_kmin, s_kmax, s_r, tid,
                                       lane, warp);
    const int64_t r_qe = block_rank<S>(end_sorted, lo, hi, e0, true, live, uniform, win, s_kmin, s_kmax, s_r, tid,
                                       lane, warp);
    const int64_t ls = block_rank<S>(m.starts, lo, hi, s0, false, live, uniform, win, s_kmin, s_kmax, s_r, tid,
                                     lane, warp);
    if (!valid) return;
    if (!live) {
        count[id] = 0;
        cov[id] = 0;
        return;
    }
    const int64_t a_u = u + 1;
    const uint64_t qe64 = (uint64_t)(int64_t)e0, qs64 = (uint64_t)(int64_t)s0;
    const uint64_t smin_sum = ps_end[r_qe] - ps_end[r_qs] + qe64 * (uint64_t)(a_u - r_qe);
    const uint64_t smax_sum = ps_start[a_u] - ps_start[ls] + qs64 * (uint64_t)(ls - r_qs);
    count[id] = (uint64_t)(a_u - r_qs);
    cov[id] = (S)(smin_sum - smax_sum);
}

// upper bounds in the original query order (plain path with an accelerator, tests).  With the
// Eytzinger provider each block first stages the top `top_n` slots (whole levels) of every
// contig's tree in shared memory; the descent continues in global memory below them.
template <typename S>
__global__ void k_ub_plain(const S* __restrict__ qe, const int32_t* __restrict__ qc, int64_t nq,
                           MapView<S> m, UbView<S> U, int32_t* __restrict__ out, int* d_err, int top_n) {
    extern __shared__ __align__(16) unsigned char smem[];
    S* top = reinterpret_cast<S*>(smem);
    if (U.mode == 1 && top_n > 0) {
        for (int64_t i = threadIdx.x; i < (int64_t)m.G * top_n; i += blockDim.x) {
            const int64_t g = i / top_n, k = i - g * top_n;
            top[i] = U.eytz_keys[g * U.eytz_n + k];
        }
        __syncthreads();
    }
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    int g = qc ? qc[q] : 0;
    if (g < 0 || g >= m.G) {
        atomicCAS(d_err, kDevOk, kDevBadContig);
        out[q] = -1;
        return;
    }
    const int64_t lo = m.seg[g], n = m.seg[g + 1] - lo;
    const S* tr = (U.mode == 1) ? U.eytz_keys + (int64_t)g * U.eytz_n : nullptr;
    out[q] = (int32_t)ub_search(U, g, m.starts + lo, n, qe[q], tr, top + (int64_t)g * top_n, (int64_t)top_n);
}

// Upper bounds of sorted queries back to the original order: contig-local position or -1.
__global__ void k_ub_scatter(const int32_t* __restrict__ sq_u, const uint32_t* __restrict__ sq_c,
                             const int32_t* __restrict__ sq_id, int64_t nq, const int64_t* __restrict__ seg, int G,
                             int32_t* __restrict__ out) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    const uint32_t c = sq_c[j];
    const int32_t id = sq_id[j];
    if (c >= 3u * (uint32_t)G) {  // a contig outside [0, G): reported by the prepare kernel
        out[id] = -1;
        return;
    }
    out[id] = sq_u[j] - (int32_t)seg[code_contig(c, G)];
}

// ---- learned upper-bound model: GPU least squares ---------------------------------------
// Per contig: the sorted starts cut into equal-count leaves whose first keys form the root;
// per leaf a least-squares line of position on key (centred on the contig's mean key), then
// the leaf's max errors.

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    return v;
}

__device__ double block_sum(double v, double* red) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    return t;
}

// acc[g] += sum of the contig's keys (their mean conditions the leaf fits).
template <typename S>
__global__ void k_key_sums(const S* __restrict__ starts, const int64_t* __restrict__ seg, int G,
                           double* __restrict__ acc) {
    __shared__ double red[32];
    for (int g = blockIdx.y; g < G; g += gridDim.y) {
        const int64_t lo = seg[g], n = seg[g + 1] - lo;
        double a0 = 0;
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
            a0 += (double)starts[lo + k];
        a0 = block_sum(a0, red);
        if (threadIdx.x == 0) atomicAdd(&acc[g], a0);
    }
}

// The root of the learned model: each leaf's first key.
template <typename S>
__global__ void k_leaf_keys(const S* __restrict__ starts, const int64_t* __restrict__ seg,
                            const int32_t* __restrict__ leaf_contig, const int32_t* __restrict__ leaf_pos, int total,
                            S* __restrict__ leaf_key) {
    const int L = blockIdx.x * blockDim.x + threadIdx.x;
    if (L >= total) return;
    const int g = leaf_contig[L];
    const int64_t lo = seg[g], n = seg[g + 1] - lo;
    leaf_key[L] = n > 0 ? starts[lo + leaf_pos[L]] : Lim<S>::lo;
}

// One warp per leaf: mean key, least-squares slope of position on key, then the leaf's max
// errors under that line (the same prediction formula as the query, ub_search).
template <typename S>
__global__ void __launch_bounds__(kThreads) k_leaf_fit(const S* __restrict__ starts, const int64_t* __restrict__ seg,
                                                       const int32_t* __restrict__ leaf_contig,
                                                       const int32_t* __restrict__ leaf_base,
                                                       const int32_t* __restrict__ bnd, const double* __restrict__ mean_x,
                                                       LeafModel* __restrict__ leaves, int total) {
    const int lane = threadIdx.x & 31;
    const int L = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (L >= total) return;  // warp-uniform
    const int g = leaf_contig[L];
    const int64_t lo = seg[g];
    const int l = L - leaf_base[g];
    const int nl = leaf_base[g + 1] - leaf_base[g];
    const int64_t a = bnd[L];
    const int64_t b = (l + 1 < nl) ? (int64_t)bnd[L + 1] : (seg[g + 1] - lo);
    const int64_t cnt = b - a;
    LeafModel M;
    if (cnt <= 0) {
        if (lane == 0) {
            M.x0 = 0;
            M.slope = 0;
            M.y0 = (double)a;
            M.err_lo = 1;
            M.err_hi = 1;
            leaves[L] = M;
        }
        return;
    }
    const double mx = mean_x[g];
    double sx = 0;
    for (int64_t k = a + lane; k < b; k += 32) sx += (double)starts[lo + k] - mx;
    sx = warp_sum(sx);
    const double x0 = sx / (double)cnt;
    const double y0 = 0.5 * (double)(a + b - 1);
    double sxy = 0, sxx = 0;
    for (int64_t k = a + lane; k < b; k += 32) {
        const double dx = (double)starts[lo + k] - mx - x0, dy = (double)k - y0;
        sxy += dx * dy;
        sxx += dx * dx;
    }
    sxy = warp_sum(sxy);
    sxx = warp_sum(sxx);
    const double slope = (sxx > 0.0 && sxy > 0.0) ? sxy / sxx : 0.0;
    int elo = 0, ehi = 0;
    for (int64_t k = a + lane; k < b; k += 32) {
        const double pred = y0 + slope * ((double)starts[lo + k] - mx - x0);
        const double e = (double)k - pred;
        if (e > 0) ehi = max(ehi, (int)ceil(e));
        else elo = max(elo, (int)ceil(-e));
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        elo = max(elo, __shfl_xor_sync(kFull, elo, d));
        ehi = max(ehi, __shfl_xor_sync(kFull, ehi, d));
    }
    if (lane == 0) {
        M.x0 = x0;
        M.slope = slope;
        M.y0 = y0;
        M.err_lo = elo;
        M.err_hi = ehi;
        leaves[L] = M;
    }
}

template <typename S>
__global__ void k_eytz_build(const S* __restrict__ starts, const int64_t* __restrict__ seg, int G, int K,
                             S* __restrict__ keys) {
    const int g = blockIdx.y;
    const int64_t lo = seg[g], n = seg[g + 1] - lo;
    const int levels = 31 - __clz(K + 1);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= K; i += gridDim.x * blockDim.x) {
        S key = Lim<S>::hi;
        if (i >= 1 && n > 0) {
            const int lvl = 31 - __clz(i);
            const int64_t off = i - (1 << lvl);
            const int below = levels - 1 - lvl;
            const int64_t r = ((2 * off + 1) << below) - 1;
            key = starts[lo + eytz_sample_pos(r, n, K)];
        }
        keys[(int64_t)g * (K + 1) + i] = key;
    }
}

inline unsigned nblk(int64_t n, int t = kThreads) { return (unsigned)std::max<int64_t>(1, ceil_div(n, t)); }

// Blocks of `threads` that fit on the whole device at once (one wave of a grid-stride kernel).
static int64_t resident_blocks(const void* fn, int threads) {
    int dev = 0, nsm = 152, per_sm = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    return (int64_t)nsm * std::max(per_sm, 1);
}

template <typename S>
Pyr<S> make_pyr(MapView<S> m, Levels<S> L, int H) {
    Pyr<S> P;
    P.ends = m.ends;
    for (int h = 0; h < kMaxLevels; ++h) P.m[h] = L.p[h];
    P.H = H;
    return P;
}

template <typename S>
UbView<S> make_ub(const BatchedWorkspace& ws, int mode) {
    UbView<S> U;
    U.mode = mode;
    U.leaf_base = ws.ub.leaf_base.as<int32_t>();
    U.leaf_key = ws.ub.leaf_key.as<S>();
    U.leaf_pos = ws.ub.leaf_pos.as<int32_t>();
    U.leaves = ws.ub.leaves.as<LeafModel>();
    U.key_mean = ws.ub.key_mean.as<double>();
    U.eytz_keys = ws.ub.eytz_keys.as<S>();
    U.eytz_n = ws.ub.eytz_n;
    if (mode == SI_UB_LEARNED && (!U.leaves || ws.ub.total_leaves == 0)) U.mode = SI_UB_BINARY;
    if (mode == SI_UB_EYTZINGER && ws.ub.eytz_n <= 1) U.mode = SI_UB_BINARY;
    return U;
}

size_t tile_smem(const BatchedParams& p, size_t s) {
    // cend + cpos, the tile's query records, then frontier list + counts + masks
    // candidates (end, position), per-query records, BFS scratch / long list (+ 64-bit starts)
    return (size_t)p.cap * (s + 4) + (size_t)p.tile_q * (s + 12 + 16 + 12) + (size_t)p.cap * 12 +
           (s == 8 ? (size_t)p.cap * 8 : 0) + 64;
}

#define SI_CU(call)                                    \
    do {                                               \
        if ((call) != cudaSuccess) return SI_ERR_CUDA; \
    } while (0)
#define SI_OKR(call)                     \
    do {                                 \
        int r_ = (call);                 \
        if (r_ != SI_OK) return r_;      \
    } while (0)

template <typename S>
int build_learned(BatchedWorkspace& ws, MapView<S> m, cudaStream_t st) {
    const int G = m.G;
    std::vector<int64_t> seg(G + 1);
    SI_CU(cudaMemcpyAsync(seg.data(), m.seg, sizeof(int64_t) * (G + 1), cudaMemcpyDeviceToHost, st));
    SI_CU(cudaStreamSynchronize(st));
    // equal-count leaves: up to 4096 per contig, at least 64 keys each
    std::vector<int32_t> base(G + 1, 0), leaf_contig, leaf_pos;
    for (int g = 0; g < G; ++g) {
        const int64_t n = seg[g + 1] - seg[g];
        const int nl = (int)std::min<int64_t>(4096, std::max<int64_t>(1, n / 64));
        base[g + 1] = base[g] + nl;
        for (int l = 0; l < nl; ++l) {
            leaf_contig.push_back(g);
            leaf_pos.push_back((int32_t)((int64_t)l * n / nl));
        }
    }
    const int total = base[G];
    ws.ub.total_leaves = total;
    DBuf acc, lc;
    SI_OKR(acc.reserve(sizeof(double) * 2 * G));
    SI_OKR(ws.ub.key_mean.reserve(sizeof(double) * G));
    SI_OKR(ws.ub.leaf_base.reserve(sizeof(int32_t) * (G + 1)));
    SI_OKR(ws.ub.leaves.reserve(sizeof(LeafModel) * std::max(total, 1)));
    SI_OKR(ws.ub.leaf_pos.reserve(sizeof(int32_t) * std::max(total, 1)));
    SI_OKR(ws.ub.leaf_key.reserve(sizeof(S) * std::max(total, 1)));
    SI_OKR(lc.reserve(sizeof(int32_t) * std::max(total, 1)));
    SI_CU(cudaMemcpyAsync(ws.ub.leaf_base.p, base.data(), sizeof(int32_t) * (G + 1), cudaMemcpyHostToDevice, st));
    SI_CU(cudaMemcpyAsync(lc.p, leaf_contig.data(), sizeof(int32_t) * total, cudaMemcpyHostToDevice, st));
    SI_CU(cudaMemcpyAsync(ws.ub.leaf_pos.p, leaf_pos.data(), sizeof(int32_t) * total, cudaMemcpyHostToDevice, st));
    // mean key per contig (conditioning of the leaf fits)
    SI_CU(cudaMemsetAsync(acc.p, 0, sizeof(double) * 2 * G, st));
    dim3 grid(64, (unsigned)std::min(G, 65535));
    k_key_sums<S><<<grid, kThreads, 0, st>>>(m.starts, m.seg, G, acc.as<double>());
    note_launch();
    SI_CU(cudaGetLastError());
    std::vector<double> a(2 * G), mean(G);
    SI_CU(cudaMemcpyAsync(a.data(), acc.p, sizeof(double) * 2 * G, cudaMemcpyDeviceToHost, st));
    SI_CU(cudaStreamSynchronize(st));
    for (int g = 0; g < G; ++g) {
        const int64_t n = seg[g + 1] - seg[g];
        mean[g] = n > 0 ? a[g] / (double)n : 0.0;
    }
    SI_CU(cudaMemcpyAsync(ws.ub.key_mean.p, mean.data(), sizeof(double) * G, cudaMemcpyHostToDevice, st));
    // the root (first key of every leaf), then each leaf's least-squares line and max errors
    k_leaf_keys<S><<<nblk(total), kThreads, 0, st>>>(m.starts, m.seg, lc.as<int32_t>(), ws.ub.leaf_pos.as<int32_t>(),
                                                     total, ws.ub.leaf_key.as<S>());
    note_launch();
    SI_CU(cudaGetLastError());
    k_leaf_fit<S><<<nblk((int64_t)total * 32), kThreads, 0, st>>>(
        m.starts, m.seg, lc.as<int32_t>(), ws.ub.leaf_base.as<int32_t>(), ws.ub.leaf_pos.as<int32_t>(),
        ws.ub.key_mean.as<double>(), ws.ub.leaves.as<LeafModel>(), total);
    note_launch();
    SI_CU(cudaGetLastError());
    SI_CU(cudaStreamSynchronize(st));
    ws.launches += 3;
    return SI_OK;
}

template <typename S>
int build_eytz(BatchedWorkspace& ws, MapView<S> m, cudaStream_t st) {
    const int G = m.G;
    int depth = ws.prm.eytz_depth;
    if (depth <= 0) {
        // shared-memory budget: at most 8191 keys, and no deeper than the average contig
        const int64_t avg = std::max<int64_t>(1, m.n / std::max(1, G));
        depth = 1;
        while (depth < 13 && ((int64_t)1 << (depth + 1)) <= avg / 4) ++depth;
    }
    const int K = (1 << depth) - 1;
    ws.ub.eytz_depth = depth;
    ws.ub.eytz_n = K + 1;
    SI_OKR(ws.ub.eytz_keys.reserve(sizeof(S) * (size_t)G * (K + 1)));
    k_eytz_build<S><<<dim3(nblk(K + 1), G), kThreads, 0, st>>>(m.starts, m.seg, G, K, ws.ub.eytz_keys.as<S>());
    note_launch();
    SI_CU(cudaGetLastError());
    SI_CU(cudaStreamSynchronize(st));
    ws.launches += 1;
    return SI_OK;
}

}  // namespace

template <typename S>
int batched_prepare(BatchedWorkspace& ws, MapView<S> m, Levels<S>, int, const int64_t*, int ub_mode,
                    cudaStream_t st) {
    ws.prepared_nq = -1;
    ws.prepared_qs = nullptr;
    ws.ub.mode = ub_mode;
    ws.ub.G = m.G;
    ws.ub.total_leaves = 0;
    ws.ub.eytz_n = 0;
    if (m.n == 0) return SI_OK;
    if (ub_mode == SI_UB_LEARNED) return build_learned<S>(ws, m, st);
    if (ub_mode == SI_UB_EYTZINGER) return build_eytz<S>(ws, m, st);
    return SI_OK;
}

template <typename S>
int batched_prepare_queries(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, int* d_err, int ub_mode,
                            cudaStream_t st, uint32_t* counts, bool tile_cuts) {
    const int64_t nq = q.nq;
    ws.prepared_nq = -1;
    if (nq <= 0) return SI_OK;
    if (nq >= (int64_t)INT32_MAX) return SI_ERR_TOO_LARGE;
    const int K = (sizeof(S) == 4) ? 2 : 3;
    uint32_t* kp[3];
    uint32_t* ka[3];
    for (int k = 0; k < K; ++k) {
        SI_OKR(ws.kw[k].reserve(sizeof(uint32_t) * nq));
        SI_OKR(ws.kalt[k].reserve(sizeof(uint32_t) * nq));
        kp[k] = ws.kw[k].as<uint32_t>();
        ka[k] = ws.kalt[k].as<uint32_t>();
    }
    SI_OKR(ws.pay.reserve(sizeof(uint32_t) * nq));
    SI_OKR(ws.palt.reserve(sizeof(uint32_t) * nq));
    const size_t tb = radix_temp_bytes(nq, K);
    SI_OKR(ws.sort_tmp.reserve(tb));
    SI_OKR(ws.sq_s.reserve(sizeof(S) * nq));
    SI_OKR(ws.sq_u.reserve(sizeof(int32_t) * nq));
    SI_OKR(ws.sq_c.reserve(sizeof(uint32_t) * nq));
    SI_OKR(ws.sq_id.reserve(sizeof(int32_t) * nq));
    // one packed key word when (class code, end offset >> shift) fits 24 bits with shift <= 16
    // (three radix passes), else one word per 32 bits of end plus the class word
    SI_OKR(ws.qminmax.reserve(2 * sizeof(unsigned long long)));
    SI_CU(cudaMemsetAsync(ws.qminmax.p, 0xff, sizeof(unsigned long long), st));       // min: all ones
    SI_CU(cudaMemsetAsync(ws.qminmax.as<unsigned long long>() + 1, 0, sizeof(unsigned long long), st));
    k_qend_minmax<S><<<(unsigned)std::min<int64_t>(nblk(nq), 152 * 8), kThreads, 0, st>>>(
        static_cast<const S*>(q.qe), nq, ws.qminmax.as<unsigned long long>());
    note_launch();
    const int code_bits = query_code_bits(m.G);
    int shift = 8, ebits = 0;
    bool packed = true;
    const int* d_pack = nullptr;
    if (ws.capturing) {
        // inside a graph capture: the packing is worked out on the device (int32 coordinates and
        // code_bits <= 8 always pack into 24 bits with shift <= 16), and the sort runs its three
        // low byte passes without reading its histograms back
        if constexpr (sizeof(S) != 4) {
            return SI_ERR_INVALID;
        } else {
            if (code_bits > 8) return SI_ERR_INVALID;
            SI_OKR(ws.qpack.reserve(2 * sizeof(int)));
            k_pack_params<<<1, 32, 0, st>>>(ws.qminmax.as<unsigned long long>(), code_bits, ws.qpack.as<int>());
            note_launch();
            d_pack = ws.qpack.as<int>();
        }
    } else {
        unsigned long long mm[2] = {0, 0};
        SI_CU(cudaMemcpyAsync(mm, ws.qminmax.p, sizeof(mm), cudaMemcpyDeviceToHost, st));
        SI_CU(cudaStreamSynchronize(st));
        const unsigned long long span = mm[1] - mm[0];
        int span_bits = 0;
        while (span_bits < 64 && (span >> span_bits) != 0) ++span_bits;
        shift = std::max(8, span_bits + code_bits - 24);
        packed = code_bits <= 16 && shift <= 16;
        ebits = packed ? std::max(0, span_bits - shift) : 0;
    }
    int Kp = K;
    uint32_t* wc = kp[K - 1];
    if (packed) {
        Kp = 1;
        wc = kp[0];
        SI_OKR(ws.qpair.reserve(2 * sizeof(S) * nq));
        // the sort's digit histograms are counted by the key kernel (radix_sort skips its own pass)
        SI_CU(cudaMemsetAsync(radix_hist(ws.sort_tmp.p), 0, sizeof(uint32_t) * 4 * 256, st));
        const int64_t kb = resident_blocks(reinterpret_cast<const void*>(&k_qkeys_packed<S>), kThreads);
        k_qkeys_packed<S><<<(unsigned)std::min<int64_t>(nblk(nq, 4 * kThreads), kb), kThreads, 0, st>>>(
            static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc, nq, ws.prm.long_len, m.G,
            ws.qminmax.as<unsigned long long>(), shift, ebits, d_pack, kp[0], ws.pay.as<uint32_t>(),
            ws.qpair.as<S>(), radix_hist(ws.sort_tmp.p));
    } else {
        k_qkeys<S><<<nblk(nq), kThreads, 0, st>>>(static_cast<const S*>(q.qs), static_cast<const S*>(q.qe), q.qc,
                                                  nq, ws.prm.long_len, m.G, kp[0], K == 3 ? kp[1] : nullptr, wc,
                                                  ws.pay.as<uint32_t>());
    }
    note_launch();
    SI_CU(cudaGetLastError());
    bool in_alt = false;
    int passes = 0;
    SI_CU(radix_sort(kp, ka, ws.pay.as<uint32_t>(), ws.palt.as<uint32_t>(), Kp, nq, ws.sort_tmp.p, tb, &in_alt,
                     &passes, st, ws.capturing ? 0x7u : 0u, d_err, packed));
    const uint32_t* spay = in_alt ? ws.palt.as<uint32_t>() : ws.pay.as<uint32_t>();
    const uint32_t* swc = in_alt ? ka[Kp - 1] : kp[Kp - 1];
    UbView<S> U = make_ub<S>(ws, ub_mode);
    SI_OKR(ws.blk_cut.reserve(2 * sizeof(int64_t) * (size_t)nblk(nq)));
    k_qprep<S><<<nblk(nq), kThreads, 0, st>>>(spay, swc, packed ? ebits : 0, d_pack, static_cast<const S*>(q.qs),
                                              static_cast<const S*>(q.qe), packed ? ws.qpair.as<S>() : nullptr,
                                              nq, m, U, ws.sq_s.as<S>(), ws.sq_u.as<int32_t>(),
                                              ws.sq_c.as<uint32_t>(), ws.sq_id.as<int32_t>(), d_err, ws.long_split,
                                              ws.long_pos, ws.long_seg,
                                              (tile_cuts && ws.long_pos) ? ws.blk_cut.as<int64_t>() : nullptr,
                                              static_cast<const S*>(ws.end_sorted), counts);
    note_launch();
    SI_CU(cudaGetLastError());
    // keys, min/max, histogram (counted by the key kernel when packed), digit offsets, passes, prepare
    ws.launches += 2 + (packed ? 1 : 2) + passes + 1;
    ws.prepared_qs = q.qs;
    ws.prepared_nq = nq;
    ws.prepared_mode = ub_mode;
    return SI_OK;
}

template <typename S>
static int run_tiles(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, int64_t nq, bool emit,
                     uint32_t* counts, int32_t* heads, const int32_t* heads_in, const int64_t* offsets,
                     int64_t out_base, int order, bool values, int32_t* out, int* d_err, bool use_cache,
                     cudaStream_t st, int64_t id_lo = 0, int64_t id_hi = INT64_MAX, int tile_q = 0) {
    BatchedParams prm = ws.prm;
    if (tile_q) prm.tile_q = tile_q;
    SI_OKR(ws.counters.reserve(sizeof(int) * 4));
    SI_CU(cudaMemsetAsync(ws.counters.p, 0, sizeof(int) * 4, st));
    TileArgs<S> a;
    a.P = make_pyr<S>(m, L, H);
    a.PL.ends = static_cast<const S*>(ws.long_ends);
    for (int h = 0; h < kMaxLevels; ++h) a.PL.m[h] = static_cast<const S*>(ws.long_lvl[h]);
    a.PL.H = ws.long_H;
    a.long_pos = ws.long_pos;
    a.long_seg = ws.long_seg;
    a.blk_cut = (prm.tile_q == kThreads && ws.blk_cut.p) ? ws.blk_cut.as<int64_t>() : nullptr;
    a.long_split = ws.long_split;
    a.end_sorted = static_cast<const S*>(ws.end_sorted);
    a.starts = m.starts;
    a.split_len = prm.split_len;
    a.data = m.data;
    a.seg = m.seg;
    a.G = m.G;
    a.sq_s = ws.sq_s.as<S>();
    a.sq_u = ws.sq_u.as<int32_t>();
    a.sq_c = ws.sq_c.as<uint32_t>();
    a.sq_id = ws.sq_id.as<int32_t>();
    a.nq = nq;
    a.tile_q = prm.tile_q;
    a.cap = prm.cap;
    a.n_tiles = (int)ceil_div(nq, a.tile_q);
    a.tile_counter = ws.counters.as<int>();
    a.counts = counts;
    a.heads = heads;
    a.heads_in = heads_in;
    a.offsets = offsets;
    a.id_lo = id_lo;
    a.id_hi = id_hi;
    a.out_cap = ws.out_cap;
    a.out_base = out_base;
    a.order = order;
    a.values = values;
    a.emit_copy = prm.emit_copy;
    a.out = out;
    a.d_err = d_err;
    a.cache = (use_cache && ws.cache_ok) ? ws.tile_cache.as<unsigned char>() : nullptr;
    a.cache_stride = ws.cache_stride;
    const size_t sm = tile_smem(prm, sizeof(S));
    // the kernel attribute and the occupancy are set / asked once per shared-memory size
    const int e = emit ? 1 : 0;
    if (ws.occ_smem[e] != sm) {
        int dev = 0, nsm = 152, per_sm = 1;
        SI_CU(cudaGetDevice(&dev));
        SI_CU(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        if (emit) {
            SI_CU(cudaFuncSetAttribute(k_tiles<S, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            SI_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tiles<S, true>, kThreads, sm));
        } else {
            SI_CU(cudaFuncSetAttribute(k_tiles<S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            SI_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tiles<S, false>, kThreads, sm));
        }
        ws.occ_blocks[e] = nsm * std::max(per_sm, 1);
        ws.occ_smem[e] = sm;
    }
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)ws.occ_blocks[e], a.n_tiles));
    if (emit) k_tiles<S, true><<<grid, kThreads, sm, st>>>(a);
    else k_tiles<S, false><<<grid, kThreads, sm, st>>>(a);
    note_launch();
    SI_CU(cudaGetLastError());
    ws.launches += 1;
    return SI_OK;
}

template <typename S>
int batched_count(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q, uint32_t* counts,
                  int* d_err, cudaStream_t st) {
    const int64_t nq = q.nq;
    if (nq <= 0) return SI_OK;
    if (ws.prepared_nq != nq || ws.prepared_qs != q.qs) return SI_ERR_INVALID;
    SI_OKR(ws.heads.reserve(sizeof(int32_t) * nq));
    ws.n_heads = nq;
    ws.cache_prm_tile = ws.prm.tile_q;
    ws.cache_prm_cap = ws.prm.cap;
    if (ws.end_sorted) {  // short queries are counted from ranks: no tile lists to keep
        ws.cache_ok = false;
        return run_tiles<S>(ws, m, L, H, nq, false, counts, ws.heads.as<int32_t>(), nullptr, nullptr, 0, 0, false,
                            nullptr, d_err, false, st);
    }
    // room for every tile's candidate lists, so that the emit pass need not gather again;
    // without room (device budget) the emit pass simply gathers again
    ws.cache_stride = (int64_t)round_up(kCacheHeader + (int64_t)ws.prm.cap * (8 + 3 * (int64_t)sizeof(S)) +
                                            (int64_t)kLnu * (4 + (int64_t)sizeof(S)), 256);
    const int64_t n_tiles = ceil_div(nq, ws.prm.tile_q);
    ws.cache_ok = ws.tile_cache.reserve((size_t)(n_tiles * ws.cache_stride)) == SI_OK;
    return run_tiles<S>(ws, m, L, H, nq, false, counts, ws.heads.as<int32_t>(), nullptr, nullptr, 0, 0, false,
                        nullptr, d_err, true, st);
}

template <typename S>
int batched_emit(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q, int64_t q_offset,
                 const int64_t* offsets, int64_t out_base, int order, bool values, int32_t* out, int* d_err,
                 int ub_mode, cudaStream_t st, int64_t total_hits) {
    const int64_t nq = q.nq;
    if (nq <= 0) return SI_OK;
    if (q_offset < 0 || q_offset + nq > ws.n_heads) return SI_ERR_INVALID;
    const bool same = (q_offset == 0 && ws.prepared_nq == nq && ws.prepared_qs == q.qs);
    // a slice of the batch prepared last: its tiles are kept (sorted neighbours share candidate
    // lists) and only the slice's ids are emitted, instead of sorting the slice on its own,
    // whose queries would lie far apart
    const bool window = !same && ws.prepared_qs != nullptr && ws.prepared_nq >= q_offset + nq &&
                        static_cast<const S*>(q.qs) - q_offset == static_cast<const S*>(ws.prepared_qs);
    const bool cache_fits = ws.cache_ok && ws.cache_prm_tile == ws.prm.tile_q && ws.cache_prm_cap == ws.prm.cap;
    // Without a count-pass cache (the rank counts), the tile size is free: the largest of 256,
    // 128, 64, 32 queries whose expected candidates, tile_q * (intervals per query) + hits per
    // query, fill at most 3/4 of the candidate slots.  Tiles that overflow fall back to
    // per-query walks, which costs up to 25x at sparse batches.
    const int64_t batch_nq = (same || window) ? ws.prepared_nq : nq;
    int tile = 0;
    if (ws.prm.auto_tile && ws.end_sorted && total_hits >= 0 && batch_nq > 0) {
        const double per_q = (double)m.n / (double)batch_nq, hpq = (double)total_hits / (double)batch_nq;
        tile = kThreads;
        while (tile > 32 && tile * per_q + hpq > 0.75 * ws.prm.cap) tile >>= 1;
    }
    if (window)
        return run_tiles<S>(ws, m, L, H, ws.prepared_nq, true, nullptr, nullptr, ws.heads.as<int32_t>(),
                            offsets - q_offset, out_base, order, values, out, d_err, cache_fits && !tile, st,
                            q_offset, q_offset + nq, tile);
    if (!same) SI_OKR(batched_prepare_queries<S>(ws, m, q, d_err, ub_mode, st));
    // sorted ids are relative to q; heads / offsets are shifted to the slice
    return run_tiles<S>(ws, m, L, H, nq, true, nullptr, nullptr, ws.heads.as<int32_t>() + q_offset, offsets,
                        out_base, order, values, out, d_err, same && cache_fits && !tile, st, 0, INT64_MAX, tile);
}

template <typename S>
int upper_bounds(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, int ub_mode, int32_t* out, int* d_err,
                 cudaStream_t st, bool sorted) {
    if (q.nq <= 0) return SI_OK;
    if (sorted) {
        QueryBatch qq = q;
        qq.qs = q.qe;  // queries [qe, qe]: one class per contig, the sort key is the end
        SI_OKR(batched_prepare_queries<S>(ws, m, qq, d_err, ub_mode, st, nullptr, false));
        k_ub_scatter<<<nblk(q.nq), kThreads, 0, st>>>(ws.sq_u.as<int32_t>(), ws.sq_c.as<uint32_t>(),
                                                      ws.sq_id.as<int32_t>(), q.nq, m.seg, m.G, out);
        note_launch();
        SI_CU(cudaGetLastError());
        ws.launches += 1;
        // the sorted records hold (qe, qe) queries: no search may take them as its own
        ws.prepared_nq = -1;
        ws.prepared_qs = nullptr;
        return SI_OK;
    }
    UbView<S> U = make_ub<S>(ws, ub_mode);
    // the tree's top levels of every contig that fit 48 KiB of shared memory (2^d slots each,
    // d <= the tree's depth)
    int top_n = 0;
    if (U.mode == 1 && U.eytz_n > 1) {
        top_n = U.eytz_n;
        while (top_n > 1 && (size_t)top_n * sizeof(S) * (size_t)m.G > 48 * 1024) top_n >>= 1;
        if (top_n <= 1) top_n = 0;
    }
    const size_t sm = sizeof(S) * (size_t)top_n * (size_t)m.G;
    k_ub_plain<S><<<nblk(q.nq), kThreads, sm, st>>>(static_cast<const S*>(q.qe), q.qc, q.nq, m, U, out, d_err,
                                                    top_n);
    note_launch();
    SI_CU(cudaGetLastError());
    ws.launches += 1;
    return SI_OK;
}

template <typename S>
int batched_coverage(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, const uint64_t* ps_start,
                     const uint64_t* ps_end, uint64_t* count, S* cov, int* d_err, int ub_mode, cudaStream_t st) {
    if (q.nq <= 0) return SI_OK;
    if (!ws.end_sorted) return SI_ERR_INVALID;
    SI_OKR(batched_prepare_queries<S>(ws, m, q, d_err, ub_mode, st));
    k_cov_ranks<S><<<nblk(q.nq), kThreads, 0, st>>>(ws.sq_s.as<S>(), ws.sq_u.as<int32_t>(), ws.sq_c.as<uint32_t>(),
                                                   ws.sq_id.as<int32_t>(), static_cast<const S*>(q.qe), q.nq, m,
                                                   static_cast<const S*>(ws.end_sorted), ps_start, ps_end, count,
                                                   cov);
    note_launch();
    SI_CU(cudaGetLastError());
    ws.launches += 1;
    return SI_OK;
}

#define SIG_BINST(S)                                                                                             \
    template int batched_prepare<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const int64_t*, int,            \
                                    cudaStream_t);                                                              \
    template int batched_prepare_queries<S>(BatchedWorkspace&, MapView<S>, const QueryBatch&, int*, int,          \
                                            cudaStream_t, uint32_t*, bool);                                                \
    template int batched_count<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const QueryBatch&, uint32_t*,   \
                                  int*, cudaStream_t);                                                          \
    template int batched_emit<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const QueryBatch&, int64_t,      \
                                 const int64_t*, int64_t, int, bool, int32_t*, int*, int, cudaStream_t,         \
                                 int64_t);                                                                      \
    template int upper_bounds<S>(BatchedWorkspace&, MapView<S>, const QueryBatch&, int, int32_t*, int*,          \
                                 cudaStream_t, bool);                                                           \
    template int batched_coverage<S>(BatchedWorkspace&, MapView<S>, const QueryBatch&, const uint64_t*,         \
                                     const uint64_t*, uint64_t*, S*, int*, int, cudaStream_t);
SIG_BINST(int32_t)
SIG_BINST(int64_t)

}  // namespace sig
