// si_build.cu -- device side of build(): sortedness check, sort keys, decode,
// the max-of-32 pyramid over ends, and the branch array.
//
// Reference: IntervalMap::build() (src/superintervals.hpp:112-130) and
// indexSuperIntervals (src/c_superintervals.h:487-521).  The reference computes
//     branch[i] = nearest j < i with ends[j] >= ends[i]   (else SIZE_MAX)
// with a sequential monotonic stack (pop while top < ends[i], hpp:122).  Here
// the same "previous greater-or-equal" relation is found in parallel:
//   * inside each 32-interval chunk with warp shuffles (one warp = one chunk);
//   * across chunks by climbing a max-of-32 pyramid of ends: at level h the
//     warp compares its node's 31 left siblings' maxima (one coalesced 128-byte
//     load, broadcast by shuffle) against each lane's end, picks the nearest
//     sibling whose max is >= the end, and the lane descends that sibling's
//     subtree (always the right-most child whose max is >= the end) down to the
//     interval.  Ties resolve exactly as the stack does (>=).
// A result that falls before the lane's contig start becomes -1 (per-contig maps).
#include <algorithm>
#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int64_t seg_of(const int64_t* __restrict__ seg, int G, int64_t i) {
    // largest g with seg[g] <= i
    int lo = 0, hi = G - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (seg[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <typename S>
__global__ void k_check_sorted(const S* __restrict__ s, const S* __restrict__ e, int64_t n,
                               const int64_t* __restrict__ seg, int G, int* __restrict__ flag) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += stride) {
        if (G > 1 && seg[seg_of(seg, G, i)] == i) continue;  // first interval of a contig
        const S s0 = s[i - 1], s1 = s[i];
        if (s1 < s0 || (s1 == s0 && e[i] > e[i - 1])) bad = true;
    }
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

template <typename S>
__global__ void k_make_keys(const S* __restrict__ s, const S* __restrict__ e, int64_t n,
                            const int64_t* __restrict__ seg, int G, uint32_t* w0, uint32_t* w1,
                            uint32_t* w2, uint32_t* w3, uint32_t* w4,
                            uint32_t* __restrict__ payload) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if constexpr (sizeof(S) == 4) {
        // end descending: complement of the order-preserving bias
        w0[i] = ~((uint32_t)e[i] ^ 0x80000000u);
        w1[i] = (uint32_t)s[i] ^ 0x80000000u;
        if (G > 1) w2[i] = (uint32_t)seg_of(seg, G, i);
    } else {
        const uint64_t eb = ~((uint64_t)e[i] ^ 0x8000000000000000ull);
        const uint64_t sb = (uint64_t)s[i] ^ 0x8000000000000000ull;
        w0[i] = (uint32_t)eb;
        w1[i] = (uint32_t)(eb >> 32);
        w2[i] = (uint32_t)sb;
        w3[i] = (uint32_t)(sb >> 32);
        if (G > 1) w4[i] = (uint32_t)seg_of(seg, G, i);
    }
    payload[i] = (uint32_t)i;
}

template <typename S>
__global__ void k_decode(const uint32_t* __restrict__ w0, const uint32_t* __restrict__ w1,
                         const uint32_t* __restrict__ w2, const uint32_t* __restrict__ w3,
                         const uint32_t* __restrict__ perm, const int32_t* __restrict__ data_in,
                         int64_t n, int64_t n_pad, S* __restrict__ starts, S* __restrict__ ends,
                         int32_t* __restrict__ data) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {
        starts[i] = Lim<S>::hi;
        ends[i] = Lim<S>::lo;
        return;
    }
    if constexpr (sizeof(S) == 4) {
        ends[i] = (S)((~w0[i]) ^ 0x80000000u);
        starts[i] = (S)(w1[i] ^ 0x80000000u);
    } else {
        const uint64_t eb = ((uint64_t)w1[i] << 32) | w0[i];
        const uint64_t sb = ((uint64_t)w3[i] << 32) | w2[i];
        ends[i] = (S)((~eb) ^ 0x8000000000000000ull);
        starts[i] = (S)(sb ^ 0x8000000000000000ull);
    }
    data[i] = data_in[perm[i]];
}

template <typename S>
__global__ void k_copy_pad(const S* __restrict__ s_in, const S* __restrict__ e_in,
                           const int32_t* __restrict__ d_in, int64_t n, int64_t n_pad,
                           S* __restrict__ starts, S* __restrict__ ends, int32_t* __restrict__ data,
                           uint32_t* __restrict__ perm) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {
        starts[i] = Lim<S>::hi;
        ends[i] = Lim<S>::lo;
        return;
    }
    starts[i] = s_in[i];
    ends[i] = e_in[i];
    data[i] = d_in[i];
    if (perm) perm[i] = (uint32_t)i;
}

// out[c] = max(in[32c .. 32c+31]); `in` is padded to a multiple of 32, `out`
// to a multiple of 32 with S_MIN.
template <typename S>
__global__ void k_level_max(const S* __restrict__ in, int64_t n_out, int64_t n_out_pad,
                            S* __restrict__ out) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_out_pad) return;
    if (c >= n_out) {
        out[c] = Lim<S>::lo;
        return;
    }
    const S* p = in + (c << 5);
    S m = p[0];
#pragma unroll
    for (int k = 1; k < 32; ++k) m = p[k] > m ? p[k] : m;
    out[c] = m;
}

// Long-interval list: the intervals with end - start >= X, in position order (their global
// positions and ends), padded with (-1, S_MIN) to a multiple of 32.
template <typename S>
__device__ __forceinline__ bool long_iv(S s, S e, int64_t X) {
    return e >= s && (uint64_t)e - (uint64_t)s >= (uint64_t)X;
}

template <typename S>
__global__ void k_long_flags(const S* __restrict__ starts, const S* __restrict__ ends, int64_t n, int64_t X,
                             uint32_t* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = long_iv(starts[i], ends[i], X) ? 1u : 0u;
}

template <typename S>
__global__ void k_long_scatter(const S* __restrict__ starts, const S* __restrict__ ends, int64_t n, int64_t X,
                               const int64_t* __restrict__ offs, int64_t n_long, int64_t n_long_pad,
                               int32_t* __restrict__ pos, S* __restrict__ lend) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && long_iv(starts[i], ends[i], X)) {
        const int64_t k = offs[i];
        pos[k] = (int32_t)i;
        lend[k] = ends[i];
    }
    if (i >= n_long && i < n_long_pad) {
        pos[i] = -1;
        lend[i] = Lim<S>::lo;
    }
}

// flag = 1 when a[i] != b[i] for some i < n
__global__ void k_differs_i32(const int32_t* __restrict__ a, const int32_t* __restrict__ b, int64_t n,
                              int* __restrict__ flag) {
    bool d = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d = d || a[i] != b[i];
    if (__any_sync(kFull, d) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// out[0] += total length of the intervals at least X long; out[1] += the contigs' extents (last
// start - first start + 1 over the sorted starts).  Their ratio is the depth of long intervals.
// Integer sums (a length is clamped to 2^40, which leaves room for 2^23 such intervals per
// block before the 64-bit total could wrap; the ratio only steers a path choice).
template <typename S>
__global__ void __launch_bounds__(kThreads) k_long_depth(const S* __restrict__ starts, const S* __restrict__ ends,
                                                         int64_t n, const int64_t* __restrict__ seg, int G,
                                                         int64_t X, unsigned long long* __restrict__ out) {
    __shared__ unsigned long long red[kThreads / 32];
    constexpr unsigned long long kClamp = 1ull << 40;
    unsigned long long a = 0, b = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t s0 = (int64_t)starts[i], e0 = (int64_t)ends[i];
        const unsigned long long d = (unsigned long long)e0 - (unsigned long long)s0;  // e - s when e >= s
        if (e0 >= s0 && d >= (unsigned long long)(X - 1))                                 // length >= X
            a += d < kClamp ? d + 1ull : kClamp;
    }
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < G; g += stride)
        if (seg[g + 1] > seg[g]) {
            const unsigned long long d =
                (unsigned long long)(int64_t)starts[seg[g + 1] - 1] - (unsigned long long)(int64_t)starts[seg[g]];
            b += d < kClamp ? d + 1ull : kClamp;
        }
    for (int k = 0; k < 2; ++k) {
        unsigned long long v = k == 0 ? a : b;
        for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0;
            for (int w = 0; w < kThreads / 32; ++w) t += red[w];
            if (t) atomicAdd(&out[k], t);
        }
        __syncthreads();
    }
}

// out[g] = offs[seg[g]]: first long-list index of each contig (g = 0..G)
__global__ void k_long_seg(const int64_t* __restrict__ offs, const int64_t* __restrict__ seg, int G,
                           int64_t* __restrict__ out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g <= G) out[g] = offs[seg[g]];
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_branch(const S* __restrict__ ends, int64_t n,
                                                     int64_t n_pad, Levels<S> L, int H,
                                                     const int64_t* __restrict__ seg, int G,
                                                     int32_t* __restrict__ branch) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((i & ~(int64_t)31) >= n_pad) return;  // warp-uniform: n_pad is a multiple of 32
    const int lane = threadIdx.x & 31;
    const bool valid = i < n;
    const S e = ends[i];

    // level 0: nearest earlier lane of this chunk with end >= e
    int best = -1;
#pragma unroll
    for (int k = 0; k < 31; ++k) {
        const S v = __shfl_sync(kFull, e, k);
        if (k < lane && v >= e) best = k;
    }
    int64_t res = (best >= 0) ? ((i & ~(int64_t)31) + best) : -1;
    bool open = valid && best < 0;
    int tgt_level = 0;
    int64_t tgt_node = -1;
    int64_t node = i >> 5;  // level-1 node (chunk) holding i
    for (int h = 1; h <= H; ++h) {
        if (!__any_sync(kFull, open)) break;
        const int64_t grp = node >> 5;
        const int pos = (int)(node & 31);
        const S mv = L.p[h - 1][(grp << 5) + lane];
        int bk = -1;
#pragma unroll
        for (int k = 0; k < 31; ++k) {
            const S v = __shfl_sync(kFull, mv, k);
            if (k < pos && v >= e) bk = k;
        }
        if (open && bk >= 0) {
            tgt_level = h;
            tgt_node = (grp << 5) + bk;
            open = false;
        }
        node = grp;
    }
    if (tgt_level > 0) {
        int64_t cur = tgt_node;
        for (int h = tgt_level; h > 1; --h) {
            const S* child = L.p[h - 2] + (cur << 5);
            int k = 31;
            while (k > 0 && child[k] < e) --k;
            cur = (cur << 5) + k;
        }
        const S* el = ends + (cur << 5);
        int k = 31;
        while (k > 0 && el[k] < e) --k;
        res = (cur << 5) + k;
    }
    if (!valid) return;
    if (G > 1 && res >= 0 && res < seg[seg_of(seg, G, i)]) res = -1;
    branch[i] = (int32_t)res;
}

// ---- branch pass with decoupled look-back across tiles ------------------------------------
// A block takes the next tile of kBrTile positions from an atomic counter and finds each
// position's nearest earlier position with end >= its end: inside its 32-position chunk with
// warp shuffles, then among the tile's earlier chunks (chunk maxima in shared memory).  The tile
// publishes its maximum end (flag 1) as soon as it is known; warp 0 then walks back over the
// earlier tiles' published maxima, 32 tiles per step, until a tile that has published its
// inclusive prefix maximum (flag 2) and publishes its own.  A position still unresolved (its end
// exceeds every earlier end of the tile) looks back the same way for the nearest earlier tile
// whose maximum reaches it -- or stops at a prefix maximum below its end, or at its contig's
// first tile -- and descends that tile's 32 chunk maxima (pyramid level 1) and the chosen
// chunk's 32 ends.  Waits on unpublished tiles are bounded; giving up records kDevTimeout.
constexpr int kBrTile = 1024;
constexpr int kBrSpinLimit = 1 << 22;

__device__ __forceinline__ void st_flag_release(int* p, int v) {
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_flag_acquire(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

template <typename S>
__global__ void __launch_bounds__(kThreads) k_branch_lookback(const S* __restrict__ ends, int64_t n, int64_t n_pad,
                                                              const S* __restrict__ lvl1,
                                                              const int64_t* __restrict__ seg, int G,
                                                              int32_t* __restrict__ branch, S* __restrict__ t_max,
                                                              S* __restrict__ t_pre, int* __restrict__ t_flag,
                                                              unsigned int* __restrict__ tile_ctr,
                                                              int* __restrict__ d_err) {
    __shared__ S se[kBrTile];
    __shared__ S cmax[kBrTile / 32];
    __shared__ int16_t s_un[kBrTile];
    __shared__ int16_t s_look[kBrTile];  // the ones of them that look back
    __shared__ int s_nun;
    __shared__ unsigned int s_t;
    __shared__ S s_before;  // the largest end of the tile's first contig before the tile
    __shared__ int64_t s_cs[2];  // contig start of the tile's first and last position
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_t = atomicAdd(tile_ctr, 1u);  // tiles in start order: earlier tiles run
        s_nun = 0;
        const int64_t b = (int64_t)s_t * kBrTile;
        const int64_t last = (b + kBrTile < n ? b + kBrTile : n) - 1;
        s_cs[0] = G > 1 ? seg[seg_of(seg, G, b)] : 0;
        s_cs[1] = G > 1 ? seg[seg_of(seg, G, last)] : 0;
    }
    __syncthreads();
    const int64_t t = s_t;
    const int64_t base = t * kBrTile;
    const int64_t cs_first = s_cs[0], cs_last = s_cs[1];
    for (int k = tid; k < kBrTile; k += kThreads) {
        const int64_t p = base + k;
        se[k] = p < n_pad ? ends[p] : Lim<S>::lo;
    }
    __syncthreads();
    for (int c = warp; c < kBrTile / 32; c += kThreads / 32) {
        S v = se[c * 32 + lane];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const S o = __shfl_xor_sync(kFull, v, d);
            v = o > v ? o : v;
        }
        if (lane == 0) cmax[c] = v;
    }
    __syncthreads();
    // t_max: the tile's largest end.  t_pre: the largest end from the start of the contig of the
    // tile's last position to the tile's end, published with flag 2; a tile where that contig
    // starts publishes it at once (it needs no earlier tile), the others after the look-back.
    if (warp == 0) {
        S m = cmax[lane];
        const int off = cs_last > base ? (int)(cs_last - base) : 0;  // positions of the last contig
        S l = Lim<S>::lo;
        if (lane * 32 >= off) {
            l = cmax[lane];
        } else if (lane * 32 + 31 >= off) {
            for (int j = off - lane * 32; j < 32; ++j) l = se[lane * 32 + j] > l ? se[lane * 32 + j] : l;
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            const S o = __shfl_xor_sync(kFull, m, d);
            m = o > m ? o : m;
            const S p = __shfl_xor_sync(kFull, l, d);
            l = p > l ? p : l;
        }
        if (lane == 0) {
            t_max[t] = m;
            if (cs_last >= base) t_pre[t] = l;
            st_flag_release(t_flag + t, cs_last >= base ? 2 : 1);
        }
    }
    // inside the tile: the chunk by shuffles, then the tile's earlier chunks
    for (int c = warp; c < kBrTile / 32; c += kThreads / 32) {
        const int k = c * 32 + lane;
        const int64_t i = base + k;
        const S e = se[k];
        int best = -1;
#pragma unroll
        for (int j = 0; j < 31; ++j) {
            const S v = __shfl_sync(kFull, e, j);
            if (j < lane && v >= e) best = j;
        }
        int64_t res = best >= 0 ? base + c * 32 + best : -1;
        if (best < 0 && i < n) {
            int cc = c - 1;
            while (cc >= 0 && cmax[cc] < e) --cc;
            if (cc >= 0) {
                int j = 31;
                while (se[cc * 32 + j] < e) --j;  // the chunk's maximum is >= e
                res = base + cc * 32 + j;
            } else {
                s_un[atomicAdd(&s_nun, 1)] = (int16_t)k;
            }
        }
        if (i < n && (best >= 0 || res >= 0)) {
            if (G > 1 && res < seg[seg_of(seg, G, i)]) res = -1;
            branch[i] = (int32_t)res;
        }
    }
    __syncthreads();
    // warp 0: the largest end of the tile's first contig before the tile, from the earlier
    // tiles' published values (every tile walked lies in that contig, or holds its start)
    if (warp == 0 && cs_first < base) {
        S pre = Lim<S>::lo;
        int64_t top = t - 1;
        int spins = 0;
        while (true) {
            const int64_t p = top - lane;
            const int f = p >= 0 ? ld_flag_acquire(t_flag + p) : 2;
            if (__any_sync(kFull, f == 0)) {
                if (++spins > kBrSpinLimit) {
                    if (lane == 0) atomicCAS(d_err, kDevOk, kDevTimeout);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            spins = 0;
            const unsigned pm = __ballot_sync(kFull, f == 2);
            const int first = pm ? __ffs(pm) - 1 : 32;
            S v = Lim<S>::lo;
            if (p >= 0 && lane <= first) v = (lane == first) ? t_pre[p] : t_max[p];
#pragma unroll
            for (int d = 16; d > 0; d >>= 1) {
                const S o = __shfl_xor_sync(kFull, v, d);
                v = o > v ? o : v;
            }
            pre = v > pre ? v : pre;
            if (pm) break;
            top -= 32;
        }
        if (lane == 0) {
            if (cs_last < base) {  // one contig throughout: its prefix runs on from the earlier tiles
                S m = t_max[t];
                t_pre[t] = m > pre ? m : pre;
                st_flag_release(t_flag + t, 2);
            }
            s_before = pre;
        }
    }
    if (tid == 0 && cs_first >= base) s_before = Lim<S>::lo;
    __syncthreads();
    // positions whose end exceeds every earlier end of the tile: those above every earlier
    // tile's ends too have none (-1); the others look back, one warp each
    {
        const S before = s_before;
        const int nun0 = s_nun;
        __syncthreads();
        if (tid == 0) s_nun = 0;
        __syncthreads();
        for (int u = tid; u < nun0; u += kThreads) {
            const int k = s_un[u];
            const int64_t i = base + k;
            // a contig that starts inside the tile has no position before it
            const bool first_contig = G <= 1 || i < n && seg[seg_of(seg, G, i)] == cs_first;
            if (!first_contig || cs_first >= base || se[k] > before) {
                if (i < n) branch[i] = -1;
            } else {
                s_look[atomicAdd(&s_nun, 1)] = (int16_t)k;
            }
        }
        __syncthreads();
    }
    const int nun = s_nun;
    for (int u = warp; u < nun; u += kThreads / 32) {
        const int k = s_look[u];
        const int64_t i = base + k;
        const S e = se[k];
        const int64_t cs = G > 1 ? seg[seg_of(seg, G, i)] : 0;  // the contig's first position
        int64_t res = -1;
        int64_t top = t - 1;
        int spins = 0;
        while (top >= 0) {
            const int64_t p = top - lane;
            const bool live = p >= 0 && (p + 1) * kBrTile > cs;  // the tile holds positions >= cs
            const int f = live ? ld_flag_acquire(t_flag + p) : 2;
            if (__any_sync(kFull, f == 0)) {
                if (++spins > kBrSpinLimit) {
                    if (lane == 0) atomicCAS(d_err, kDevOk, kDevTimeout);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            spins = 0;
            const bool reach = live && t_max[p] >= e;
            const bool stop = !live || (f == 2 && t_pre[p] < e);  // nothing at or before p reaches
            const unsigned hm = __ballot_sync(kFull, reach), sm = __ballot_sync(kFull, stop);
            const int fh = hm ? __ffs(hm) - 1 : 32, fs = sm ? __ffs(sm) - 1 : 32;
            if (fh < fs) {
                // the nearest tile reaching e: its last chunk, then the chunk's last position
                const int64_t pt = top - fh;
                const S cm = lvl1[pt * 32 + lane];
                const unsigned cmask = __ballot_sync(kFull, cm >= e);
                const int64_t ch = pt * 32 + (31 - __clz(cmask));
                const S v = ends[ch * 32 + lane];
                const unsigned vmask = __ballot_sync(kFull, v >= e);
                res = ch * 32 + (31 - __clz(vmask));
                break;
            }
            if (sm) break;
            top -= 32;
        }
        if (lane == 0 && i < n) branch[i] = (int32_t)(res >= cs ? res : -1);
    }
}

inline unsigned blocks_for(int64_t n, int t = kThreads) {
    return (unsigned)std::max<int64_t>(1, ceil_div(n, t));
}

}  // namespace

template <typename S>
cudaError_t launch_check_sorted(const S* s, const S* e, int64_t n, const int64_t* seg, int G,
                                int* d_flag, cudaStream_t st) {
    cudaError_t err = cudaMemsetAsync(d_flag, 0, sizeof(int), st);
    if (err != cudaSuccess || n <= 1) return err;
    const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(n, kThreads), 152 * 16);
    k_check_sorted<S><<<blocks, kThreads, 0, st>>>(s, e, n, seg, G, d_flag);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
int key_words(int G) {
    return (sizeof(S) == 4 ? 2 : 4) + (G > 1 ? 1 : 0);
}

template <typename S>
cudaError_t launch_make_keys(const S* s, const S* e, int64_t n, const int64_t* seg, int G,
                             uint32_t* const* kw, uint32_t* payload, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int K = key_words<S>(G);
    uint32_t* w[kMaxKeyWords] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < K; ++k) w[k] = kw[k];
    k_make_keys<S><<<blocks_for(n), kThreads, 0, st>>>(s, e, n, seg, G, w[0], w[1], w[2], w[3],
                                                      w[4], payload);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_decode(const uint32_t* const* kw, const uint32_t* perm, const int32_t* data_in,
                          int64_t n, int64_t n_pad, S* starts, S* ends, int32_t* data,
                          cudaStream_t st) {
    if (n_pad <= 0) return cudaSuccess;
    const uint32_t* w2 = sizeof(S) == 8 ? kw[2] : nullptr;
    const uint32_t* w3 = sizeof(S) == 8 ? kw[3] : nullptr;
    k_decode<S><<<blocks_for(n_pad), kThreads, 0, st>>>(kw[0], kw[1], w2, w3, perm, data_in, n,
                                                       n_pad, starts, ends, data);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_copy_pad(const S* s_in, const S* e_in, const int32_t* d_in, int64_t n,
                            int64_t n_pad, S* starts, S* ends, int32_t* data, uint32_t* perm,
                            cudaStream_t st) {
    if (n_pad <= 0) return cudaSuccess;
    k_copy_pad<S><<<blocks_for(n_pad), kThreads, 0, st>>>(s_in, e_in, d_in, n, n_pad, starts, ends,
                                                         data, perm);
    note_launch();
    return cudaGetLastError();
}

int pyramid_levels(int64_t n_pad, int64_t* sizes) {
    // sizes[h] = padded length of level h; the top level must hold <= 32 nodes
    sizes[0] = n_pad;
    int H = 0;
    int64_t m = n_pad;
    while (m > 32 && H < kMaxLevels) {
        const int64_t nodes = ceil_div(m, 32);
        ++H;
        sizes[H] = round_up(nodes, 32);
        m = nodes;
    }
    return H;
}

template <typename S>
cudaError_t launch_pyramid(const S* ends, const int64_t* sizes, int H, S* const* lvl,
                           cudaStream_t st) {
    const S* in = ends;
    int64_t m = sizes[0];
    for (int h = 1; h <= H; ++h) {
        const int64_t nodes = ceil_div(m, 32);
        k_level_max<S><<<blocks_for(sizes[h]), kThreads, 0, st>>>(in, nodes, sizes[h], lvl[h - 1]);
        note_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        in = lvl[h - 1];
        m = nodes;
    }
    return cudaSuccess;
}

template <typename S>
cudaError_t launch_long_flags(const S* starts, const S* ends, int64_t n, int64_t X, uint32_t* flags,
                              cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_long_flags<S><<<blocks_for(n), kThreads, 0, st>>>(starts, ends, n, X, flags);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_long_scatter(const S* starts, const S* ends, int64_t n, int64_t X, const int64_t* offs,
                                int64_t n_long, int64_t n_long_pad, const int64_t* seg, int G, int32_t* pos,
                                S* lend, int64_t* long_seg, cudaStream_t st) {
    const int64_t m = std::max(n, n_long_pad);
    if (m > 0) {
        k_long_scatter<S><<<blocks_for(m), kThreads, 0, st>>>(starts, ends, n, X, offs, n_long, n_long_pad, pos, lend);
        note_launch();
    }
    k_long_seg<<<blocks_for(G + 1), kThreads, 0, st>>>(offs, seg, G, long_seg);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_long_depth(const S* starts, const S* ends, int64_t n, const int64_t* seg, int G, int64_t X,
                              unsigned long long* out, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess || n <= 0) return e;
    k_long_depth<S><<<(unsigned)std::min<int64_t>(blocks_for(std::max<int64_t>(n, G)), 152 * 4), kThreads, 0, st>>>(
        starts, ends, n, seg, G, X, out);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_differs_i32(const int32_t* a, const int32_t* b, int64_t n, int* flag, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
    if (e != cudaSuccess || n <= 0) return e;
    k_differs_i32<<<(unsigned)std::min<int64_t>(blocks_for(n), 152 * 8), kThreads, 0, st>>>(a, b, n, flag);
    note_launch();
    return cudaGetLastError();
}

// Sort keys of the ends inside each contig: offset-binary end (word 0 low), contig above.
template <typename S>
__global__ void k_end_keys(const S* __restrict__ e, int64_t n, const int64_t* __restrict__ seg, int G,
                           uint32_t* __restrict__ w0, uint32_t* __restrict__ w1, uint32_t* __restrict__ w2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if constexpr (sizeof(S) == 4) {
        w0[i] = (uint32_t)e[i] ^ 0x80000000u;
        if (G > 1) w1[i] = (uint32_t)seg_of(seg, G, i);
    } else {
        const uint64_t b = (uint64_t)e[i] ^ 0x8000000000000000ull;
        w0[i] = (uint32_t)b;
        w1[i] = (uint32_t)(b >> 32);
        if (G > 1) w2[i] = (uint32_t)seg_of(seg, G, i);
    }
}

template <typename S>
__global__ void k_end_decode(const uint32_t* __restrict__ w0, const uint32_t* __restrict__ w1, int64_t n,
                             int64_t n_pad, S* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    if (i >= n) {
        out[i] = Lim<S>::hi;
    } else if constexpr (sizeof(S) == 4) {
        out[i] = (S)(w0[i] ^ 0x80000000u);
    } else {
        out[i] = (S)((((uint64_t)w1[i] << 32) | w0[i]) ^ 0x8000000000000000ull);
    }
}

template <typename S>
int end_key_words(int G) {
    return (sizeof(S) == 4 ? 1 : 2) + (G > 1 ? 1 : 0);
}

template <typename S>
cudaError_t launch_end_keys(const S* ends, int64_t n, const int64_t* seg, int G, uint32_t* const* kw,
                            cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const int K = end_key_words<S>(G);
    uint32_t* w[3] = {nullptr, nullptr, nullptr};
    for (int k = 0; k < K; ++k) w[k] = kw[k];
    k_end_keys<S><<<blocks_for(n), kThreads, 0, st>>>(ends, n, seg, G, w[0], w[1], w[2]);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_end_decode(const uint32_t* const* kw, int64_t n, int64_t n_pad, S* out, cudaStream_t st) {
    if (n_pad <= 0) return cudaSuccess;
    k_end_decode<S><<<blocks_for(n_pad), kThreads, 0, st>>>(kw[0], sizeof(S) == 8 ? kw[1] : nullptr, n, n_pad,
                                                           out);
    note_launch();
    return cudaGetLastError();
}

size_t branch_temp_bytes(int64_t n_pad) {
    const int64_t tiles = ceil_div(std::max<int64_t>(n_pad, 1), kBrTile);
    return (size_t)round_up(tiles, 64) * (2 * sizeof(int64_t) + sizeof(int)) + 1024;
}

template <typename S>
cudaError_t launch_branch(const S* ends, int64_t n, int64_t n_pad, Levels<S> L, int H,
                          const int64_t* seg, int G, int32_t* branch, cudaStream_t st, void* temp,
                          int* d_err) {
    if (n <= 0) return cudaSuccess;
    if (!temp || !d_err || H < 1) {
        k_branch<S><<<blocks_for(n_pad), kThreads, 0, st>>>(ends, n, n_pad, L, H, seg, G, branch);
        note_launch();
        return cudaGetLastError();
    }
    const int64_t tiles = ceil_div(n_pad, kBrTile);
    const int64_t tp = round_up(tiles, 64);
    char* p = static_cast<char*>(temp);
    S* t_max = reinterpret_cast<S*>(p);
    S* t_pre = t_max + tp;
    int* t_flag = reinterpret_cast<int*>(p + 2 * sizeof(int64_t) * tp);
    unsigned int* ctr = reinterpret_cast<unsigned int*>(t_flag + tp);
    cudaError_t e = cudaMemsetAsync(t_flag, 0, sizeof(int) * tp + 256, st);
    if (e != cudaSuccess) return e;
    k_branch_lookback<S><<<(unsigned)tiles, kThreads, 0, st>>>(ends, n, n_pad, L.p[0], seg, G, branch, t_max, t_pre,
                                                               t_flag, ctr, d_err);
    note_launch();
    return cudaGetLastError();
}

#define SIG_INST(S)                                                                              \
    template cudaError_t launch_check_sorted<S>(const S*, const S*, int64_t, const int64_t*, int, \
                                                int*, cudaStream_t);                             \
    template int key_words<S>(int);                                                              \
    template cudaError_t launch_make_keys<S>(const S*, const S*, int64_t, const int64_t*, int,    \
                                             uint32_t* const*, uint32_t*, cudaStream_t);         \
    template cudaError_t launch_decode<S>(const uint32_t* const*, const uint32_t*, const int32_t*, \
                                          int64_t, int64_t, S*, S*, int32_t*, cudaStream_t);     \
    template cudaError_t launch_copy_pad<S>(const S*, const S*, const int32_t*, int64_t, int64_t, \
                                            S*, S*, int32_t*, uint32_t*, cudaStream_t);          \
    template cudaError_t launch_pyramid<S>(const S*, const int64_t*, int, S* const*, cudaStream_t); \
    template cudaError_t launch_long_flags<S>(const S*, const S*, int64_t, int64_t, uint32_t*, cudaStream_t); \
    template cudaError_t launch_long_scatter<S>(const S*, const S*, int64_t, int64_t, const int64_t*, int64_t, \
                                                int64_t, const int64_t*, int, int32_t*, S*, int64_t*,        \
                                                cudaStream_t);                                               \
    template cudaError_t launch_branch<S>(const S*, int64_t, int64_t, Levels<S>, int,           \
                                          const int64_t*, int, int32_t*, cudaStream_t, void*, int*); \
    template int end_key_words<S>(int);                                                          \
    template cudaError_t launch_long_depth<S>(const S*, const S*, int64_t, const int64_t*, int, int64_t,         \
                                              unsigned long long*,                                              \
                                              cudaStream_t);                                                    \
    template cudaError_t launch_end_keys<S>(const S*, int64_t, const int64_t*, int, uint32_t* const*, \
                                            cudaStream_t);                                       \
    template cudaError_t launch_end_decode<S>(const uint32_t* const*, int64_t, int64_t, S*, cudaStream_t);
SIG_INST(int32_t)
SIG_INST(int64_t)

}  // namespace sig
