// si_ubound.cuh -- upper-bound search: last k with starts[k] <= v inside one contig.
//
// Three interchangeable providers, all exact:
//   binary     the reference's branch-free halving search (src/superintervals.hpp:501-516);
//   eytzinger  the top levels of the contig's sorted starts sampled into a breadth-first
//              (Eytzinger) tree -- the layout of IntervalMapEytz (hpp:1457-1535), here only
//              as an accelerator: the tree picks a bucket of sorted positions, a bounded
//              halving search inside the bucket gives the answer;
//   learned    a two-stage piecewise-linear model.  Stage 1 (root): the contig's sorted starts
//              cut into up to 4096 leaves of equal count; the leaves' first keys form a
//              piecewise-linear map from key to leaf, searched per query.  Stage 2: each leaf
//              a least-squares line (key -> position) with its stored max errors.  The answer
//              lies inside the chosen leaf's position range, so the error window is clamped
//              to it; a two-read check of the answer falls back to a halving search over the
//              leaf whenever it fails (exact either way).  Equal-count leaves keep every leaf
//              small where keys are clustered (a root line over the key range would put a
//              whole hotspot into one leaf).
#pragma once
#include "si_internal.cuh"

namespace sig {

struct LeafModel {
    double x0;      // key offset of the leaf
    double slope;   // positions per key unit
    double y0;      // predicted position at x0
    int32_t err_lo; // max(pred - k) over the leaf's keys (>= 0)
    int32_t err_hi; // max(k - pred) over the leaf's keys (>= 0)
};

template <typename S>
struct UbView {
    int mode;                    // SI_UB_*: 0 binary, 1 eytzinger, 2 learned
    // learned
    const int32_t* leaf_base;    // per contig+1: first leaf of each contig
    const S* leaf_key;           // per leaf: its first key (the root)
    const int32_t* leaf_pos;     // per leaf: its first contig-local position
    const LeafModel* leaves;
    const double* key_mean;      // per contig: key origin
    // eytzinger
    const S* eytz_keys;          // G * eytz_n, 1-based per contig (slot 0 unused)
    int eytz_n;                  // slots per contig including the unused slot 0
};

// last k in [a, b] (inclusive, local positions) with starts[k] <= v, else a-1
template <typename S>
__device__ __forceinline__ int64_t ub_range(const S* __restrict__ starts, int64_t a, int64_t b, S v) {
    int64_t length = b - a + 1;
    if (length <= 0) return a - 1;
    int64_t idx = a;
    while (length > 1) {
        const int64_t half = length >> 1;
        idx += (starts[idx + half] <= v) ? (length - half) : 0;
        length = half;
    }
    return (starts[idx] > v) ? idx - 1 : idx;
}

// Position of rank r among the K evenly spaced samples of a contig of n keys.
__device__ __forceinline__ int64_t eytz_sample_pos(int64_t r, int64_t n, int64_t K) {
    return ((r + 1) * n) / (K + 1);
}

// Upper bound inside one contig: starts points at the contig's first key, n keys.
// `tree` holds the contig's Eytzinger keys, 1-based; its slots below `top_n` may also be
// read from `top` (the tree's top levels staged in shared memory).
template <typename S>
__device__ __forceinline__ int64_t ub_search(const UbView<S>& U, int g, const S* __restrict__ starts,
                                             int64_t n, S v, const S* tree, const S* top = nullptr,
                                             int64_t top_n = 0) {
    if (n <= 0) return -1;
    if (U.mode == 1 && U.eytz_n > 1) {
        const int64_t K = U.eytz_n - 1;
        int64_t i = 1;
        while (i < top_n) i = 2 * i + (top[i] <= v ? 1 : 0);
        while (i <= K) i = 2 * i + (tree[i] <= v ? 1 : 0);
        i >>= __ffsll(~i);
        // rank of the first sample > v (K when every sample is <= v)
        int64_t r;
        if (i == 0) {
            r = K;
        } else {
            // in-order rank of 1-based BFS node i of a complete tree with K nodes
            const int levels = 63 - __clzll(K + 1);    // K = 2^levels - 1
            const int lvl = 63 - __clzll(i);           // depth of node i (root 0)
            const int64_t off = i - ((int64_t)1 << lvl);  // index within its level
            const int below = levels - 1 - lvl;        // levels under node i
            r = ((2 * off + 1) << below) - 1;
        }
        const int64_t lo = (r == 0) ? 0 : eytz_sample_pos(r - 1, n, K);
        const int64_t hi = (r == K) ? n - 1 : eytz_sample_pos(r, n, K) - 1;
        // ub in [lo-1, hi]; starts[lo] <= v whenever r > 0
        return ub_range(starts, lo, hi, v);
    }
    if (U.mode == 2 && U.leaves) {
        if (v < starts[0]) return -1;
        const int base = U.leaf_base[g];
        const int nl = U.leaf_base[g + 1] - base;
        // root: the last leaf whose first key is <= v (leaf 0 starts at starts[0] <= v)
        const S* __restrict__ lk = U.leaf_key + base;
        int l0 = 0, len = nl;
        while (len > 1) {
            const int half = len >> 1;
            l0 += (lk[l0 + half] <= v) ? (len - half) : 0;
            len = half;
        }
        if (lk[l0] > v) --l0;  // >= 0: lk[0] = starts[0] <= v
        // the answer lies in the leaf: starts[pa] <= v < starts[first position of leaf l0 + 1]
        const int64_t pa = U.leaf_pos[base + l0];
        const int64_t pb = (l0 + 1 < nl ? (int64_t)U.leaf_pos[base + l0 + 1] : n) - 1;
        const LeafModel M = U.leaves[base + l0];
        const double pred = M.y0 + M.slope * ((double)v - U.key_mean[g] - M.x0);
        const double plo = pred - (double)M.err_lo - 1.0, phi = pred + (double)M.err_hi + 1.0;
        int64_t a = plo <= (double)pa ? pa : (plo >= (double)pb ? pb : (int64_t)plo);
        int64_t b = phi >= (double)pb ? pb : (phi <= (double)pa ? pa : (int64_t)phi + 1);
        if (b > pb) b = pb;
        const int64_t r = ub_range(starts, a, b, v);
        const bool ok_lo = r >= pa && starts[r] <= v;
        const bool ok_hi = (r + 1 >= n) || (starts[r + 1] > v);
        if (ok_lo && ok_hi) return r;
        return ub_range(starts, pa, pb, v);  // the window missed: the whole leaf
    }
    return ub_range(starts, (int64_t)0, n - 1, v);
}

}  // namespace sig
