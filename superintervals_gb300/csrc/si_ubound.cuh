// si_ubound.cuh -- upper-bound search: last k with starts[k] <= v inside one contig.
//
// Three interchangeable providers, all exact:
//   binary     the reference's branch-free halving search (src/superintervals.hpp:501-516);
//   eytzinger  the top levels of the contig's sorted starts sampled into a breadth-first
//              (Eytzinger) tree -- the layout of IntervalMapEytz (hpp:1457-1535), here only
//              as an accelerator: the tree picks a bucket of sorted positions, a bounded
//              halving search inside the bucket gives the answer;
//   learned    a two-stage piecewise-linear model (root model -> one of up to 4096 leaf
//              segments -> predicted position) with each leaf's stored max error; a bounded
//              search inside the error window, then a two-read check of the answer, with the
//              full halving search as fallback whenever the check fails.
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
    const double2* root;         // per contig: (slope, intercept) key -> leaf coordinate
    const int32_t* leaf_base;    // per contig+1
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
// `tree` (may be shared memory) holds the contig's Eytzinger keys, 1-based.
template <typename S>
__device__ __forceinline__ int64_t ub_search(const UbView<S>& U, int g, const S* __restrict__ starts,
                                             int64_t n, S v, const S* tree) {
    if (n <= 0) return -1;
    if (U.mode == 1 && U.eytz_n > 1) {
        const int64_t K = U.eytz_n - 1;
        int64_t i = 1;
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
        const double x = (double)v - U.key_mean[g];
        const double2 rt = U.root[g];
        const int base = U.leaf_base[g];
        const int nl = U.leaf_base[g + 1] - base;
        double lf = rt.x * x + rt.y;
        int l = lf <= 0.0 ? 0 : (lf >= (double)(nl - 1) ? nl - 1 : (int)lf);
        const LeafModel M = U.leaves[base + l];
        const double pred = M.y0 + M.slope * (x - M.x0);
        double plo = pred - (double)M.err_lo - 1.0, phi = pred + (double)M.err_hi + 1.0;
        int64_t a = plo <= 0.0 ? 0 : (plo >= (double)(n - 1) ? n - 1 : (int64_t)plo);
        int64_t b = phi <= 0.0 ? 0 : (phi >= (double)(n - 1) ? n - 1 : (int64_t)phi + 1);
        if (b > n - 1) b = n - 1;
        const int64_t r = ub_range(starts, a, b, v);
        const bool ok_lo = (r < 0) ? (v < starts[0]) : (starts[r] <= v);
        const bool ok_hi = (r + 1 >= n) || (starts[r + 1] > v);
        if (ok_lo && ok_hi) return r;
        // the model's window missed: full search (exact either way)
    }
    return ub_range(starts, (int64_t)0, n - 1, v);
}

}  // namespace sig
