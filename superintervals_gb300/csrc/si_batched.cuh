// si_batched.cuh -- the BATCHED query path (sorted-query tiles).
#pragma once
#include "si_internal.cuh"

namespace sig {

// Device allocation through the library's budgeted allocator (si_capi.cu).
int dev_reserve(void** p, size_t* bytes, size_t need);
void dev_release(void** p, size_t* bytes);

struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { dev_release(&p, &bytes); }
    int reserve(size_t need) { return dev_reserve(&p, &bytes, need); }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

// Tunables of the batched path (picked by the autotuner, see si_autotune in the C-ABI).
struct BatchedParams {
    int tile_q = 256;            // sorted queries per tile
    int cap = 2048;              // candidate slots per tile (shared memory)
    int64_t long_len = 16384;    // queries longer than this take the per-query walk
    int64_t split_len = 2048;    // candidates at least this long form the tile's long list
    int eytz_depth = 0;          // 0: automatic
    // emit: copy the section of a tile's long candidates that comes from the long-interval list
    // (all hits but a few) as runs between its misses instead of checking each candidate (the
    // check measured faster on configuration 3; the autotuner tries both)
    bool emit_copy = false;
    // pick tile_q per batch (emit without a count-pass cache) from the batch's intervals per
    // query and hits per query, so that a tile's candidates fit its shared memory
    bool auto_tile = true;
};

// Per-contig upper-bound accelerators built once per index.
struct UpperBoundModel {
    int mode = 0;                // SI_UB_*
    int G = 0;
    // learned: two-stage piecewise-linear model per contig
    DBuf leaf_base;              // int32 per contig+1: first leaf of each contig
    DBuf leaf_key;               // S per leaf: its first key (the root, equal-count leaves)
    DBuf leaf_pos;               // int32 per leaf: its first contig-local position
    DBuf leaves;                 // LeafModel per leaf
    DBuf key_mean;               // double per contig: key offset for conditioning
    int total_leaves = 0;
    int leaves_per_contig = 0;
    // eytzinger: top levels of each contig, laid out breadth-first
    DBuf eytz_keys;              // S[G * eytz_n]
    DBuf eytz_pos;               // int32[G * eytz_n]: position of each sampled key
    int eytz_n = 0;              // keys per contig (2^depth - 1)
    int eytz_depth = 0;
};

struct BatchedWorkspace {
    BatchedParams prm;
    UpperBoundModel ub;
    // query sort
    DBuf kw[3], kalt[3], pay, palt, sort_tmp;
    DBuf qpair;                  // (start, end) per query, interleaved: one sector per gather
    DBuf blk_cut;                // per 256 sorted queries: (p_cut, long-list end) or -1, for the tiles
    DBuf qminmax;                // smallest and largest query end (key packing)
    // sorted query records
    DBuf sq_s, sq_u, sq_c, sq_id;
    DBuf heads;                  // head-run length per query (original order)
    DBuf counters;               // work-queue counters
    // identity of the batch the sorted records belong to
    const void* prepared_qs = nullptr;
    int64_t prepared_nq = -1;
    int prepared_mode = -1;
    int64_t n_heads = 0;
    long long launches = 0;      // kernels launched by this path
    // candidate lists of every tile, written by the count pass, read by the emit pass
    DBuf tile_cache;
    bool cache_ok = false;
    int64_t cache_stride = 0;
    int cache_prm_tile = 0, cache_prm_cap = 0;
    // tiles kernels (count, emit): dynamic shared memory their attribute was set for, and
    // resident blocks on the device at that size
    size_t occ_smem[2] = {0, 0};
    int occ_blocks[2] = {0, 0};
    // long-interval list: global positions and ends of the intervals at least long_split long,
    // in position order, its max pyramid (long_H levels) and each contig's first list index
    const void* long_ends = nullptr;
    const int32_t* long_pos = nullptr;
    const int64_t* long_seg = nullptr;
    const void* long_lvl[kMaxLevels] = {nullptr};
    int long_H = 0;
    int64_t long_split = 0;
    // each contig's ends in ascending order (positions as the index), when no interval has
    // start > end: short queries are then counted from two ranks instead of the tile lists
    const void* end_sorted = nullptr;
    // graph capture of the whole path: no host round trips (device-side key packing, fixed
    // sort passes) and an emit that skips the queries whose lists would end past out_cap
    bool capturing = false;
    DBuf qpack;                  // {shift, end bits} of the packed query key
    int64_t out_cap = INT64_MAX; // values the emit's output holds
};

// Bits of the batched path's query class codes (0 .. 3G: short, long and start > end queries
// of each contig, and contig ids outside [0, G)).
inline int query_code_bits(int G) {
    int b = 1;
    while (b < 32 && ((uint64_t)1 << b) <= (uint64_t)(3 * (int64_t)G)) ++b;
    return b;
}

// Interval length from which an interval enters the long-interval list.
constexpr int64_t kLongIntervalSplit = 32768;

template <typename S>
int batched_prepare(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const int64_t* lvl_sizes,
                    int ub_mode, cudaStream_t st);
// Sorts the queries by (class, contig, end) and finds each one's upper bound.  With counts and
// an index that keeps its sorted ends (no interval has start > end), also writes the count of
// every short query (the count pass then handles the long ones only).
// tile_cuts: also record each 256-query block's long-list cut for the tiles (search paths).
template <typename S>
int batched_prepare_queries(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, int* d_err,
                            int ub_mode, cudaStream_t st, uint32_t* counts = nullptr, bool tile_cuts = true);
template <typename S>
int batched_count(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q,
                  uint32_t* counts, int* d_err, cudaStream_t st);
// q may be a slice [q_offset, q_offset + q.nq) of the batch counted last.
// total_hits: the result count of the whole batch prepared last (-1 unknown), for the tile size.
template <typename S>
int batched_emit(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q,
                 int64_t q_offset, const int64_t* offsets, int64_t out_base, int order, bool values,
                 int32_t* out, int* d_err, int ub_mode, cudaStream_t st, int64_t total_hits = -1);

// Coverage (count and the wrapped sum of min(end, qe) - max(start, qs)) of every query, from
// ranks and prefix sums (ps_start / ps_end: exclusive prefix sums mod 2^64 of the starts and of
// the sorted ends, n + 1 entries).  Needs the sorted ends (no interval with start > end) and
// queries with start <= end.
template <typename S>
int batched_coverage(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, const uint64_t* ps_start,
                     const uint64_t* ps_end, uint64_t* count, S* cov, int* d_err, int ub_mode, cudaStream_t st);

// Upper bound of every query end (original order) with the handle's accelerator.  Per query
// (one thread each, in the batch's order), or, with sorted, through the batched path's
// preparation: the ends are radix-sorted, each block of 256 sorted ends searches only its
// smallest and largest end and resolves the rest in a shared-memory window of starts, and the
// answers are scattered back to the original order.
template <typename S>
int upper_bounds(BatchedWorkspace& ws, MapView<S> m, const QueryBatch& q, int ub_mode, int32_t* out,
                 int* d_err, cudaStream_t st, bool sorted = false);

}  // namespace sig
