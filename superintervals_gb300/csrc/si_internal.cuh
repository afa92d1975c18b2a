// si_internal.cuh -- shared device/host helpers of the GB300 overlap-query library.
//
// Index layout in HBM (one handle = one set of per-contig maps):
//   starts[n_pad], ends[n_pad]   coordinate type S (int32 or int64), sorted per
//                                contig by (start asc, end desc); padded to a
//                                multiple of 32 with S_MAX / S_MIN
//   data[n]                      int32 payload, permuted with the intervals
//   branch[n]                    int32 GLOBAL position of the nearest preceding
//                                interval of the same contig with end >= ends[i],
//                                or -1 (the reference's SIZE_MAX)
//   seg[G+1]                     int64 contig offsets
//   lvl[h][...]                  max-of-32 pyramid over ends (h = 1..H), each level
//                                padded to a multiple of 32 with S_MIN
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace sig {

constexpr int kWarp = 32;
constexpr uint32_t kFull = 0xffffffffu;

template <typename S> struct Lim;
template <> struct Lim<int32_t> {
    static constexpr int32_t lo = INT32_MIN;
    static constexpr int32_t hi = INT32_MAX;
};
template <> struct Lim<int64_t> {
    static constexpr int64_t lo = INT64_MIN;
    static constexpr int64_t hi = INT64_MAX;
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Counts the library's own kernel launches (reported by getLaunchCountGpu).
void note_launch(int n = 1);
inline int64_t round_up(int64_t a, int64_t b) { return ceil_div(a, b) * b; }

// Device-side error word written by kernels that detect bad input or give up
// on a bounded wait; the host reads it after the launch sequence.
enum DeviceError : int {
    kDevOk = 0,
    kDevBadContig = 1,     // a query named a contig outside [0, G)
    kDevOverflow = 2,      // an output offset ran past the output capacity
    kDevTimeout = 3,       // a bounded wait on another block's published result gave up
};

// ---------------------------------------------------------------- scan
// Exclusive prefix sums over n values; `out` receives n+1 values (the last one
// is the total).  `temp` must hold scan_temp_bytes(n).  With d_err (a device error word) the
// u32 -> i64 scan is one kernel with decoupled look-back across tiles; a wait that gives up
// records kDevTimeout there.  Without it, tile totals are scanned first (reduce-then-scan).
size_t scan_temp_bytes(int64_t n);
cudaError_t exclusive_scan_u32_to_i64(const uint32_t* in, int64_t* out, int64_t n, void* temp,
                                      cudaStream_t st, int* d_err = nullptr);
cudaError_t exclusive_scan_u32_to_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp,
                                      cudaStream_t st);
// exclusive prefix sums mod 2^64 of signed coordinates (sign-extended), n + 1 entries
cudaError_t exclusive_scan_i32_to_u64(const int32_t* in, uint64_t* out, int64_t n, void* temp, cudaStream_t st);
cudaError_t exclusive_scan_i64_to_u64(const int64_t* in, uint64_t* out, int64_t n, void* temp, cudaStream_t st);

// ---------------------------------------------------------------- BED ingest (si_bed.cu)
int64_t bed_chunks(int64_t len);
cudaError_t launch_nl_count(const unsigned char* text, int64_t len, uint32_t* counts, cudaStream_t st);
cudaError_t launch_nl_write(const unsigned char* text, int64_t len, const int64_t* offs, int64_t* nl,
                            cudaStream_t st);
cudaError_t launch_bed_parse(const unsigned char* t, int64_t len, const int64_t* nl, int64_t n_nl, int64_t n_lines,
                             int half_open, int64_t lo_lim, int64_t hi_lim, uint8_t* status, uint32_t* valid,
                             uint64_t* hash, int64_t* start, int64_t* end, int64_t* name_off, int32_t* name_len,
                             cudaStream_t st);
cudaError_t launch_bed_compact(const uint32_t* valid, const int64_t* offs, int64_t n_lines, const uint64_t* hash,
                               const int64_t* start, const int64_t* end, const int64_t* name_off,
                               const int32_t* name_len, uint32_t* h_lo, uint32_t* h_hi, uint32_t* rec_id,
                               int64_t* r_start, int64_t* r_end, int64_t* r_noff, int32_t* r_nlen, int64_t* r_line,
                               cudaStream_t st);
cudaError_t launch_hash_heads(const uint32_t* lo, const uint32_t* hi, int64_t m, uint32_t* head, cudaStream_t st);
cudaError_t launch_hash_groups(const unsigned char* t, const uint32_t* head, const uint32_t* ex,
                               const uint32_t* perm, int64_t m, const int64_t* r_noff, const int32_t* r_nlen,
                               uint32_t* gid, uint32_t* first, uint32_t* grp_key, int* collision, cudaStream_t st);
cudaError_t launch_record_contig(const uint32_t* sorted_groups, int64_t G, uint32_t* rank, const uint32_t* gid,
                                 const uint32_t* perm, int64_t m, uint32_t* cid, cudaStream_t st);
template <typename S>
cudaError_t launch_bed_out(const uint32_t* cid_sorted, const uint32_t* order, int64_t m, const int64_t* r_start,
                           const int64_t* r_end, const int64_t* r_line, S* os, S* oe, int32_t* oline, int64_t* seg,
                           cudaStream_t st);
cudaError_t launch_bed_lookup(const unsigned char* t, const uint32_t* h_lo, const uint32_t* h_hi,
                              const int64_t* r_noff, const int32_t* r_nlen, int64_t m, const uint64_t* ctg_hash,
                              const int32_t* ctg_id, int G, const unsigned char* names, const int64_t* name_at,
                              int32_t* qc, cudaStream_t st);
cudaError_t launch_iota_u32(uint32_t* out, int64_t n, cudaStream_t st);
cudaError_t launch_known(const int32_t* qc, int64_t m, uint32_t* flag, cudaStream_t st);
template <typename S>
cudaError_t launch_query_out(const int32_t* qc, const int64_t* offs, int64_t m, const int64_t* r_start,
                             const int64_t* r_end, const int64_t* r_line, S* qs, S* qe, int32_t* qc_out,
                             int64_t* line_out, cudaStream_t st);
cudaError_t launch_contig_names(const uint32_t* first_rec, const int64_t* r_noff, const int32_t* r_nlen, int64_t G,
                                int64_t* off, int32_t* len, cudaStream_t st);

// ---------------------------------------------------------------- sort
// Stable LSD radix sort of n records whose key is K 32-bit words (word 0 least
// significant) with one 32-bit payload.  keys[w] / payload are double
// buffered with alt_keys[w] / alt_payload; the sorted result is left in the
// buffers reported through *result_in_alt.  Passes whose digit is constant
// over all records are skipped (the digit histograms are read back to the host).  With a
// nonzero pass_mask exactly the passes of its bits run (bit 4w + b: byte b of word w), with
// no host round trip, so that the sort can be captured in a CUDA graph.
constexpr int kMaxKeyWords = 5;
size_t radix_temp_bytes(int64_t n, int K);
// With d_err (a device error word) each pass is one kernel with decoupled look-back across
// tiles (one-sweep); a wait that gives up records kDevTimeout there.  Without it, each pass is
// a tile histogram, a scan and a scatter.
// With hist_ready the caller has already written the digit histograms of every key byte into
// radix_hist(temp) (K x 4 x 256 counts, byte b of word w at (4w + b) x 256).
cudaError_t radix_sort(uint32_t* const* keys, uint32_t* const* alt_keys, uint32_t* payload,
                       uint32_t* alt_payload, int K, int64_t n, void* temp, size_t temp_bytes,
                       bool* result_in_alt, int* passes_run, cudaStream_t st, uint32_t pass_mask = 0,
                       int* d_err = nullptr, bool hist_ready = false);
uint32_t* radix_hist(void* temp);

// ---------------------------------------------------------------- build
template <typename S>
struct IndexView {
    const S* starts;
    const S* ends;
    const int32_t* data;
    const int32_t* branch;
    const int64_t* seg;
    int32_t n_seg;
    int64_t n;
    int n_levels;              // H: pyramid levels above ends
    const S* lvl[8];           // lvl[h-1] = level h maxima
};

}  // namespace sig

namespace sig {

// Pyramid level pointers passed by value to kernels.
template <typename S>
struct Levels {
    const S* p[8];
};
constexpr int kMaxLevels = 8;

// ---------------------------------------------------------------- build launchers (si_build.cu)
// Sets *d_flag to 1 when some contig is NOT in canonical (start asc, end desc)
// order, following the add() flag logic of src/superintervals.hpp:95-105.
template <typename S>
cudaError_t launch_check_sorted(const S* s, const S* e, int64_t n, const int64_t* seg, int G,
                                int* d_flag, cudaStream_t st);
// Number of 32-bit key words for a coordinate type and contig count.
template <typename S>
int key_words(int G);
template <typename S>
cudaError_t launch_make_keys(const S* s, const S* e, int64_t n, const int64_t* seg, int G,
                             uint32_t* const* kw, uint32_t* payload, cudaStream_t st);
// Decode sorted keys back into padded starts/ends and gather the payload.
template <typename S>
cudaError_t launch_decode(const uint32_t* const* kw, const uint32_t* perm, const int32_t* data_in,
                          int64_t n, int64_t n_pad, S* starts, S* ends, int32_t* data,
                          cudaStream_t st);
// Identity build (input already canonical): copy + pad.
template <typename S>
cudaError_t launch_copy_pad(const S* s_in, const S* e_in, const int32_t* d_in, int64_t n,
                            int64_t n_pad, S* starts, S* ends, int32_t* data, uint32_t* perm,
                            cudaStream_t st);
// Pyramid sizes: fills sizes[0..H] (sizes[0] = n_pad) and returns H.
int pyramid_levels(int64_t n_pad, int64_t* sizes);
template <typename S>
cudaError_t launch_pyramid(const S* ends, const int64_t* sizes, int H, S* const* lvl,
                           cudaStream_t st);
// long-interval list (end - start >= X) in position order: flags per interval; then, with
// offs = exclusive scan of the flags (n + 1 entries), the positions and ends of the n_long
// long intervals padded to n_long_pad, and each contig's first list index (G + 1 entries)
template <typename S>
cudaError_t launch_long_flags(const S* starts, const S* ends, int64_t n, int64_t X, uint32_t* flags,
                              cudaStream_t st);
template <typename S>
cudaError_t launch_long_scatter(const S* starts, const S* ends, int64_t n, int64_t X, const int64_t* offs,
                                int64_t n_long, int64_t n_long_pad, const int64_t* seg, int G, int32_t* pos,
                                S* lend, int64_t* long_seg, cudaStream_t st);
// flag = 1 when a[i] != b[i] for some i < n
cudaError_t launch_differs_i32(const int32_t* a, const int32_t* b, int64_t n, int* flag, cudaStream_t st);
// branch array: with temp (branch_temp_bytes(n_pad)) and an error word, one kernel with
// decoupled look-back across tiles; otherwise the pyramid climb
size_t branch_temp_bytes(int64_t n_pad);
template <typename S>
cudaError_t launch_branch(const S* ends, int64_t n, int64_t n_pad, Levels<S> L, int H,
                          const int64_t* seg, int G, int32_t* branch, cudaStream_t st, void* temp = nullptr,
                          int* d_err = nullptr);
// each contig's ends in ascending order: sort keys (end_key_words<S>(G) words, for
// radix_sort), then the sorted keys decoded into out[0, n_pad) (padding: the largest value)
template <typename S>
int end_key_words(int G);
template <typename S>
cudaError_t launch_end_keys(const S* ends, int64_t n, const int64_t* seg, int G, uint32_t* const* kw,
                            cudaStream_t st);
template <typename S>
cudaError_t launch_end_decode(const uint32_t* const* kw, int64_t n, int64_t n_pad, S* out, cudaStream_t st);
// out[0] = total length of intervals at least X long, out[1] = total contig extent (sorted starts)
template <typename S>
cudaError_t launch_long_depth(const S* starts, const S* ends, int64_t n, const int64_t* seg, int G, int64_t X,
                              unsigned long long* out, cudaStream_t st);

// ---------------------------------------------------------------- query launchers (si_query.cu)
struct QueryBatch {
    const void* qs;          // S[nq]
    const void* qe;          // S[nq]
    const int32_t* qc;       // contig per query, or nullptr (all contig 0)
    int64_t nq;
};

enum Order : int { kOrderIdxsCpp = 0, kOrderDesc = 1 };

// One interval as one aligned record (start, end, payload): the operations that read all of a
// hit's fields (intersection, difference, keys, coverage) then make one memory transaction per
// hit instead of one per field.
template <typename S>
struct IvRec;
template <>
struct alignas(16) IvRec<int32_t> {
    int32_t s, e, d, pad;
};
template <>
struct alignas(32) IvRec<int64_t> {
    int64_t s, e;
    int32_t d, pad;
    int64_t pad2;
};

template <typename S>
struct MapView {
    const S* starts;
    const S* ends;
    const int32_t* branch;
    const int32_t* data;
    const int64_t* seg;
    int32_t G;
    int64_t n;
    const S* end_sorted = nullptr;  // each contig's ends ascending; only when no interval has start > end
    const IvRec<S>* rec = nullptr;  // the intervals as records, where an operation asked for them
};

// rec[i] = (starts[i], ends[i], data[i]) for i < n
template <typename S>
cudaError_t launch_records(const S* starts, const S* ends, const int32_t* data, int64_t n, IvRec<S>* rec,
                           cudaStream_t st);

// set operations over hit lists (CSR of contig-local positions): intersection pieces (kept when
// start <= end) and difference pieces; counts when ooff is null, else writes at ooff
template <typename S>
cudaError_t launch_isect(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits,
                         uint32_t* counts, const int64_t* ooff, S* os, S* oe, int32_t* ob, int* d_err,
                         cudaStream_t st);
template <typename S>
cudaError_t launch_diff(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits, bool sequential,
                        uint32_t* counts, const int64_t* ooff, S* os, S* oe, int* d_err, cudaStream_t st);
// the hits' (start, end, data) in hit-list order (od may be null)
template <typename S>
cudaError_t launch_keys(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits, S* os, S* oe,
                        int32_t* od, cudaStream_t st);
// per query: number of hits and the wrapped sum of min(end, qe) - max(start, qs)
template <typename S>
cudaError_t launch_coverage(MapView<S> m, QueryBatch q, const int64_t* hoff, const int32_t* hits,
                            uint64_t* count, S* cov, cudaStream_t st);
// flag = 1 when some interval has start > end
template <typename S>
cudaError_t launch_any_inverted(MapView<S> m, int* flag, cudaStream_t st);

// error word = kDevBadContig when a contig id is outside [0, G) (for empty indexes, where no
// other kernel reads the ids)
cudaError_t launch_check_contigs(const int32_t* qc, int64_t nq, int G, int* d_err, cudaStream_t st);

// plain one-query-per-thread path: upper_bound + branch walk per query
template <typename S>
cudaError_t launch_count_plain(MapView<S> m, QueryBatch q, uint32_t* counts, int* d_err,
                               cudaStream_t st);
template <typename S>
cudaError_t launch_emit_plain(MapView<S> m, QueryBatch q, const int64_t* offsets, int64_t out_base,
                              int order, bool values, int32_t* out, int* d_err, cudaStream_t st,
                              int64_t total_cap = INT64_MAX);
template <typename S>
cudaError_t launch_any_plain(MapView<S> m, QueryBatch q, uint8_t* out, int* d_err,
                             cudaStream_t st);

}  // namespace sig
