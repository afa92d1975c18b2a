// si_bed.cu -- BED text ingest on the GPU: the format step in front of the index.
//
// The reference reads BED with per-line host parsers (examples/bed-intersect-si.rs:63-120
// parse_bed_line / read_bed_file: chrom = first tab field, start = second, end = third - 1,
// lines with end < 0 or end < start skipped, intervals bucketed per chrom in a hash map;
// test/bench.cpp:67-102 load_intervals).  Here the whole text sits in device memory:
//
//   1. newline index: each 8 KiB chunk counts its '\n' bytes; a scan of the chunk counts
//      gives every chunk its output offset; each chunk writes its newline positions in order.
//   2. parse: one thread per line.  Header lines ('#', "track", "browser"), empty lines and
//      lines with fewer than three tab-separated columns or a non-integer start / end are
//      skipped; the chrom name is hashed (FNV-1a, 64 bit); start and end are parsed as
//      decimal integers with an optional '-' sign.
//   3. contig dictionary and bucketing (host-driven sorts in si_capi.cu): records are
//      radix-sorted by name hash, names inside a hash group are compared byte by byte (a
//      collision is an error, never a silent merge), contig ids follow first appearance in
//      the file, and a stable sort by contig id groups the records per contig in file order.
#include <algorithm>
#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
constexpr int kBytesPerThread = 32;
constexpr int kChunk = kThreads * kBytesPerThread;  // 8192 bytes per block

__device__ __forceinline__ uint32_t count_nl(const unsigned char* b, int n) {
    uint32_t c = 0;
    for (int k = 0; k < n; ++k) c += b[k] == '\n' ? 1u : 0u;
    return c;
}

// This thread's up to 32 bytes of the chunk (global offset base + 32 * tid).
__device__ __forceinline__ int load_bytes(const unsigned char* __restrict__ text, int64_t len, int64_t base,
                                          unsigned char* b) {
    const int64_t p = base + (int64_t)threadIdx.x * kBytesPerThread;
    const int n = (int)std::max<int64_t>(0, std::min<int64_t>(kBytesPerThread, len - p));
    if (n == kBytesPerThread && ((p & 15) == 0)) {
        const uint4 v0 = *reinterpret_cast<const uint4*>(text + p);
        const uint4 v1 = *reinterpret_cast<const uint4*>(text + p + 16);
        *reinterpret_cast<uint4*>(b) = v0;
        *reinterpret_cast<uint4*>(b + 16) = v1;
    } else {
        for (int k = 0; k < n; ++k) b[k] = text[p + k];
    }
    return n;
}

__global__ void __launch_bounds__(kThreads) k_nl_count(const unsigned char* __restrict__ text, int64_t len,
                                                       uint32_t* __restrict__ counts) {
    __align__(16) unsigned char b[kBytesPerThread];
    const int64_t base = (int64_t)blockIdx.x * kChunk;
    const int n = load_bytes(text, len, base, b);
    uint32_t c = count_nl(b, n);
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
    __shared__ uint32_t ws[kThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < kThreads / 32; ++w) t += ws[w];
        counts[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kThreads) k_nl_write(const unsigned char* __restrict__ text, int64_t len,
                                                       const int64_t* __restrict__ offs, int64_t* __restrict__ nl) {
    __align__(16) unsigned char b[kBytesPerThread];
    const int64_t base = (int64_t)blockIdx.x * kChunk;
    const int n = load_bytes(text, len, base, b);
    const uint32_t c = count_nl(b, n);
    // block exclusive scan of the per-thread counts (thread order = byte order)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = c;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(kFull, incl, d);
        if (lane >= d) incl += o;
    }
    __shared__ uint32_t ws[kThreads / 32];
    if (lane == 31) ws[w] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (int k = 0; k < w; ++k) before += ws[k];
    int64_t at = offs[blockIdx.x] + before + incl - c;
    const int64_t p = base + (int64_t)threadIdx.x * kBytesPerThread;
    for (int k = 0; k < n; ++k)
        if (b[k] == '\n') nl[at++] = p + k;
}

// Decimal integer with an optional leading '-' over [b, e); false when empty, not all digits,
// or beyond 18 digits.
__device__ __forceinline__ bool parse_int(const unsigned char* __restrict__ t, int64_t b, int64_t e, int64_t* v) {
    bool neg = false;
    if (b < e && t[b] == '-') {
        neg = true;
        ++b;
    }
    if (b >= e || e - b > 18) return false;
    int64_t x = 0;
    for (int64_t p = b; p < e; ++p) {
        const unsigned char c = t[p];
        if (c < '0' || c > '9') return false;
        x = x * 10 + (c - '0');
    }
    *v = neg ? -x : x;
    return true;
}

__device__ __forceinline__ bool has_prefix(const unsigned char* __restrict__ t, int64_t b, int64_t e,
                                           const char* w, int n) {
    if (e - b < n) return false;
    for (int k = 0; k < n; ++k)
        if (t[b + k] != (unsigned char)w[k]) return false;
    return e - b == n || t[b + n] == ' ' || t[b + n] == '\t';
}

// One thread per line.  status: 0 interval, 1 skipped header / empty line, 2 malformed line,
// 3 filtered (end < 0 or end < start), 4 coordinate outside the handle's range.
__global__ void k_bed_parse(const unsigned char* __restrict__ t, int64_t len, const int64_t* __restrict__ nl,
                            int64_t n_nl, int64_t n_lines, int half_open, int64_t lo_lim, int64_t hi_lim,
                            uint8_t* __restrict__ status, uint32_t* __restrict__ valid, uint64_t* __restrict__ hash,
                            int64_t* __restrict__ start, int64_t* __restrict__ end, int64_t* __restrict__ name_off,
                            int32_t* __restrict__ name_len) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_lines) return;
    const int64_t b = k == 0 ? 0 : nl[k - 1] + 1;
    int64_t e = k < n_nl ? nl[k] : len;
    if (e > b && t[e - 1] == '\r') --e;
    uint8_t st = 0;
    int64_t s = 0, x = 0, p1 = b, p2 = 0, p3 = 0;
    uint64_t h = 1469598103934665603ull;  // FNV-1a offset basis
    if (e == b || t[b] == '#' || has_prefix(t, b, e, "track", 5) || has_prefix(t, b, e, "browser", 7)) {
        st = 1;
    } else {
        while (p1 < e && t[p1] != '\t') {
            h = (h ^ t[p1]) * 1099511628211ull;  // FNV-1a prime
            ++p1;
        }
        p2 = p1 + 1;
        while (p2 < e && t[p2] != '\t') ++p2;
        p3 = p2 + 1;
        while (p3 < e && t[p3] != '\t') ++p3;
        if (p1 >= e || p2 >= e || p1 == b || !parse_int(t, p1 + 1, p2, &s) || !parse_int(t, p2 + 1, p3, &x)) {
            st = 2;
        } else {
            if (half_open) x -= 1;  // BED ends are exclusive; the index is end-inclusive
            if (x < 0 || x < s) st = 3;
            else if (s < lo_lim || s > hi_lim || x < lo_lim || x > hi_lim) st = 4;
        }
    }
    status[k] = st;
    valid[k] = st == 0 ? 1u : 0u;
    hash[k] = h;
    start[k] = s;
    end[k] = x;
    name_off[k] = b;
    name_len[k] = (int32_t)(p1 - b);
}

// Compact the parsed lines into records (record r = the r-th interval line): hash words for
// the sort, coordinates, name location and line number.
__global__ void k_bed_compact(const uint32_t* __restrict__ valid, const int64_t* __restrict__ offs,
                              int64_t n_lines, const uint64_t* __restrict__ hash, const int64_t* __restrict__ start,
                              const int64_t* __restrict__ end, const int64_t* __restrict__ name_off,
                              const int32_t* __restrict__ name_len, uint32_t* __restrict__ h_lo,
                              uint32_t* __restrict__ h_hi, uint32_t* __restrict__ rec_id, int64_t* __restrict__ r_start,
                              int64_t* __restrict__ r_end, int64_t* __restrict__ r_noff, int32_t* __restrict__ r_nlen,
                              int64_t* __restrict__ r_line) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_lines || !valid[k]) return;
    const int64_t r = offs[k];
    h_lo[r] = (uint32_t)hash[k];
    h_hi[r] = (uint32_t)(hash[k] >> 32);
    rec_id[r] = (uint32_t)r;
    r_start[r] = start[k];
    r_end[r] = end[k];
    r_noff[r] = name_off[k];
    r_nlen[r] = name_len[k];
    r_line[r] = k;
}

// After the sort by hash: head[i] = 1 where a new hash starts.
__global__ void k_hash_heads(const uint32_t* __restrict__ lo, const uint32_t* __restrict__ hi, int64_t m,
                             uint32_t* __restrict__ head) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    head[i] = (i == 0 || lo[i] != lo[i - 1] || hi[i] != hi[i - 1]) ? 1u : 0u;
}

// Group number of each sorted record (gid = heads before it, inclusive, minus one) and the
// first sorted position of each group.
__global__ void k_hash_groups(const uint32_t* __restrict__ head, const uint32_t* __restrict__ ex, int64_t m,
                              uint32_t* __restrict__ gid, uint32_t* __restrict__ first) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t g = ex[i] + head[i] - 1;
    gid[i] = g;
    if (head[i]) first[g] = (uint32_t)i;
}

__global__ void k_name_check(const unsigned char* __restrict__ t, const uint32_t* __restrict__ gid,
                             const uint32_t* __restrict__ first, const uint32_t* __restrict__ perm, int64_t m,
                             const int64_t* __restrict__ r_noff, const int32_t* __restrict__ r_nlen,
                             uint32_t* __restrict__ grp_key, int* __restrict__ collision) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t g = gid[i], f = first[g];
    const uint32_t a = perm[i], b = perm[f];
    if ((int64_t)f == i) grp_key[g] = b;  // the group's first record: its first appearance (stable sort)
    const int32_t la = r_nlen[a], lb = r_nlen[b];
    bool same = la == lb;
    for (int32_t k = 0; same && k < la; ++k) same = t[r_noff[a] + k] == t[r_noff[b] + k];
    if (!same) atomicOr(collision, 1);
}

// contig id of each record: cid[perm[i]] = rank of its group by first appearance.
__global__ void k_record_contig(const uint32_t* __restrict__ gid, const uint32_t* __restrict__ perm, int64_t m,
                                const uint32_t* __restrict__ grp_rank, uint32_t* __restrict__ cid) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    cid[perm[i]] = grp_rank[gid[i]];
}

// rank[group] = position of the group in first-appearance order (payload of the sort).
__global__ void k_rank_of(const uint32_t* __restrict__ sorted_groups, int64_t G, uint32_t* __restrict__ rank) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < G) rank[sorted_groups[i]] = (uint32_t)i;
}

// After the sort by contig id: seg[c] = first position of contig c; gather the records.
template <typename S>
__global__ void k_bed_out(const uint32_t* __restrict__ cid_sorted, const uint32_t* __restrict__ order, int64_t m,
                          const int64_t* __restrict__ r_start, const int64_t* __restrict__ r_end,
                          const int64_t* __restrict__ r_line, S* __restrict__ os, S* __restrict__ oe,
                          int32_t* __restrict__ oline, int64_t* __restrict__ seg) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t r = order[i];
    os[i] = (S)r_start[r];
    oe[i] = (S)r_end[r];
    oline[i] = (int32_t)r_line[r];
    if (i == 0 || cid_sorted[i] != cid_sorted[i - 1]) seg[cid_sorted[i]] = i;
}

// Queries: contig id of each record from the index's sorted contig-name hashes (-1 when the
// name is not a contig of the index), name bytes compared with the index's name blob.
__global__ void k_bed_lookup(const unsigned char* __restrict__ t, const uint32_t* __restrict__ h_lo,
                             const uint32_t* __restrict__ h_hi, const int64_t* __restrict__ r_noff,
                             const int32_t* __restrict__ r_nlen, int64_t m, const uint64_t* __restrict__ ctg_hash,
                             const int32_t* __restrict__ ctg_id, int G, const unsigned char* __restrict__ names,
                             const int64_t* __restrict__ name_at, int32_t* __restrict__ qc) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint64_t h = ((uint64_t)h_hi[i] << 32) | h_lo[i];
    int lo = 0, hi = G;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ctg_hash[mid] < h) lo = mid + 1;
        else hi = mid;
    }
    int32_t id = -1;
    if (lo < G && ctg_hash[lo] == h) {
        const int32_t c = ctg_id[lo];
        const int64_t a = name_at[c], n = name_at[c + 1] - a;
        bool same = n == r_nlen[i];
        for (int64_t k = 0; same && k < n; ++k) same = names[a + k] == t[r_noff[i] + k];
        if (same) id = c;
    }
    qc[i] = id;
}

__global__ void k_iota(uint32_t* __restrict__ out, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (uint32_t)i;
}

// Name location of contig c from its first record (first_rec = the group keys in contig order).
__global__ void k_contig_names(const uint32_t* __restrict__ first_rec, const int64_t* __restrict__ r_noff,
                               const int32_t* __restrict__ r_nlen, int64_t G, int64_t* __restrict__ off,
                               int32_t* __restrict__ len) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= G) return;
    const uint32_t r = first_rec[c];
    off[c] = r_noff[r];
    len[c] = r_nlen[r];
}

__global__ void k_known(const int32_t* __restrict__ qc, int64_t m, uint32_t* __restrict__ flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) flag[i] = qc[i] >= 0 ? 1u : 0u;
}

// Queries on known contigs, in file order.
template <typename S>
__global__ void k_query_out(const int32_t* __restrict__ qc, const int64_t* __restrict__ offs, int64_t m,
                            const int64_t* __restrict__ r_start, const int64_t* __restrict__ r_end,
                            const int64_t* __restrict__ r_line, S* __restrict__ qs, S* __restrict__ qe,
                            int32_t* __restrict__ qc_out, int64_t* __restrict__ line_out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || qc[i] < 0) return;
    const int64_t k = offs[i];
    qs[k] = (S)r_start[i];
    qe[k] = (S)r_end[i];
    qc_out[k] = qc[i];
    line_out[k] = r_line[i];
}

inline unsigned blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, ceil_div(n, kThreads)); }

}  // namespace

int64_t bed_chunks(int64_t len) { return std::max<int64_t>(1, ceil_div(len, kChunk)); }

cudaError_t launch_nl_count(const unsigned char* text, int64_t len, uint32_t* counts, cudaStream_t st) {
    k_nl_count<<<(unsigned)bed_chunks(len), kThreads, 0, st>>>(text, len, counts);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_nl_write(const unsigned char* text, int64_t len, const int64_t* offs, int64_t* nl,
                            cudaStream_t st) {
    k_nl_write<<<(unsigned)bed_chunks(len), kThreads, 0, st>>>(text, len, offs, nl);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_bed_parse(const unsigned char* t, int64_t len, const int64_t* nl, int64_t n_nl, int64_t n_lines,
                             int half_open, int64_t lo_lim, int64_t hi_lim, uint8_t* status, uint32_t* valid,
                             uint64_t* hash, int64_t* start, int64_t* end, int64_t* name_off, int32_t* name_len,
                             cudaStream_t st) {
    if (n_lines <= 0) return cudaSuccess;
    k_bed_parse<<<blocks(n_lines), kThreads, 0, st>>>(t, len, nl, n_nl, n_lines, half_open, lo_lim, hi_lim, status,
                                                      valid, hash, start, end, name_off, name_len);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_bed_compact(const uint32_t* valid, const int64_t* offs, int64_t n_lines, const uint64_t* hash,
                               const int64_t* start, const int64_t* end, const int64_t* name_off,
                               const int32_t* name_len, uint32_t* h_lo, uint32_t* h_hi, uint32_t* rec_id,
                               int64_t* r_start, int64_t* r_end, int64_t* r_noff, int32_t* r_nlen, int64_t* r_line,
                               cudaStream_t st) {
    if (n_lines <= 0) return cudaSuccess;
    k_bed_compact<<<blocks(n_lines), kThreads, 0, st>>>(valid, offs, n_lines, hash, start, end, name_off, name_len,
                                                        h_lo, h_hi, rec_id, r_start, r_end, r_noff, r_nlen, r_line);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_hash_heads(const uint32_t* lo, const uint32_t* hi, int64_t m, uint32_t* head, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_hash_heads<<<blocks(m), kThreads, 0, st>>>(lo, hi, m, head);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_hash_groups(const unsigned char* t, const uint32_t* head, const uint32_t* ex,
                               const uint32_t* perm, int64_t m, const int64_t* r_noff, const int32_t* r_nlen,
                               uint32_t* gid, uint32_t* first, uint32_t* grp_key, int* collision, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_hash_groups<<<blocks(m), kThreads, 0, st>>>(head, ex, m, gid, first);
    note_launch();
    k_name_check<<<blocks(m), kThreads, 0, st>>>(t, gid, first, perm, m, r_noff, r_nlen, grp_key, collision);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_record_contig(const uint32_t* sorted_groups, int64_t G, uint32_t* rank, const uint32_t* gid,
                                 const uint32_t* perm, int64_t m, uint32_t* cid, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_rank_of<<<blocks(G), kThreads, 0, st>>>(sorted_groups, G, rank);
    note_launch();
    k_record_contig<<<blocks(m), kThreads, 0, st>>>(gid, perm, m, rank, cid);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_bed_out(const uint32_t* cid_sorted, const uint32_t* order, int64_t m, const int64_t* r_start,
                           const int64_t* r_end, const int64_t* r_line, S* os, S* oe, int32_t* oline, int64_t* seg,
                           cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_bed_out<S><<<blocks(m), kThreads, 0, st>>>(cid_sorted, order, m, r_start, r_end, r_line, os, oe, oline, seg);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_bed_lookup(const unsigned char* t, const uint32_t* h_lo, const uint32_t* h_hi,
                              const int64_t* r_noff, const int32_t* r_nlen, int64_t m, const uint64_t* ctg_hash,
                              const int32_t* ctg_id, int G, const unsigned char* names, const int64_t* name_at,
                              int32_t* qc, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_bed_lookup<<<blocks(m), kThreads, 0, st>>>(t, h_lo, h_hi, r_noff, r_nlen, m, ctg_hash, ctg_id, G, names,
                                                 name_at, qc);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_iota_u32(uint32_t* out, int64_t n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_iota<<<blocks(n), kThreads, 0, st>>>(out, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_contig_names(const uint32_t* first_rec, const int64_t* r_noff, const int32_t* r_nlen, int64_t G,
                                int64_t* off, int32_t* len, cudaStream_t st) {
    if (G <= 0) return cudaSuccess;
    k_contig_names<<<blocks(G), kThreads, 0, st>>>(first_rec, r_noff, r_nlen, G, off, len);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_known(const int32_t* qc, int64_t m, uint32_t* flag, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_known<<<blocks(m), kThreads, 0, st>>>(qc, m, flag);
    note_launch();
    return cudaGetLastError();
}

template <typename S>
cudaError_t launch_query_out(const int32_t* qc, const int64_t* offs, int64_t m, const int64_t* r_start,
                             const int64_t* r_end, const int64_t* r_line, S* qs, S* qe, int32_t* qc_out,
                             int64_t* line_out, cudaStream_t st) {
    if (m <= 0) return cudaSuccess;
    k_query_out<S><<<blocks(m), kThreads, 0, st>>>(qc, offs, m, r_start, r_end, r_line, qs, qe, qc_out, line_out);
    note_launch();
    return cudaGetLastError();
}
template cudaError_t launch_query_out<int32_t>(const int32_t*, const int64_t*, int64_t, const int64_t*,
                                               const int64_t*, const int64_t*, int32_t*, int32_t*, int32_t*,
                                               int64_t*, cudaStream_t);
template cudaError_t launch_query_out<int64_t>(const int32_t*, const int64_t*, int64_t, const int64_t*,
                                               const int64_t*, const int64_t*, int64_t*, int64_t*, int32_t*,
                                               int64_t*, cudaStream_t);

template cudaError_t launch_bed_out<int32_t>(const uint32_t*, const uint32_t*, int64_t, const int64_t*,
                                             const int64_t*, const int64_t*, int32_t*, int32_t*, int32_t*, int64_t*,
                                             cudaStream_t);
template cudaError_t launch_bed_out<int64_t>(const uint32_t*, const uint32_t*, int64_t, const int64_t*,
                                             const int64_t*, const int64_t*, int64_t*, int64_t*, int32_t*, int64_t*,
                                             cudaStream_t);

}  // namespace sig
