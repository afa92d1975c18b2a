// si_scan.cu -- device-wide exclusive prefix sum.
//
// Used for the per-query result offsets (count -> exclusive scan -> emit, the
// CSR form of the per-query result lists of src/superintervals/intervalmap.pyx:402-494)
// and for the digit offsets of the three-kernel radix sort.  HBM-bound.
//
// Two forms:
//  * single pass (u32 counts -> i64 offsets, when the caller passes a device error word):
//    a block takes the next 4096-value tile from an atomic counter, publishes its total, and
//    its first warp looks back over the earlier tiles' published totals 32 tiles at a time
//    (decoupled look-back: a tile's inclusive prefix, once published, ends the walk), then
//    publishes its own inclusive prefix and writes its offsets: one read and one write;
//  * reduce-then-scan: tile totals, their scan, then the tiles: two reads and one write.
#include <algorithm>

#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;   // 4096 values per block
constexpr int kWarps = kThreads / kWarp;

template <typename T>
__device__ __forceinline__ T warp_inclusive_sum(T x, int lane) {
#pragma unroll
    for (int d = 1; d < kWarp; d <<= 1) {
        T y = __shfl_up_sync(kFull, x, d);
        if (lane >= d) x += y;
    }
    return x;
}

// Per-tile totals.  Items are read warp-round-major (coalesced).
template <typename Tin, typename Tacc>
__global__ void __launch_bounds__(kThreads) k_tile_totals(const Tin* __restrict__ in, int64_t n,
                                                          Tacc* __restrict__ totals) {
    __shared__ Tacc wsum[kWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)w * (kItems * kWarp) + lane;
    Tacc s = 0;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        int64_t i = base + r * kWarp;
        if (i < n) s += (Tacc)in[i];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_xor_sync(kFull, s, d);
    if (lane == 0) wsum[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        Tacc t = 0;
#pragma unroll
        for (int k = 0; k < kWarps; ++k) t += wsum[k];
        totals[blockIdx.x] = t;
    }
}

// Scan of one tile with a precomputed tile prefix (or 0 when prefix == nullptr).
// out has n+1 slots; the block holding the last value writes the grand total.
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(kThreads) k_tile_scan(const Tin* __restrict__ in, int64_t n,
                                                        const Tout* __restrict__ prefix,
                                                        Tout* __restrict__ out) {
    __shared__ Tout wtot[kWarps];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)w * (kItems * kWarp) + lane;
    Tout v[kItems];
    Tout carry = 0;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        int64_t i = base + r * kWarp;
        Tout x = (i < n) ? (Tout)in[i] : (Tout)0;
        Tout inc = warp_inclusive_sum(x, lane);
        v[r] = carry + inc - x;
        carry += __shfl_sync(kFull, inc, 31);
    }
    if (lane == 0) wtot[w] = carry;
    __syncthreads();
    Tout off = prefix ? prefix[blockIdx.x] : (Tout)0;
    Tout total = off;
    for (int k = 0; k < kWarps; ++k) {
        Tout t = wtot[k];
        if (k < w) off += t;
        total += t;
    }
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        int64_t i = base + r * kWarp;
        if (i < n) out[i] = v[r] + off;
    }
    const int64_t tile_end = (int64_t)(blockIdx.x + 1) * kTile;
    if (threadIdx.x == 0 && tile_end >= n) out[n] = total;
}

// Look-back status of a tile: 2 flag bits over a 62-bit sum.
constexpr unsigned long long kTileAgg = 1ull << 62;   // the tile's own total
constexpr unsigned long long kTilePre = 2ull << 62;   // the total of this and all earlier tiles
constexpr unsigned long long kTileVal = (1ull << 62) - 1ull;
constexpr int kScanSpinLimit = 1 << 22;               // polls of one window before giving up

__device__ __forceinline__ void st_tile(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_tile(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Single-pass exclusive scan of u32 counts into i64 offsets (out has n + 1 slots).  status holds
// one word per tile and tile_ctr one counter, all zero at launch.  A look-back window that stays
// unpublished for kScanSpinLimit polls records kDevTimeout in *d_err and the walk goes on, so
// the kernel always ends.
__global__ void __launch_bounds__(kThreads) k_scan_lookback(const uint32_t* __restrict__ in, int64_t n,
                                                            int64_t* __restrict__ out,
                                                            unsigned long long* __restrict__ status,
                                                            unsigned int* __restrict__ tile_ctr,
                                                            int* __restrict__ d_err) {
    __shared__ int64_t wtot[kWarps];
    __shared__ int64_t s_prefix;
    __shared__ unsigned int s_t;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_t = atomicAdd(tile_ctr, 1u);  // tiles in start order: earlier tiles run
    __syncthreads();
    const int64_t t = s_t;
    const int64_t base = t * kTile + (int64_t)w * (kItems * kWarp) + lane;
    int64_t v[kItems];
    int64_t carry = 0;
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + r * kWarp;
        const int64_t x = (i < n) ? (int64_t)in[i] : 0;
        const int64_t inc = warp_inclusive_sum(x, lane);
        v[r] = carry + inc - x;
        carry += __shfl_sync(kFull, inc, 31);
    }
    if (lane == 0) wtot[w] = carry;
    __syncthreads();
    int64_t total = 0;
#pragma unroll
    for (int k = 0; k < kWarps; ++k) total += wtot[k];
    if (w == 0) {
        if (lane == 0) st_tile(status + t, (t == 0 ? kTilePre : kTileAgg) | (unsigned long long)total);
        int64_t excl = 0;
        if (t > 0) {
            // earlier tiles, 32 at a time: lane l holds tile top - l; the nearest published
            // inclusive prefix ends the walk, the totals of the tiles after it are added
            int64_t top = t - 1;
            int spins = 0;
            while (true) {
                const int64_t p = top - lane;
                const unsigned long long s = p >= 0 ? ld_tile(status + p) : kTilePre;
                const unsigned long long f = s & ~kTileVal;
                if (__any_sync(kFull, f == 0ull)) {
                    if (++spins > kScanSpinLimit) {
                        if (lane == 0) atomicCAS(d_err, kDevOk, kDevTimeout);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                spins = 0;
                const unsigned pm = __ballot_sync(kFull, f == kTilePre);
                const int first = pm ? __ffs(pm) - 1 : 32;
                int64_t x = lane <= first ? (int64_t)(s & kTileVal) : 0;
#pragma unroll
                for (int d = 16; d > 0; d >>= 1) x += __shfl_xor_sync(kFull, x, d);
                excl += x;
                if (pm) break;
                top -= 32;
            }
            if (lane == 0) st_tile(status + t, kTilePre | (unsigned long long)(excl + total));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();
    int64_t off = s_prefix;
    for (int k = 0; k < w; ++k) off += wtot[k];
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + r * kWarp;
        if (i < n) out[i] = v[r] + off;
    }
    if (threadIdx.x == 0 && (t + 1) * kTile >= n) out[n] = s_prefix + total;
}

template <typename Tin, typename Tout>
cudaError_t scan_impl(const Tin* in, Tout* out, int64_t n, char* temp, cudaStream_t st) {
    if (n <= 0) {
        return cudaMemsetAsync(out, 0, sizeof(Tout), st);
    }
    const int64_t tiles = ceil_div(n, kTile);
    if (tiles == 1) {
        k_tile_scan<Tin, Tout><<<1, kThreads, 0, st>>>(in, n, (const Tout*)nullptr, out);
        note_launch();
        return cudaGetLastError();
    }
    Tout* totals = reinterpret_cast<Tout*>(temp);
    Tout* tprefix = totals + round_up(tiles, 64);
    char* next = reinterpret_cast<char*>(tprefix + round_up(tiles + 1, 64));
    k_tile_totals<Tin, Tout><<<(unsigned)tiles, kThreads, 0, st>>>(in, n, totals);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = scan_impl<Tout, Tout>(totals, tprefix, tiles, next, st);
    if (e != cudaSuccess) return e;
    k_tile_scan<Tin, Tout><<<(unsigned)tiles, kThreads, 0, st>>>(in, n, tprefix, out);
    note_launch();
    return cudaGetLastError();
}

template <typename Tout>
size_t scan_temp_impl(int64_t n) {
    size_t bytes = 0;
    int64_t m = n;
    while (m > kTile) {
        int64_t tiles = ceil_div(m, kTile);
        bytes += sizeof(Tout) * (size_t)(round_up(tiles, 64) + round_up(tiles + 1, 64));
        m = tiles;
    }
    // the single-pass form: one status word per tile and the tile counter
    const size_t one = sizeof(unsigned long long) * (size_t)round_up(ceil_div(n > 0 ? n : 1, kTile), 64) + 256;
    return std::max(bytes, one) + 256;
}

cudaError_t scan_lookback(const uint32_t* in, int64_t* out, int64_t n, char* temp, int* d_err, cudaStream_t st) {
    const int64_t tiles = ceil_div(n, kTile);
    unsigned long long* status = reinterpret_cast<unsigned long long*>(temp);
    const size_t sb = sizeof(unsigned long long) * (size_t)round_up(tiles, 64);
    unsigned int* ctr = reinterpret_cast<unsigned int*>(temp + sb);
    cudaError_t e = cudaMemsetAsync(temp, 0, sb + 256, st);
    if (e != cudaSuccess) return e;
    k_scan_lookback<<<(unsigned)tiles, kThreads, 0, st>>>(in, n, out, status, ctr, d_err);
    note_launch();
    return cudaGetLastError();
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
    return scan_temp_impl<int64_t>(n);   // the widest accumulator bounds both variants
}

cudaError_t exclusive_scan_u32_to_i64(const uint32_t* in, int64_t* out, int64_t n, void* temp,
                                      cudaStream_t st, int* d_err) {
    if (d_err && n > 0) return scan_lookback(in, out, n, static_cast<char*>(temp), d_err, st);
    return scan_impl<uint32_t, int64_t>(in, out, n, static_cast<char*>(temp), st);
}

cudaError_t exclusive_scan_u32_to_u32(const uint32_t* in, uint32_t* out, int64_t n, void* temp,
                                      cudaStream_t st) {
    return scan_impl<uint32_t, uint32_t>(in, out, n, static_cast<char*>(temp), st);
}

cudaError_t exclusive_scan_i32_to_u64(const int32_t* in, uint64_t* out, int64_t n, void* temp, cudaStream_t st) {
    return scan_impl<int32_t, uint64_t>(in, out, n, static_cast<char*>(temp), st);
}

cudaError_t exclusive_scan_i64_to_u64(const int64_t* in, uint64_t* out, int64_t n, void* temp, cudaStream_t st) {
    return scan_impl<int64_t, uint64_t>(in, out, n, static_cast<char*>(temp), st);
}

}  // namespace sig
