// si_scan.cu -- device-wide exclusive prefix sum (reduce-then-scan).
//
// Used for the per-query result offsets (count -> exclusive scan -> emit, the
// CSR form of the per-query result lists of src/superintervals/intervalmap.pyx:402-494)
// and for the digit offsets of the radix sort.  HBM-bound: one read for the
// tile totals, one read + one write for the scan itself.
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
    return bytes + 256;
}

}  // namespace

size_t scan_temp_bytes(int64_t n) {
    return scan_temp_impl<int64_t>(n);   // the widest accumulator bounds both variants
}

cudaError_t exclusive_scan_u32_to_i64(const uint32_t* in, int64_t* out, int64_t n, void* temp,
                                      cudaStream_t st) {
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
