// si_sort.cu -- stable LSD radix sort of (K x 32-bit key words, 32-bit payload).
//
// Replaces the reference's comparison sort in build(): sort_intervals /
// sort_block (src/superintervals.hpp:1396-1439, std::sort with the comparator
// start asc / end desc at 1418) and sortIntervals (src/c_superintervals.h:440-485,
// qsort).  The key encodes (contig, start asc, end desc), see si_build.cu.
// Unlike std::sort this sort is stable, so exact (start, end) duplicates keep
// their insertion order.
//
// One pass = 8-bit digit.  Per pass: tile histogram -> exclusive scan of the
// digit-major (digit, tile) counts -> scatter.  The scatter ranks every item
// inside its 4096-item tile with warp match/ballot (stable: warp-round order
// equals input order), stages the tile in shared memory in digit order and
// writes each digit's run with consecutive addresses.  A pass whose digit is
// the same for every record is skipped (one global histogram over all digit
// positions decides this up front).
#include <algorithm>
#include "si_internal.cuh"

namespace sig {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096
constexpr int kWarps = kThreads / kWarp;
constexpr int kRadix = 256;

struct KeyPtrs {
    const uint32_t* w[kMaxKeyWords];
};
struct KeyOutPtrs {
    uint32_t* w[kMaxKeyWords];
};

__global__ void __launch_bounds__(kThreads) k_global_hist(KeyPtrs keys, int K, int64_t n,
                                                          uint32_t* __restrict__ ghist) {
    __shared__ uint32_t h[kMaxKeyWords * 4 * kRadix];
    for (int i = threadIdx.x; i < K * 4 * kRadix; i += kThreads) h[i] = 0;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * kThreads;
    for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < n; i += stride) {
        for (int w = 0; w < K; ++w) {
            uint32_t v = keys.w[w][i];
#pragma unroll
            for (int b = 0; b < 4; ++b) atomicAdd(&h[(w * 4 + b) * kRadix + ((v >> (8 * b)) & 255u)], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < K * 4 * kRadix; i += kThreads) {
        if (h[i]) atomicAdd(&ghist[i], h[i]);
    }
}

__global__ void __launch_bounds__(kThreads) k_pass_hist(const uint32_t* __restrict__ kw, int sh,
                                                        int64_t n, uint32_t* __restrict__ H,
                                                        int64_t tiles) {
    __shared__ uint32_t h[kRadix];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll 4
    for (int k = 0; k < kItems; ++k) {
        int64_t i = base + k * kThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(kw[i] >> sh) & 255u], 1u);
    }
    __syncthreads();
    H[(int64_t)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads) k_pass_scatter(KeyPtrs kin, KeyOutPtrs kout, int K,
                                                           const uint32_t* __restrict__ pin,
                                                           uint32_t* __restrict__ pout, int dw,
                                                           int sh, int64_t n,
                                                           const uint32_t* __restrict__ O,
                                                           int64_t tiles) {
    __shared__ uint32_t wcnt[kWarps][kRadix + 1];
    __shared__ uint32_t tdo[kRadix];
    __shared__ int32_t go[kRadix];
    __shared__ uint32_t wsum[kWarps];
    __shared__ uint32_t stage[kTile];
    __shared__ uint8_t sd[kTile];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int i = tid; i < kWarps * (kRadix + 1); i += kThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();

    const int64_t t = blockIdx.x;
    const int64_t base = t * kTile + (int64_t)w * (kItems * kWarp) + lane;
    const uint32_t* dword = kin.w[dw];
    uint32_t dg[kItems];
    uint32_t lp[kItems];
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + r * kWarp;
        const uint32_t d = (i < n) ? ((dword[i] >> sh) & 255u) : (uint32_t)kRadix;
        const uint32_t peers = __match_any_sync(kFull, d);
        const uint32_t rank = __popc(peers & lanemask_lt());
        const uint32_t b = wcnt[w][d];
        __syncwarp();
        if (rank == 0) wcnt[w][d] = b + __popc(peers);
        __syncwarp();
        dg[r] = d;
        lp[r] = b + rank;
    }
    __syncthreads();

    // per digit: exclusive prefix over warps, tile total
    uint32_t cnt = 0;
    {
        const int d = tid;  // kThreads == kRadix
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kWarps; ++ww) {
            uint32_t c = wcnt[ww][d];
            wcnt[ww][d] = run;
            run += c;
        }
        cnt = run;
    }
    // block exclusive scan of cnt over digits
    uint32_t inc = cnt;
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, inc, dd);
        if (lane >= dd) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    uint32_t woff = 0;
    for (int ww = 0; ww < w; ++ww) woff += wsum[ww];
    const uint32_t excl = woff + inc - cnt;
    tdo[tid] = excl;
    go[tid] = (int32_t)O[(int64_t)tid * tiles + t] - (int32_t)excl;
    __syncthreads();

#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        if (dg[r] < (uint32_t)kRadix) {
            lp[r] = tdo[dg[r]] + wcnt[w][dg[r]] + lp[r];
            sd[lp[r]] = (uint8_t)dg[r];
        }
    }
    const int tile_n = (int)((n - t * kTile) < kTile ? (n - t * kTile) : kTile);
    for (int a = 0; a <= K; ++a) {
        const uint32_t* src = (a < K) ? kin.w[a] : pin;
        uint32_t* dst = (a < K) ? kout.w[a] : pout;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < kItems; ++r) {
            if (dg[r] < (uint32_t)kRadix) stage[lp[r]] = src[base + r * kWarp];
        }
        __syncthreads();
        for (int j = tid; j < tile_n; j += kThreads) {
            dst[(int64_t)go[sd[j]] + j] = stage[j];
        }
    }
}

}  // namespace

size_t radix_temp_bytes(int64_t n, int K) {
    const int64_t tiles = ceil_div(n > 0 ? n : 1, kTile);
    size_t b = sizeof(uint32_t) * (size_t)round_up(K * 4 * kRadix, 64);      // ghist
    b += sizeof(uint32_t) * (size_t)round_up(kRadix * tiles, 64);             // H
    b += sizeof(uint32_t) * (size_t)round_up(kRadix * tiles + 1, 64);         // O
    b += scan_temp_bytes(kRadix * tiles);
    return b + 1024;
}

cudaError_t radix_sort(uint32_t* const* keys, uint32_t* const* alt_keys, uint32_t* payload,
                       uint32_t* alt_payload, int K, int64_t n, void* temp, size_t temp_bytes,
                       bool* result_in_alt, int* passes_run, cudaStream_t st, uint32_t pass_mask) {
    *result_in_alt = false;
    if (passes_run) *passes_run = 0;
    if (n <= 1) return cudaSuccess;
    if (K < 1 || K > kMaxKeyWords) return cudaErrorInvalidValue;
    if (n >= (int64_t)INT32_MAX) return cudaErrorInvalidValue;
    if (temp_bytes < radix_temp_bytes(n, K)) return cudaErrorInvalidValue;
    const int64_t tiles = ceil_div(n, kTile);
    char* p = static_cast<char*>(temp);
    uint32_t* ghist = reinterpret_cast<uint32_t*>(p);
    p += sizeof(uint32_t) * round_up(K * 4 * kRadix, 64);
    uint32_t* H = reinterpret_cast<uint32_t*>(p);
    p += sizeof(uint32_t) * round_up(kRadix * tiles, 64);
    uint32_t* O = reinterpret_cast<uint32_t*>(p);
    p += sizeof(uint32_t) * round_up(kRadix * tiles + 1, 64);
    void* scan_tmp = p;

    cudaError_t e = cudaSuccess;
    uint32_t hh[kMaxKeyWords * 4 * kRadix];
    if (!pass_mask) {
        e = cudaMemsetAsync(ghist, 0, sizeof(uint32_t) * K * 4 * kRadix, st);
        if (e != cudaSuccess) return e;
        KeyPtrs kp{};
        for (int w = 0; w < K; ++w) kp.w[w] = keys[w];
        int gblocks = (int)std::min<int64_t>(ceil_div(n, kThreads), 152 * 8);
        k_global_hist<<<gblocks, kThreads, 0, st>>>(kp, K, n, ghist);
        note_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        e = cudaMemcpyAsync(hh, ghist, sizeof(uint32_t) * K * 4 * kRadix, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
    }

    uint32_t* cur_k[kMaxKeyWords];
    uint32_t* oth_k[kMaxKeyWords];
    for (int w = 0; w < K; ++w) {
        cur_k[w] = keys[w];
        oth_k[w] = alt_keys[w];
    }
    uint32_t* cur_p = payload;
    uint32_t* oth_p = alt_payload;
    bool in_alt = false;
    int passes = 0;
    for (int w = 0; w < K; ++w) {
        for (int b = 0; b < 4; ++b) {
            if (pass_mask) {
                if (!((pass_mask >> (w * 4 + b)) & 1u)) continue;
            } else {
                const uint32_t* hb = hh + (w * 4 + b) * kRadix;
                bool constant = false;
                for (int d = 0; d < kRadix; ++d)
                    if (hb[d] == (uint32_t)n) constant = true;
                if (constant) continue;
            }
            k_pass_hist<<<(unsigned)tiles, kThreads, 0, st>>>(cur_k[w], 8 * b, n, H, tiles);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            e = exclusive_scan_u32_to_u32(H, O, kRadix * tiles, scan_tmp, st);
            if (e != cudaSuccess) return e;
            KeyPtrs in{};
            KeyOutPtrs out{};
            for (int ww = 0; ww < K; ++ww) {
                in.w[ww] = cur_k[ww];
                out.w[ww] = oth_k[ww];
            }
            k_pass_scatter<<<(unsigned)tiles, kThreads, 0, st>>>(in, out, K, cur_p, oth_p, w, 8 * b,
                                                                 n, O, tiles);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            for (int ww = 0; ww < K; ++ww) {
                uint32_t* tmp = cur_k[ww];
                cur_k[ww] = oth_k[ww];
                oth_k[ww] = tmp;
            }
            uint32_t* tp = cur_p;
            cur_p = oth_p;
            oth_p = tp;
            in_alt = !in_alt;
            ++passes;
        }
    }
    *result_in_alt = in_alt;
    if (passes_run) *passes_run = passes;
    return cudaSuccess;
}

}  // namespace sig
