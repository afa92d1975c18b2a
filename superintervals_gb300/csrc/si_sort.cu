// si_sort.cu -- stable LSD radix sort of (K x 32-bit key words, 32-bit payload).
//
// Replaces the reference's comparison sort in build(): sort_intervals /
// sort_block (src/superintervals.hpp:1396-1439, std::sort with the comparator
// start asc / end desc at 1418) and sortIntervals (src/c_superintervals.h:440-485,
// qsort).  The key encodes (contig, start asc, end desc), see si_build.cu.
// Unlike std::sort this sort is stable, so exact (start, end) duplicates keep
// their insertion order.
//
// One pass = 8-bit digit.  One histogram kernel counts every digit position up
// front; a pass whose digit is the same for every record is skipped.  Each pass
// is then ONE kernel (one-sweep): a block takes the next 4096-item tile from an
// atomic counter, ranks every item inside its tile with warp match/ballot
// (stable: warp-round order equals input order), publishes its per-digit counts
// and finds, per digit, the count of the same digit in all earlier tiles by
// decoupled look-back over the tiles' published counts (an inclusive prefix
// ends the walk); it then stages the tile in shared memory in digit order and
// writes each digit's run with consecutive addresses.  Without an error word
// from the caller the sort takes the three-kernel form per pass (tile
// histogram -> exclusive scan of the digit-major counts -> scatter).
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

// Exclusive prefix over the 256 digits of each pass's global histogram: where each digit's
// run starts in the sorted output.  One block of 256 threads per digit position.
__global__ void __launch_bounds__(kRadix) k_digit_offsets(const uint32_t* __restrict__ ghist,
                                                         uint32_t* __restrict__ goff) {
    __shared__ uint32_t wsum[kRadix / kWarp];
    const int d = threadIdx.x, lane = d & 31, w = d >> 5;
    const uint32_t c = ghist[blockIdx.x * kRadix + d];
    uint32_t inc = c;
#pragma unroll
    for (int k = 1; k < 32; k <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, inc, k);
        if (lane >= k) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    uint32_t off = 0;
    for (int k = 0; k < w; ++k) off += wsum[k];
    goff[blockIdx.x * kRadix + d] = off + inc - c;
}

// Look-back status word per (tile, digit): 2 flag bits over a 30-bit count.
constexpr uint32_t kStAgg = 1u << 30;     // the tile's own count of the digit
constexpr uint32_t kStPre = 2u << 30;     // the count of the digit in this and all earlier tiles
constexpr uint32_t kStVal = (1u << 30) - 1u;
constexpr int kSpinLimit = 1 << 22;       // polls of one status word before giving up
constexpr int kLookWindow = 8;            // earlier tiles read per look-back step

__device__ __forceinline__ void st_status(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_status(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// One radix pass in one kernel (see the file comment).  status holds tiles x 256 words and
// tile_ctr one counter, both zero at launch.  A look-back that polls one word kSpinLimit
// times (which needs an earlier tile that never publishes) records kDevTimeout in *d_err and
// goes on, so the kernel always ends.
__global__ void __launch_bounds__(kThreads, 3) k_onesweep(KeyPtrs kin, KeyOutPtrs kout, int K,
                                                       const uint32_t* __restrict__ pin,
                                                       uint32_t* __restrict__ pout, int dw, int sh,
                                                       int64_t n, const uint32_t* __restrict__ goff,
                                                       uint32_t* __restrict__ status,
                                                       unsigned int* __restrict__ tile_ctr,
                                                       int* __restrict__ d_err) {
    __shared__ uint32_t wcnt[kWarps][kRadix + 1];
    __shared__ uint32_t tdo[kRadix];
    __shared__ int32_t go[kRadix];
    __shared__ uint32_t wsum[kWarps];
    __shared__ uint32_t stage[kTile];
    __shared__ uint8_t sd[kTile];
    __shared__ unsigned int s_t;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) s_t = atomicAdd(tile_ctr, 1u);  // tiles in start order: earlier tiles run
    for (int i = tid; i < kWarps * (kRadix + 1); i += kThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();

    const int64_t t = s_t;
    const int64_t base = t * kTile + (int64_t)w * (kItems * kWarp) + lane;
    const uint32_t* dword = kin.w[dw];
    uint32_t lp[kItems];
    uint32_t key[kItems];  // the digit word of every item, loaded before any ranking step waits
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + r * kWarp;
        key[r] = (i < n) ? dword[i] : 0u;
    }
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        const int64_t i = base + r * kWarp;
        const uint32_t d = (i < n) ? ((key[r] >> sh) & 255u) : (uint32_t)kRadix;
        const uint32_t peers = __match_any_sync(kFull, d);
        const uint32_t rank = __popc(peers & lanemask_lt());
        const uint32_t b = wcnt[w][d];
        __syncwarp();
        if (rank == 0) wcnt[w][d] = b + __popc(peers);
        __syncwarp();
        lp[r] = b + rank;
    }
    __syncthreads();

    // per digit (thread = digit): exclusive prefix over warps and the tile's count
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
    uint32_t* my = status + t * kRadix + tid;
    st_status(my, (t == 0 ? kStPre : kStAgg) | cnt);  // published before anything waits
    // block exclusive scan of cnt over digits: where each digit's run starts in the tile
    uint32_t inc = cnt;
#pragma unroll
    for (int dd = 1; dd < 32; dd <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, inc, dd);
        if (lane >= dd) inc += y;
    }
    if (lane == 31) wsum[w] = inc;
    // decoupled look-back: the digit's count in all earlier tiles, kLookWindow tiles per step
    // (independent reads, so that a chain of tiles that have published only their own counts
    // costs one memory round trip per window instead of one per tile)
    uint32_t pre = 0;
    if (t > 0) {
        int64_t p = t - 1;
        int spins = 0;
        while (true) {
            uint32_t v[kLookWindow];
#pragma unroll
            for (int k = 0; k < kLookWindow; ++k)
                v[k] = p - k >= 0 ? ld_status(status + (p - k) * kRadix + tid) : kStPre;  // before tile 0: none
            int used = kLookWindow;  // window entries consumed
            bool done = false, wait = false;
#pragma unroll
            for (int k = 0; k < kLookWindow; ++k) {
                if (!done && !wait) {
                    const uint32_t f = v[k] & ~kStVal;
                    if (f == 0u) {
                        wait = true;  // tile p - k has published nothing yet
                        used = k;
                    } else {
                        pre += v[k] & kStVal;
                        if (f == kStPre) {
                            done = true;
                            used = k + 1;
                        }
                    }
                }
            }
            if (done) break;
            p -= used;
            if (wait) {
                if (++spins > kSpinLimit) {
                    atomicCAS(d_err, kDevOk, kDevTimeout);
                    break;
                }
                __nanosleep(32);
            } else {
                spins = 0;
            }
        }
        st_status(my, kStPre | ((pre + cnt) & kStVal));
    }
    __syncthreads();
    uint32_t woff = 0;
    for (int ww = 0; ww < w; ++ww) woff += wsum[ww];
    const uint32_t excl = woff + inc - cnt;
    tdo[tid] = excl;
    go[tid] = (int32_t)(goff[tid] + pre) - (int32_t)excl;
    __syncthreads();

    const int64_t n_here = n - base;  // items of this thread with r * kWarp < n_here are valid
#pragma unroll
    for (int r = 0; r < kItems; ++r) {
        if (r * kWarp < n_here) {
            const uint32_t dr = (key[r] >> sh) & 255u;
            lp[r] = tdo[dr] + wcnt[w][dr] + lp[r];
            sd[lp[r]] = (uint8_t)dr;
        }
    }
    const int tile_n = (int)((n - t * kTile) < kTile ? (n - t * kTile) : kTile);
    for (int a = 0; a <= K; ++a) {
        const uint32_t* src = (a < K) ? kin.w[a] : pin;
        uint32_t* dst = (a < K) ? kout.w[a] : pout;
        __syncthreads();
        if (a == dw) {  // the digit word is already in registers
#pragma unroll
            for (int r = 0; r < kItems; ++r)
                if (r * kWarp < n_here) stage[lp[r]] = key[r];
        } else {
            uint32_t v[kItems];
#pragma unroll
            for (int r = 0; r < kItems; ++r) {
                const int64_t i = base + r * kWarp;
                v[r] = (i < n) ? src[i] : 0u;
            }
#pragma unroll
            for (int r = 0; r < kItems; ++r)
                if (r * kWarp < n_here) stage[lp[r]] = v[r];
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
    // three-kernel passes: tile histograms H and their scan O
    size_t three = sizeof(uint32_t) * (size_t)round_up(kRadix * tiles, 64);  // H
    three += sizeof(uint32_t) * (size_t)round_up(kRadix * tiles + 1, 64);    // O
    three += scan_temp_bytes(kRadix * tiles);
    // one-sweep passes: digit offsets of every pass, look-back status, tile counter
    size_t one = sizeof(uint32_t) * (size_t)round_up(K * 4 * kRadix, 64);    // goff
    one += sizeof(uint32_t) * (size_t)round_up(kRadix * tiles, 64);          // status
    one += 256;                                                              // counter
    return b + std::max(three, one) + 1024;
}

uint32_t* radix_hist(void* temp) { return static_cast<uint32_t*>(temp); }

cudaError_t radix_sort(uint32_t* const* keys, uint32_t* const* alt_keys, uint32_t* payload,
                       uint32_t* alt_payload, int K, int64_t n, void* temp, size_t temp_bytes,
                       bool* result_in_alt, int* passes_run, cudaStream_t st, uint32_t pass_mask,
                       int* d_err, bool hist_ready) {
    *result_in_alt = false;
    if (passes_run) *passes_run = 0;
    if (n <= 1) return cudaSuccess;
    if (K < 1 || K > kMaxKeyWords) return cudaErrorInvalidValue;
    if (n >= (int64_t)INT32_MAX) return cudaErrorInvalidValue;
    if (temp_bytes < radix_temp_bytes(n, K)) return cudaErrorInvalidValue;
    const int64_t tiles = ceil_div(n, kTile);
    // the one-sweep form needs an error word for its bounded waits and counts below 2^30
    const bool one = d_err != nullptr && n < (int64_t)kStVal;
    char* p = static_cast<char*>(temp);
    uint32_t* ghist = reinterpret_cast<uint32_t*>(p);
    p += sizeof(uint32_t) * round_up(K * 4 * kRadix, 64);
    uint32_t* H = reinterpret_cast<uint32_t*>(p);     // three-kernel form
    uint32_t* goff = H;                                // one-sweep form (same space)
    p += sizeof(uint32_t) * round_up(kRadix * tiles, 64);
    uint32_t* O = reinterpret_cast<uint32_t*>(p);
    p += sizeof(uint32_t) * round_up(kRadix * tiles + 1, 64);
    void* scan_tmp = p;
    char* q1 = reinterpret_cast<char*>(goff) + sizeof(uint32_t) * round_up(K * 4 * kRadix, 64);
    uint32_t* status = reinterpret_cast<uint32_t*>(q1);
    unsigned int* tile_ctr = reinterpret_cast<unsigned int*>(q1 + sizeof(uint32_t) * round_up(kRadix * tiles, 64));
    const size_t status_bytes = sizeof(uint32_t) * (size_t)round_up(kRadix * tiles, 64) + 256;

    cudaError_t e = cudaSuccess;
    uint32_t hh[kMaxKeyWords * 4 * kRadix];
    if (!pass_mask || one) {
        if (!hist_ready) {
            e = cudaMemsetAsync(ghist, 0, sizeof(uint32_t) * K * 4 * kRadix, st);
            if (e != cudaSuccess) return e;
            KeyPtrs kp{};
            for (int w = 0; w < K; ++w) kp.w[w] = keys[w];
            int gblocks = (int)std::min<int64_t>(ceil_div(n, kThreads), 152 * 8);
            k_global_hist<<<gblocks, kThreads, 0, st>>>(kp, K, n, ghist);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (one) {
            k_digit_offsets<<<K * 4, kRadix, 0, st>>>(ghist, goff);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (!pass_mask) {
            e = cudaMemcpyAsync(hh, ghist, sizeof(uint32_t) * K * 4 * kRadix, cudaMemcpyDeviceToHost, st);
            if (e != cudaSuccess) return e;
            if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        }
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
            KeyPtrs in{};
            KeyOutPtrs out{};
            for (int ww = 0; ww < K; ++ww) {
                in.w[ww] = cur_k[ww];
                out.w[ww] = oth_k[ww];
            }
            if (one) {
                e = cudaMemsetAsync(status, 0, status_bytes, st);
                if (e != cudaSuccess) return e;
                k_onesweep<<<(unsigned)tiles, kThreads, 0, st>>>(in, out, K, cur_p, oth_p, w, 8 * b, n,
                                                                 goff + (w * 4 + b) * kRadix, status, tile_ctr,
                                                                 d_err);
                note_launch();
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
            } else {
                k_pass_hist<<<(unsigned)tiles, kThreads, 0, st>>>(cur_k[w], 8 * b, n, H, tiles);
                note_launch();
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
                e = exclusive_scan_u32_to_u32(H, O, kRadix * tiles, scan_tmp, st);
                if (e != cudaSuccess) return e;
                k_pass_scatter<<<(unsigned)tiles, kThreads, 0, st>>>(in, out, K, cur_p, oth_p, w, 8 * b,
                                                                     n, O, tiles);
                note_launch();
                if ((e = cudaGetLastError()) != cudaSuccess) return e;
            }
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
