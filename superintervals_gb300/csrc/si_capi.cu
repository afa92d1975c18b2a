// si_capi.cu -- host runtime behind include/si_gpu/c_api.h.
//
// Owns the device index of a handle, its CUDA stream and a grow-only query
// workspace, drives build() and the count -> scan -> emit query pipeline, and
// chunks large result sets against a device output budget.  All device memory
// goes through one allocator that honours a process-wide byte budget, so an
// oversize request fails with SI_ERR_OOM instead of faulting.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "si_gpu/c_api.h"
#include "si_internal.cuh"
#include "si_batched.cuh"

namespace {

thread_local std::string g_err;
std::atomic<size_t> g_used{0};
// bumped by every device allocation and release of the library: a captured graph whose
// buffers may have moved is captured again
std::atomic<unsigned long long> g_alloc_gen{0};
std::atomic<size_t> g_budget{0};

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define SI_CK(call)                                                                          \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(SI_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
    } while (0)

#define SI_TRY(call)                  \
    do {                              \
        int r_ = (call);              \
        if (r_ != SI_OK) return r_;   \
    } while (0)

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) {
            cudaFree(p);
            g_used -= bytes;
            ++g_alloc_gen;
        }
        p = nullptr;
        bytes = 0;
    }
    // Grow-only: keeps the buffer when it is already large enough.
    int reserve(size_t b) {
        if (b <= bytes && p) return SI_OK;
        release();
        if (b == 0) b = 256;
        b = (b + 255) & ~(size_t)255;
        const size_t cap = g_budget.load();
        if (cap && g_used.load() + b > cap)
            return fail(SI_ERR_OOM, "device budget exceeded: %zu in use + %zu requested > %zu", g_used.load(),
                        b, cap);
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            return fail(SI_ERR_OOM, "cudaMalloc(%zu) failed: %s", b, cudaGetErrorString(e));
        }
        bytes = b;
        g_used += b;
        ++g_alloc_gen;
        return SI_OK;
    }
    template <typename T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

}  // namespace

namespace sig {
int dev_reserve(void** p, size_t* bytes, size_t need) {
    if (*p && need <= *bytes) return SI_OK;
    dev_release(p, bytes);
    if (need == 0) need = 256;
    need = (need + 255) & ~(size_t)255;
    const size_t cap = g_budget.load();
    if (cap && g_used.load() + need > cap)
        return fail(SI_ERR_OOM, "device budget exceeded: %zu in use + %zu requested > %zu", g_used.load(), need, cap);
    cudaError_t e = cudaMalloc(p, need);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(SI_ERR_OOM, "cudaMalloc(%zu) failed: %s", need, cudaGetErrorString(e));
    }
    *bytes = need;
    g_used += need;
    ++g_alloc_gen;
    return SI_OK;
}
void dev_release(void** p, size_t* bytes) {
    if (*p) {
        cudaFree(*p);
        g_used -= *bytes;
        ++g_alloc_gen;
    }
    *p = nullptr;
    *bytes = 0;
}
}  // namespace sig

struct gSuperIntervals {
    int bits = 32;
    int device = 0;
    cudaStream_t st = nullptr;
    // host staging in insertion order
    std::vector<int32_t> hs32, he32;
    std::vector<int64_t> hs64, he64;
    std::vector<int32_t> hdata;
    std::vector<int64_t> hseg;  // empty: one contig
    bool built = false;
    // device index
    int64_t n = 0, n_pad = 0;
    int G = 1, H = 0;
    int64_t lvl_sizes[sig::kMaxLevels + 1] = {0};
    DevBuf starts, ends, data, branch, seg, perm;
    DevBuf lvl[sig::kMaxLevels];
    // long-interval list: intervals >= kLongIntervalSplit long, position order, own pyramid
    DevBuf long_pos, long_end, long_seg;
    DevBuf end_sorted;  // each contig's ends ascending (built when no interval has start > end)
    // exclusive prefix sums (mod 2^64) of the starts and of the sorted ends, for coverage from
    // ranks; built by the first such call after a build
    DevBuf ps_start, ps_end;
    bool cov_ready = false;
    DevBuf rec;             // the intervals as (start, end, payload) records, made on first use
    bool rec_ready = false;
    DevBuf long_lvl[sig::kMaxLevels];
    int64_t long_sizes[sig::kMaxLevels + 1] = {0};
    int long_H = 0;
    int sort_passes = 0;
    bool input_was_sorted = false;
    // query workspace
    DevBuf wq_s, wq_e, wq_c, w_counts, w_offsets, w_out, w_tmp, w_err;
    // host-buffer searches of several chunks: a second result buffer and a copy stream, so
    // that the emit of one chunk overlaps the device-to-host copy of the previous one
    DevBuf w_out2;
    cudaStream_t copy_st = nullptr;
    cudaEvent_t ev_emitted[2] = {nullptr, nullptr}, ev_copied[2] = {nullptr, nullptr};
    sig::BatchedWorkspace bws;
    // set operations: hit lists, staged pieces, and whether some interval has start > end
    DevBuf so_hoff, so_hits, so_off, so_os, so_oe, so_ob, so_flag;
    int inverted = -1;  // -1 unknown, else 0 / 1 (reset by every build)
    // mean number of intervals at least 32768 long over a position (set by every build): hits
    // of such intervals lie far apart in position order, so one walk per query is long
    double long_depth = 0.0;
    // contig names, in contig-id order, when the intervals came from BED text
    std::vector<std::string> contig_names;
    // options
    int path = SI_PATH_AUTO;
    int ub_mode = SI_UB_BINARY;
    size_t out_budget = (size_t)4 << 30;
    // captured count -> scan -> emit graph and the call it was captured for
    cudaGraphExec_t gexec = nullptr;
    const void* gkey[8] = {nullptr};
    size_t gkey_n[5] = {0, 0, 0, 0, 0};
    long long g_kernels = 0;  // kernels inside the captured graph
    // phase profiling (count, scan, emit, prepare)
    bool prof = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double phase_ms[4] = {0, 0, 0, 0};
    int64_t phase_n[4] = {0, 0, 0, 0};
};

namespace {

size_t staged(const gSuperIntervals* si) { return si->hdata.size(); }

// Brackets one pipeline phase with CUDA events when profiling is on.
struct PhaseTimer {
    gSuperIntervals* si;
    int phase;
    cudaStream_t st;
    PhaseTimer(gSuperIntervals* s, int p, cudaStream_t t) : si(s), phase(p), st(t) {
        if (si->prof) cudaEventRecord(si->ev0, st);
    }
    ~PhaseTimer() {
        if (!si->prof) return;
        cudaEventRecord(si->ev1, st);
        if (cudaEventSynchronize(si->ev1) == cudaSuccess) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, si->ev0, si->ev1) == cudaSuccess) {
                si->phase_ms[phase] += ms;
                si->phase_n[phase] += 1;
            }
        }
    }
};

int set_dev(const gSuperIntervals* si) {
    SI_CK(cudaSetDevice(si->device));
    return SI_OK;
}

template <typename S>
std::vector<S>& hs(gSuperIntervals* si);
template <>
std::vector<int32_t>& hs<int32_t>(gSuperIntervals* si) { return si->hs32; }
template <>
std::vector<int64_t>& hs<int64_t>(gSuperIntervals* si) { return si->hs64; }
template <typename S>
std::vector<S>& he(gSuperIntervals* si);
template <>
std::vector<int32_t>& he<int32_t>(gSuperIntervals* si) { return si->he32; }
template <>
std::vector<int64_t>& he<int64_t>(gSuperIntervals* si) { return si->he64; }

template <typename S>
int check_width(const gSuperIntervals* si) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if ((int)sizeof(S) * 8 != si->bits)
        return fail(SI_ERR_INVALID, "coordinate width %d does not match the handle (%d)",
                    (int)sizeof(S) * 8, si->bits);
    return SI_OK;
}

template <typename S>
int add_many(gSuperIntervals* si, const S* s, const S* e, const int32_t* v, size_t n) {
    SI_TRY(check_width<S>(si));
    if (n && (!s || !e)) return fail(SI_ERR_INVALID, "null interval arrays");
    const size_t base = staged(si);
    if (base + n >= (size_t)INT32_MAX - 64)
        return fail(SI_ERR_TOO_LARGE, "more than 2^31-65 intervals in one handle");
    hs<S>(si).insert(hs<S>(si).end(), s, s + n);
    he<S>(si).insert(he<S>(si).end(), e, e + n);
    if (v) {
        si->hdata.insert(si->hdata.end(), v, v + n);
    } else {
        si->hdata.resize(base + n);
        for (size_t i = 0; i < n; ++i) si->hdata[base + i] = (int32_t)(base + i);
    }
    if (!si->hseg.empty()) si->hseg.back() = (int64_t)staged(si);  // grow the last contig
    si->built = false;
    return SI_OK;
}

template <typename S>
sig::MapView<S> view(const gSuperIntervals* si) {
    sig::MapView<S> m;
    m.starts = si->starts.as<S>();
    m.ends = si->ends.as<S>();
    m.branch = si->branch.as<int32_t>();
    m.data = si->data.as<int32_t>();
    m.seg = si->seg.as<int64_t>();
    m.G = si->G;
    m.n = si->n;
    m.end_sorted = (si->inverted == 0) ? static_cast<const S*>(si->bws.end_sorted) : nullptr;
    return m;
}

// The view with the interval records, made on the first call after a build: the operations
// that read every field of each hit (set operations, keys, coverage) read one record per hit.
template <typename S>
int view_rec(gSuperIntervals* si, cudaStream_t st, sig::MapView<S>* out) {
    *out = view<S>(si);
    if (si->n <= 0) return SI_OK;
    if (!si->rec_ready) {
        SI_TRY(si->rec.reserve(sizeof(sig::IvRec<S>) * (size_t)si->n));
        SI_CK(sig::launch_records<S>(si->starts.as<S>(), si->ends.as<S>(), si->data.as<int32_t>(), si->n,
                                     si->rec.as<sig::IvRec<S>>(), st));
        si->rec_ready = true;
    }
    out->rec = si->rec.as<sig::IvRec<S>>();
    return SI_OK;
}

template <typename S>
sig::Levels<S> levels(const gSuperIntervals* si) {
    sig::Levels<S> L;
    for (int h = 0; h < sig::kMaxLevels; ++h) L.p[h] = si->lvl[h].as<S>();
    return L;
}

template <typename S>
int build_impl(gSuperIntervals* si) {
    SI_TRY(set_dev(si));
    cudaStream_t st = si->st;
    const int64_t n = (int64_t)staged(si);
    std::vector<int64_t> segv = si->hseg;
    if (segv.empty()) segv = {0, n};
    const int G = (int)segv.size() - 1;
    if (G < 1 || segv[0] != 0 || segv[G] != n)
        return fail(SI_ERR_INVALID, "contig offsets do not cover the %lld staged intervals", (long long)n);
    for (int g = 0; g < G; ++g)
        if (segv[g + 1] < segv[g]) return fail(SI_ERR_INVALID, "contig offsets decrease at %d", g);
    si->built = false;
    si->inverted = -1;
    si->bws.long_ends = nullptr;  // set again once the long-interval list exists
    si->bws.end_sorted = nullptr;
    si->cov_ready = false;
    si->rec_ready = false;
    if (si->gexec) {              // a captured graph holds the old buffers
        cudaGraphExecDestroy(si->gexec);
        si->gexec = nullptr;
    }
    si->n = n;
    si->G = G;
    si->n_pad = sig::round_up(std::max<int64_t>(n, 1), 32);
    const int64_t n_pad = si->n_pad;
    SI_TRY(si->starts.reserve(sizeof(S) * n_pad));
    SI_TRY(si->ends.reserve(sizeof(S) * n_pad));
    SI_TRY(si->data.reserve(sizeof(int32_t) * n_pad));
    SI_TRY(si->branch.reserve(sizeof(int32_t) * n_pad));
    SI_TRY(si->perm.reserve(sizeof(uint32_t) * n_pad));
    SI_TRY(si->seg.reserve(sizeof(int64_t) * (G + 1)));
    SI_CK(cudaMemcpyAsync(si->seg.p, segv.data(), sizeof(int64_t) * (G + 1), cudaMemcpyHostToDevice, st));
    si->H = sig::pyramid_levels(n_pad, si->lvl_sizes);
    for (int h = 1; h <= si->H; ++h) SI_TRY(si->lvl[h - 1].reserve(sizeof(S) * si->lvl_sizes[h]));
    if (n == 0) {
        SI_CK(cudaStreamSynchronize(st));
        si->built = true;
        return SI_OK;
    }
    DevBuf s_in, e_in, d_in, flag, berr;
    SI_TRY(berr.reserve(sizeof(int)));  // bounded waits of the one-sweep sorts and scans
    SI_CK(cudaMemsetAsync(berr.p, 0, sizeof(int), st));
    SI_TRY(s_in.reserve(sizeof(S) * n));
    SI_TRY(e_in.reserve(sizeof(S) * n));
    SI_TRY(d_in.reserve(sizeof(int32_t) * n));
    SI_TRY(flag.reserve(sizeof(int)));
    SI_CK(cudaMemcpyAsync(s_in.p, hs<S>(si).data(), sizeof(S) * n, cudaMemcpyHostToDevice, st));
    SI_CK(cudaMemcpyAsync(e_in.p, he<S>(si).data(), sizeof(S) * n, cudaMemcpyHostToDevice, st));
    SI_CK(cudaMemcpyAsync(d_in.p, si->hdata.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
    SI_CK(sig::launch_check_sorted<S>(s_in.as<S>(), e_in.as<S>(), n, si->seg.as<int64_t>(), G,
                                      flag.as<int>(), st));
    int unsorted = 0;
    SI_CK(cudaMemcpyAsync(&unsorted, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    si->input_was_sorted = !unsorted;
    si->sort_passes = 0;
    if (!unsorted) {
        SI_CK(sig::launch_copy_pad<S>(s_in.as<S>(), e_in.as<S>(), d_in.as<int32_t>(), n, n_pad,
                                      si->starts.as<S>(), si->ends.as<S>(), si->data.as<int32_t>(),
                                      si->perm.as<uint32_t>(), st));
    } else {
        const int K = sig::key_words<S>(G);
        DevBuf kw[sig::kMaxKeyWords], kalt[sig::kMaxKeyWords], pay, palt, tmp;
        uint32_t* kp[sig::kMaxKeyWords];
        uint32_t* ka[sig::kMaxKeyWords];
        for (int k = 0; k < K; ++k) {
            SI_TRY(kw[k].reserve(sizeof(uint32_t) * n));
            SI_TRY(kalt[k].reserve(sizeof(uint32_t) * n));
            kp[k] = kw[k].as<uint32_t>();
            ka[k] = kalt[k].as<uint32_t>();
        }
        SI_TRY(pay.reserve(sizeof(uint32_t) * n));
        SI_TRY(palt.reserve(sizeof(uint32_t) * n));
        const size_t tb = sig::radix_temp_bytes(n, K);
        SI_TRY(tmp.reserve(tb));
        SI_CK(sig::launch_make_keys<S>(s_in.as<S>(), e_in.as<S>(), n, si->seg.as<int64_t>(), G, kp,
                                       pay.as<uint32_t>(), st));
        bool in_alt = false;
        SI_CK(sig::radix_sort(kp, ka, pay.as<uint32_t>(), palt.as<uint32_t>(), K, n, tmp.p, tb,
                              &in_alt, &si->sort_passes, st, 0, berr.as<int>()));
        uint32_t* const* res_k = in_alt ? ka : kp;
        const uint32_t* res_p = in_alt ? palt.as<uint32_t>() : pay.as<uint32_t>();
        SI_CK(sig::launch_decode<S>(res_k, res_p, d_in.as<int32_t>(), n, n_pad, si->starts.as<S>(),
                                    si->ends.as<S>(), si->data.as<int32_t>(), st));
        SI_CK(cudaMemcpyAsync(si->perm.p, res_p, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
        SI_CK(cudaStreamSynchronize(st));  // temps are released on scope exit
    }
    const S* ends = si->ends.as<S>();
    S* lp[sig::kMaxLevels];
    for (int h = 0; h < sig::kMaxLevels; ++h) lp[h] = si->lvl[h].as<S>();
    SI_CK(sig::launch_pyramid<S>(ends, si->lvl_sizes, si->H, lp, st));
    {
        DevBuf btmp;
        SI_TRY(btmp.reserve(sig::branch_temp_bytes(n_pad)));
        SI_CK(sig::launch_branch<S>(ends, n, n_pad, levels<S>(si), si->H, si->seg.as<int64_t>(), G,
                                    si->branch.as<int32_t>(), st, btmp.p, berr.as<int>()));
        SI_CK(cudaStreamSynchronize(st));  // the temporary is released on scope exit
    }
    // long-interval list of the batched path: intervals at least kLongIntervalSplit long, in
    // position order, with their own max pyramid (a tile reaches them without visiting the
    // positions in between)
    {
        DevBuf flags, offs, tmp;
        SI_TRY(flags.reserve(sizeof(uint32_t) * n));
        SI_TRY(offs.reserve(sizeof(int64_t) * (n + 1)));
        SI_TRY(tmp.reserve(sig::scan_temp_bytes(n)));
        SI_CK(sig::launch_long_flags<S>(si->starts.as<S>(), ends, n, sig::kLongIntervalSplit, flags.as<uint32_t>(),
                                        st));
        SI_CK(sig::exclusive_scan_u32_to_i64(flags.as<uint32_t>(), offs.as<int64_t>(), n, tmp.p, st, berr.as<int>()));
        int64_t n_long = 0;
        SI_CK(cudaMemcpyAsync(&n_long, offs.as<int64_t>() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        const int64_t n_long_pad = sig::round_up(std::max<int64_t>(n_long, 1), 32);
        SI_TRY(si->long_pos.reserve(sizeof(int32_t) * n_long_pad));
        SI_TRY(si->long_end.reserve(sizeof(S) * n_long_pad));
        SI_TRY(si->long_seg.reserve(sizeof(int64_t) * (G + 1)));
        si->long_H = sig::pyramid_levels(n_long_pad, si->long_sizes);
        for (int h = 1; h <= si->long_H; ++h) SI_TRY(si->long_lvl[h - 1].reserve(sizeof(S) * si->long_sizes[h]));
        SI_CK(sig::launch_long_scatter<S>(si->starts.as<S>(), ends, n, sig::kLongIntervalSplit, offs.as<int64_t>(),
                                          n_long, n_long_pad, si->seg.as<int64_t>(), G, si->long_pos.as<int32_t>(),
                                          si->long_end.as<S>(), si->long_seg.as<int64_t>(), st));
        S* llv[sig::kMaxLevels];
        for (int h = 0; h < sig::kMaxLevels; ++h) llv[h] = si->long_lvl[h].as<S>();
        SI_CK(sig::launch_pyramid<S>(si->long_end.as<S>(), si->long_sizes, si->long_H, llv, st));
        SI_CK(cudaStreamSynchronize(st));  // the temporaries are released on scope exit
    }
    si->bws.long_ends = si->long_end.p;
    si->bws.long_pos = si->long_pos.as<int32_t>();
    si->bws.long_seg = si->long_seg.as<int64_t>();
    for (int h = 0; h < sig::kMaxLevels; ++h) si->bws.long_lvl[h] = si->long_lvl[h].p;
    si->bws.long_H = si->long_H;
    si->bws.long_split = sig::kLongIntervalSplit;
    // intervals with start > end; when there are none, each contig's ends in ascending order,
    // from which the batched path counts short queries (two ranks per query)
    {
        DevBuf flag2;
        SI_TRY(flag2.reserve(8 + 2 * sizeof(unsigned long long)));
        unsigned long long* sums = reinterpret_cast<unsigned long long*>(flag2.as<char>() + 8);
        SI_CK(sig::launch_any_inverted<S>(view<S>(si), flag2.as<int>(), st));
        SI_CK(sig::launch_long_depth<S>(si->starts.as<S>(), si->ends.as<S>(), n, si->seg.as<int64_t>(), G,
                                         sig::kLongIntervalSplit, sums, st));
        int f = 0;
        unsigned long long h[2] = {0, 0};
        SI_CK(cudaMemcpyAsync(&f, flag2.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaMemcpyAsync(h, sums, sizeof(h), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        si->inverted = f ? 1 : 0;
        si->long_depth = h[1] > 0 ? (double)h[0] / (double)h[1] : 0.0;
    }
    if (si->inverted == 0) {
        const int K = sig::end_key_words<S>(G);
        DevBuf kw[3], kalt[3], pay, palt, tmp;
        uint32_t* kp[3];
        uint32_t* ka[3];
        for (int k = 0; k < K; ++k) {
            SI_TRY(kw[k].reserve(sizeof(uint32_t) * n));
            SI_TRY(kalt[k].reserve(sizeof(uint32_t) * n));
            kp[k] = kw[k].as<uint32_t>();
            ka[k] = kalt[k].as<uint32_t>();
        }
        SI_TRY(pay.reserve(sizeof(uint32_t) * n));
        SI_TRY(palt.reserve(sizeof(uint32_t) * n));
        const size_t tb = sig::radix_temp_bytes(n, K);
        SI_TRY(tmp.reserve(tb));
        SI_CK(sig::launch_end_keys<S>(ends, n, si->seg.as<int64_t>(), G, kp, st));
        bool in_alt = false;
        int passes = 0;
        SI_CK(sig::radix_sort(kp, ka, pay.as<uint32_t>(), palt.as<uint32_t>(), K, n, tmp.p, tb, &in_alt, &passes,
                              st, 0, berr.as<int>()));
        SI_TRY(si->end_sorted.reserve(sizeof(S) * n_pad));
        SI_CK(sig::launch_end_decode<S>(in_alt ? ka : kp, n, n_pad, si->end_sorted.as<S>(), st));
        SI_CK(cudaStreamSynchronize(st));  // the temporaries are released on scope exit
        si->bws.end_sorted = si->end_sorted.p;
    }
    SI_TRY(sig::batched_prepare<S>(si->bws, view<S>(si), levels<S>(si), si->H, si->lvl_sizes,
                                   si->ub_mode, st));
    SI_CK(cudaStreamSynchronize(st));
    SI_CK(cudaGetLastError());
    {
        int be = 0;
        SI_CK(cudaMemcpy(&be, berr.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (be) return fail(SI_ERR_CUDA, "build: a bounded wait in a sort or scan kernel gave up (%d)", be);
    }
    si->built = true;
    return SI_OK;
}

int check_built(const gSuperIntervals* si) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (!si->built) return fail(SI_ERR_NOT_BUILT, "index not built (call indexSuperIntervalsGpu after adding)");
    return SI_OK;
}

// Reads the device error word after the work queued on `st` (the handle's stream by default).
int read_dev_err(gSuperIntervals* si, cudaStream_t st = nullptr) {
    if (!st) st = si->st;
    int e = 0;
    SI_CK(cudaMemcpyAsync(&e, si->w_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (e == sig::kDevBadContig) return fail(SI_ERR_INVALID, "a query names a contig outside [0, %d)", si->G);
    if (e == sig::kDevOverflow) return fail(SI_ERR_CUDA, "internal: emit overran its offsets");
    if (e == sig::kDevTimeout) return fail(SI_ERR_CUDA, "a bounded wait in a sort or scan kernel gave up");
    if (e != 0) return fail(SI_ERR_CUDA, "device error word %d", e);
    return SI_OK;
}

// The automatic choice: the batched path for batches of 4096+ queries; for smaller ones the plain
// path (one warp per query), except that searches (emit) over an index whose long intervals
// nest deeply (kDeepLong or more over a position on average) take the batched path, which
// gathers long candidates per tile instead of walking to each one.
constexpr double kDeepLong = 32.0;
bool use_batched(const gSuperIntervals* si, int64_t nq, bool emit = false) {
    if (si->path == SI_PATH_PLAIN) return false;
    if (si->path == SI_PATH_BATCHED) return true;
    if (si->n < 4096) return false;
    return nq >= 4096 || (emit && si->long_depth >= kDeepLong);
}

// count into d_counts (device) for device-resident queries
template <typename S>
int run_count(gSuperIntervals* si, const sig::QueryBatch& q, uint32_t* d_counts, cudaStream_t st,
              bool for_emit = false) {
    SI_TRY(si->w_err.reserve(sizeof(int)));
    SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st));
    if (si->n == 0) {
        SI_CK(cudaMemsetAsync(d_counts, 0, sizeof(uint32_t) * std::max<int64_t>(q.nq, 1), st));
        SI_CK(sig::launch_check_contigs(q.qc, q.nq, si->G, si->w_err.as<int>(), st));
        return SI_OK;
    }
    if (use_batched(si, q.nq, for_emit)) {
        {
            PhaseTimer pt(si, 3, st);
            int r = sig::batched_prepare_queries<S>(si->bws, view<S>(si), q, si->w_err.as<int>(), si->ub_mode, st,
                                                    d_counts);
            if (r != SI_OK) return fail(r, "batched query preparation failed (status %d)", r);
        }
        PhaseTimer pt(si, 0, st);
        int r = sig::batched_count<S>(si->bws, view<S>(si), levels<S>(si), si->H, q, d_counts, si->w_err.as<int>(), st);
        if (r != SI_OK) return fail(r, "batched count failed (status %d)", r);
    } else {
        PhaseTimer pt(si, 0, st);
        SI_CK(sig::launch_count_plain<S>(view<S>(si), q, d_counts, si->w_err.as<int>(), st));
    }
    return SI_OK;
}

// q may be a slice starting at query q_offset of the batch counted last.
// total_hits: the result count of the whole batch counted last (-1 unknown; sizes the tiles)
template <typename S>
int run_emit(gSuperIntervals* si, const sig::QueryBatch& q, int64_t q_offset, const int64_t* d_offsets,
             int64_t out_base, int order, bool values, int32_t* d_out, cudaStream_t st, int64_t total_hits) {
    if (si->n == 0 || q.nq == 0) return SI_OK;
    PhaseTimer pt(si, 2, st);
    if (use_batched(si, q.nq + q_offset, true)) {
        int r = sig::batched_emit<S>(si->bws, view<S>(si), levels<S>(si), si->H, q, q_offset, d_offsets, out_base,
                                     order, values, d_out, si->w_err.as<int>(), si->ub_mode, st, total_hits);
        if (r != SI_OK) return fail(r, "batched emit failed (status %d)", r);
    } else {
        SI_CK(sig::launch_emit_plain<S>(view<S>(si), q, d_offsets, out_base, order, values, d_out,
                                        si->w_err.as<int>(), st));
    }
    return SI_OK;
}

// device-resident queries and outputs
template <typename S>
int search_device(gSuperIntervals* si, const sig::QueryBatch& q, int order, bool values,
                  int64_t* d_offsets, int32_t* d_out, size_t cap, size_t* total, cudaStream_t st) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * std::max<int64_t>(q.nq, 1)));
    SI_TRY(si->w_tmp.reserve(sig::scan_temp_bytes(q.nq)));
    SI_TRY(run_count<S>(si, q, si->w_counts.as<uint32_t>(), st, true));
    {
        PhaseTimer pt(si, 1, st);
        SI_CK(sig::exclusive_scan_u32_to_i64(si->w_counts.as<uint32_t>(), d_offsets, q.nq, si->w_tmp.p, st, si->w_err.as<int>()));
    }
    int64_t P = 0;
    SI_CK(cudaMemcpyAsync(&P, d_offsets + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (total) *total = (size_t)P;
    if ((size_t)P > cap) return fail(SI_ERR_CAPACITY, "output needs %lld values, capacity %zu", (long long)P, cap);
    SI_TRY(run_emit<S>(si, q, 0, d_offsets, 0, order, values, d_out, st, P));
    return read_dev_err(si, st);
}

template <typename S>
int upload_queries(gSuperIntervals* si, const S* qs, const S* qe, const int32_t* qc, size_t nq,
                   sig::QueryBatch& q) {
    if (nq && (!qs || !qe)) return fail(SI_ERR_INVALID, "null query arrays");
    SI_TRY(si->wq_s.reserve(sizeof(S) * std::max<size_t>(nq, 1)));
    SI_TRY(si->wq_e.reserve(sizeof(S) * std::max<size_t>(nq, 1)));
    if (nq) {
        SI_CK(cudaMemcpyAsync(si->wq_s.p, qs, sizeof(S) * nq, cudaMemcpyHostToDevice, si->st));
        SI_CK(cudaMemcpyAsync(si->wq_e.p, qe, sizeof(S) * nq, cudaMemcpyHostToDevice, si->st));
    }
    q.qs = si->wq_s.p;
    q.qe = si->wq_e.p;
    q.qc = nullptr;
    if (qc) {
        // contig ids are checked on the device by the kernels that read them (error word)
        SI_TRY(si->wq_c.reserve(sizeof(int32_t) * std::max<size_t>(nq, 1)));
        if (nq) SI_CK(cudaMemcpyAsync(si->wq_c.p, qc, sizeof(int32_t) * nq, cudaMemcpyHostToDevice, si->st));
        q.qc = si->wq_c.as<int32_t>();
    }
    q.nq = (int64_t)nq;
    return SI_OK;
}

// host queries -> host CSR; result grown when `grow` is set, else caller buffers
template <typename S>
int search_host(gSuperIntervals* si, const S* qs, const S* qe, const int32_t* qc, size_t nq, int order,
                bool values, cCsrResult* grow, int64_t* h_off, int32_t* h_out, size_t cap, size_t* total) {
    SI_TRY(check_width<S>(si));
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    cudaStream_t st = si->st;
    if (grow) {
        if (grow->offsets_capacity < nq + 1) {
            int64_t* p = (int64_t*)realloc(grow->offsets, sizeof(int64_t) * (nq + 1));
            if (!p) return fail(SI_ERR_OOM, "host allocation of %zu offsets failed", nq + 1);
            grow->offsets = p;
            grow->offsets_capacity = nq + 1;
        }
        h_off = grow->offsets;
        grow->n_queries = nq;
        grow->size = 0;
    }
    sig::QueryBatch q;
    SI_TRY(upload_queries<S>(si, qs, qe, qc, nq, q));
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * std::max<size_t>(nq, 1)));
    SI_TRY(si->w_offsets.reserve(sizeof(int64_t) * (nq + 1)));
    SI_TRY(si->w_tmp.reserve(sig::scan_temp_bytes((int64_t)nq)));
    SI_TRY(run_count<S>(si, q, si->w_counts.as<uint32_t>(), st, true));
    int64_t* d_off = si->w_offsets.as<int64_t>();
    {
        PhaseTimer pt(si, 1, st);
        SI_CK(sig::exclusive_scan_u32_to_i64(si->w_counts.as<uint32_t>(), d_off, (int64_t)nq, si->w_tmp.p, st, si->w_err.as<int>()));
    }
    SI_CK(cudaMemcpyAsync(h_off, d_off, sizeof(int64_t) * (nq + 1), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    const int64_t P = h_off[nq];
    if (total) *total = (size_t)P;
    if (grow) {
        if (grow->capacity < (size_t)P) {
            int32_t* p = (int32_t*)realloc(grow->values, sizeof(int32_t) * std::max<int64_t>(P, 1));
            if (!p) return fail(SI_ERR_OOM, "host allocation of %lld values failed", (long long)P);
            grow->values = p;
            grow->capacity = (size_t)P;
        }
        h_out = grow->values;
        grow->size = (size_t)P;
    } else if ((size_t)P > cap) {
        return fail(SI_ERR_CAPACITY, "output needs %lld values, capacity %zu", (long long)P, cap);
    }
    if (P == 0) return read_dev_err(si);
    // Results are staged in device memory and copied in bulk: the emit writes every query's
    // list at a scattered place, and such writes over the host link run several times slower
    // than one large copy.  The output is cut into chunks of queries whose lists fit the
    // device output budget; with more than one chunk, chunks alternate between two device
    // buffers and the emit of one overlaps the copy of the one before (copy stream).
    const int64_t budget = std::max<int64_t>((int64_t)(si->out_budget / sizeof(int32_t)), 1 << 20);
    const int64_t buf = std::min<int64_t>(P, budget);
    std::vector<size_t> cuts{0};
    for (size_t qa = 0; qa < nq;) {
        // largest qb with off[qb] - off[qa] <= buf (at least one query)
        const int64_t limit = h_off[qa] + buf;
        size_t lo = qa + 1, hi = nq;
        while (lo < hi) {
            size_t mid = lo + (hi - lo + 1) / 2;
            if (h_off[mid] <= limit) lo = mid;
            else hi = mid - 1;
        }
        cuts.push_back(lo);
        qa = lo;
    }
    const size_t n_chunks = cuts.size() - 1;
    int64_t max_need = 1;
    for (size_t c = 0; c < n_chunks; ++c) max_need = std::max<int64_t>(max_need, h_off[cuts[c + 1]] - h_off[cuts[c]]);
    SI_TRY(si->w_out.reserve(sizeof(int32_t) * max_need));
    if (n_chunks > 1) {
        SI_TRY(si->w_out2.reserve(sizeof(int32_t) * max_need));
        if (!si->copy_st) SI_CK(cudaStreamCreateWithFlags(&si->copy_st, cudaStreamNonBlocking));
        for (int b = 0; b < 2; ++b) {
            if (!si->ev_emitted[b]) SI_CK(cudaEventCreateWithFlags(&si->ev_emitted[b], cudaEventDisableTiming));
            if (!si->ev_copied[b]) SI_CK(cudaEventCreateWithFlags(&si->ev_copied[b], cudaEventDisableTiming));
        }
    }
    auto chunk = [&](size_t c) -> int {
        const size_t qa = cuts[c], qb = cuts[c + 1];
        const int64_t need = h_off[qb] - h_off[qa];
        const int b = (int)(c & 1);
        int32_t* dbuf = b ? si->w_out2.as<int32_t>() : si->w_out.as<int32_t>();
        // the buffer's previous copy (chunk c - 2) must be done before the emit overwrites it
        if (c >= 2) SI_CK(cudaStreamWaitEvent(st, si->ev_copied[b], 0));
        sig::QueryBatch sub = q;
        sub.qs = static_cast<const S*>(q.qs) + qa;
        sub.qe = static_cast<const S*>(q.qe) + qa;
        sub.qc = q.qc ? q.qc + qa : nullptr;
        sub.nq = (int64_t)(qb - qa);
        SI_TRY(run_emit<S>(si, sub, (int64_t)qa, d_off + qa, h_off[qa], order, values, dbuf, st, P));
        if (n_chunks == 1) {
            if (need)
                SI_CK(cudaMemcpyAsync(h_out + h_off[qa], dbuf, sizeof(int32_t) * need, cudaMemcpyDeviceToHost, st));
            return SI_OK;
        }
        SI_CK(cudaEventRecord(si->ev_emitted[b], st));
        SI_CK(cudaStreamWaitEvent(si->copy_st, si->ev_emitted[b], 0));
        if (need)
            SI_CK(cudaMemcpyAsync(h_out + h_off[qa], dbuf, sizeof(int32_t) * need, cudaMemcpyDeviceToHost,
                                  si->copy_st));
        SI_CK(cudaEventRecord(si->ev_copied[b], si->copy_st));
        return SI_OK;
    };
    for (size_t c = 0; c < n_chunks; ++c) {
        const int r = chunk(c);
        if (r != SI_OK) {
            // copies already queued finish before the buffers can be reused by a later call
            if (si->copy_st) cudaStreamSynchronize(si->copy_st);
            cudaStreamSynchronize(st);
            return r;
        }
    }
    // the compute stream waits for the last copy (the copy stream runs in order), so later
    // work on it sees the results
    if (n_chunks > 1) SI_CK(cudaStreamWaitEvent(st, si->ev_copied[(n_chunks - 1) & 1], 0));
    SI_CK(cudaStreamSynchronize(st));
    return read_dev_err(si);
}

template <typename S>
int count_host(gSuperIntervals* si, const S* qs, const S* qe, const int32_t* qc, size_t nq, uint32_t* counts) {
    SI_TRY(check_width<S>(si));
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (nq && !counts) return fail(SI_ERR_INVALID, "null output");
    sig::QueryBatch q;
    SI_TRY(upload_queries<S>(si, qs, qe, qc, nq, q));
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * std::max<size_t>(nq, 1)));
    SI_TRY(run_count<S>(si, q, si->w_counts.as<uint32_t>(), si->st));
    if (nq) SI_CK(cudaMemcpyAsync(counts, si->w_counts.p, sizeof(uint32_t) * nq, cudaMemcpyDeviceToHost, si->st));
    return read_dev_err(si);
}

template <typename S>
int any_host(gSuperIntervals* si, const S* qs, const S* qe, const int32_t* qc, size_t nq, uint8_t* out) {
    SI_TRY(check_width<S>(si));
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (nq && !out) return fail(SI_ERR_INVALID, "null output");
    sig::QueryBatch q;
    SI_TRY(upload_queries<S>(si, qs, qe, qc, nq, q));
    SI_TRY(si->w_err.reserve(sizeof(int)));
    SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), si->st));
    if (si->n == 0) {
        memset(out, 0, nq);
        SI_CK(sig::launch_check_contigs(q.qc, q.nq, si->G, si->w_err.as<int>(), si->st));
        return read_dev_err(si);
    }
    SI_TRY(si->w_out.reserve(std::max<size_t>(nq, 1)));
    SI_CK(sig::launch_any_plain<S>(view<S>(si), q, si->w_out.as<uint8_t>(), si->w_err.as<int>(), si->st));
    if (nq) SI_CK(cudaMemcpyAsync(out, si->w_out.p, nq, cudaMemcpyDeviceToHost, si->st));
    return read_dev_err(si);
}

template <typename S>
int get_arrays(const gSuperIntervals* si, S* s, S* e, int32_t* d, int64_t* br) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    const int64_t n = si->n;
    if (n == 0) return SI_OK;
    cudaStream_t st = si->st;
    if (s) SI_CK(cudaMemcpyAsync(s, si->starts.p, sizeof(S) * n, cudaMemcpyDeviceToHost, st));
    if (e) SI_CK(cudaMemcpyAsync(e, si->ends.p, sizeof(S) * n, cudaMemcpyDeviceToHost, st));
    if (d) SI_CK(cudaMemcpyAsync(d, si->data.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    std::vector<int32_t> b32;
    if (br) {
        b32.resize(n);
        SI_CK(cudaMemcpyAsync(b32.data(), si->branch.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
    }
    SI_CK(cudaStreamSynchronize(st));
    if (br) {
        std::vector<int64_t> segv = si->hseg;
        if (segv.empty()) segv = {0, n};
        for (int g = 0; g < si->G; ++g)
            for (int64_t i = segv[g]; i < segv[g + 1]; ++i) br[i] = b32[i] < 0 ? -1 : (int64_t)b32[i] - segv[g];
    }
    return SI_OK;
}

}  // namespace

// =====================================================================================
extern "C" {

int createSuperIntervalsGpu(gSuperIntervals** out, int coord_bits, int device) {
    if (!out) return fail(SI_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (coord_bits != 32 && coord_bits != 64) return fail(SI_ERR_INVALID, "coord_bits must be 32 or 64");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SI_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    }
    if (device < 0 || device >= ndev) return fail(SI_ERR_INVALID, "device %d outside [0, %d)", device, ndev);
    SI_CK(cudaSetDevice(device));
    auto* si = new gSuperIntervals();
    si->bits = coord_bits;
    si->device = device;
    {
        // result chunks of host-buffer searches: 1/16 of the device's memory (at least 4 GiB), so
        // that a result of tens of GB takes a few emit passes over the batch's tiles, not dozens
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
            si->out_budget = std::max(si->out_budget, total_b / 16);
        cudaGetLastError();
    }
    e = cudaStreamCreateWithFlags(&si->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete si;
        return fail(SI_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    *out = si;
    return SI_OK;
}

void destroySuperIntervalsGpu(gSuperIntervals* si) {
    if (!si) return;
    cudaSetDevice(si->device);
    cudaStreamSynchronize(si->st);
    if (si->ev0) cudaEventDestroy(si->ev0);
    if (si->ev1) cudaEventDestroy(si->ev1);
    if (si->copy_st) {
        cudaStreamSynchronize(si->copy_st);
        cudaStreamDestroy(si->copy_st);
    }
    for (int b = 0; b < 2; ++b) {
        if (si->ev_emitted[b]) cudaEventDestroy(si->ev_emitted[b]);
        if (si->ev_copied[b]) cudaEventDestroy(si->ev_copied[b]);
    }
    if (si->gexec) cudaGraphExecDestroy(si->gexec);
    cudaStream_t st = si->st;
    delete si;  // releases device buffers
    cudaStreamDestroy(st);
}

int clearSuperIntervalsGpu(gSuperIntervals* si) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    si->hs32.clear(); si->he32.clear(); si->hs64.clear(); si->he64.clear(); si->hdata.clear();
    si->hseg.clear();
    si->contig_names.clear();
    si->built = false;
    si->n = 0;
    return SI_OK;
}

int reserveSuperIntervalsGpu(gSuperIntervals* si, size_t n) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (si->bits == 32) { si->hs32.reserve(n); si->he32.reserve(n); }
    else { si->hs64.reserve(n); si->he64.reserve(n); }
    si->hdata.reserve(n);
    return SI_OK;
}

int addIntervalGpu(gSuperIntervals* si, int32_t start, int32_t end, int32_t value) {
    return add_many<int32_t>(si, &start, &end, &value, 1);
}
int addIntervalGpu_i64(gSuperIntervals* si, int64_t start, int64_t end, int32_t value) {
    return add_many<int64_t>(si, &start, &end, &value, 1);
}
int addIntervalsGpu(gSuperIntervals* si, const int32_t* s, const int32_t* e, const int32_t* v, size_t n) {
    return add_many<int32_t>(si, s, e, v, n);
}
int addIntervalsGpu_i64(gSuperIntervals* si, const int64_t* s, const int64_t* e, const int32_t* v, size_t n) {
    return add_many<int64_t>(si, s, e, v, n);
}

int setContigsGpu(gSuperIntervals* si, size_t n_contigs, const int64_t* offsets) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (n_contigs == 0 || !offsets) return fail(SI_ERR_INVALID, "need at least one contig");
    if (offsets[0] != 0 || offsets[n_contigs] != (int64_t)staged(si))
        return fail(SI_ERR_INVALID, "contig offsets must run from 0 to the staged count %zu", staged(si));
    for (size_t g = 0; g < n_contigs; ++g)
        if (offsets[g + 1] < offsets[g]) return fail(SI_ERR_INVALID, "contig offsets decrease at %zu", g);
    if (n_contigs >= (size_t)INT32_MAX) return fail(SI_ERR_INVALID, "too many contigs");
    si->hseg.assign(offsets, offsets + n_contigs + 1);
    if (si->contig_names.size() != n_contigs) si->contig_names.clear();
    si->built = false;
    return SI_OK;
}

size_t sizeSuperIntervalsGpu(const gSuperIntervals* si) { return si ? staged(si) : 0; }
size_t numContigsGpu(const gSuperIntervals* si) {
    return si ? (si->hseg.empty() ? 1 : si->hseg.size() - 1) : 0;
}

int indexSuperIntervalsGpu(gSuperIntervals* si) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    return si->bits == 64 ? build_impl<int64_t>(si) : build_impl<int32_t>(si);
}

int getIndexArraysGpu(const gSuperIntervals* si, void* s, void* e, int32_t* d, int64_t* br) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (si->bits == 64) return get_arrays<int64_t>(si, (int64_t*)s, (int64_t*)e, d, br);
    return get_arrays<int32_t>(si, (int32_t*)s, (int32_t*)e, d, br);
}

int setQueryPathGpu(gSuperIntervals* si, int path) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (path < SI_PATH_AUTO || path > SI_PATH_BATCHED) return fail(SI_ERR_INVALID, "unknown path %d", path);
    si->path = path;
    return SI_OK;
}

int setUpperBoundModeGpu(gSuperIntervals* si, int mode) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (mode < SI_UB_BINARY || mode > SI_UB_LEARNED) return fail(SI_ERR_INVALID, "unknown mode %d", mode);
    si->ub_mode = mode;
    if (si->built) {
        SI_TRY(set_dev(si));
        int r = si->bits == 64
                    ? sig::batched_prepare<int64_t>(si->bws, view<int64_t>(si), levels<int64_t>(si), si->H,
                                                    si->lvl_sizes, mode, si->st)
                    : sig::batched_prepare<int32_t>(si->bws, view<int32_t>(si), levels<int32_t>(si), si->H,
                                                    si->lvl_sizes, mode, si->st);
        if (r != SI_OK) return r;
        SI_CK(cudaStreamSynchronize(si->st));
    }
    return SI_OK;
}

int setOutputBudgetGpu(gSuperIntervals* si, size_t bytes) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    si->out_budget = std::max<size_t>(bytes, 1 << 20);
    return SI_OK;
}

int setProfilingGpu(gSuperIntervals* si, int on) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    SI_TRY(set_dev(si));
    if (on && !si->ev0) {
        SI_CK(cudaEventCreate(&si->ev0));
        SI_CK(cudaEventCreate(&si->ev1));
    }
    si->prof = on != 0;
    for (int k = 0; k < 4; ++k) {
        si->phase_ms[k] = 0;
        si->phase_n[k] = 0;
    }
    return SI_OK;
}

int getPhaseTimesGpu(const gSuperIntervals* si, double* ms, int64_t* calls) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    for (int k = 0; k < 4; ++k) {
        if (ms) ms[k] = si->phase_ms[k];
        if (calls) calls[k] = si->phase_n[k];
    }
    return SI_OK;
}

int setDeviceBudgetGpu(size_t bytes) {
    g_budget = bytes;
    return SI_OK;
}
size_t deviceBytesInUseGpu(void) { return g_used.load(); }

int deviceMemInfoGpu(int device, size_t* free_bytes, size_t* total_bytes) {
    SI_CK(cudaSetDevice(device));
    size_t f = 0, t = 0;
    SI_CK(cudaMemGetInfo(&f, &t));
    if (free_bytes) *free_bytes = f;
    if (total_bytes) *total_bytes = t;
    return SI_OK;
}

int countOverlapsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe, const int32_t* qc,
                          size_t nq, uint32_t* counts) {
    return count_host<int32_t>(si, qs, qe, qc, nq, counts);
}
int countOverlapsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe, const int32_t* qc,
                              size_t nq, uint32_t* counts) {
    return count_host<int64_t>(si, qs, qe, qc, nq, counts);
}
int anyOverlapsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe, const int32_t* qc,
                        size_t nq, uint8_t* out) {
    return any_host<int32_t>(si, qs, qe, qc, nq, out);
}
int anyOverlapsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe, const int32_t* qc,
                            size_t nq, uint8_t* out) {
    return any_host<int64_t>(si, qs, qe, qc, nq, out);
}
int searchIdxsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe, const int32_t* qc,
                       size_t nq, int order, cCsrResult* out) {
    if (!out) return fail(SI_ERR_INVALID, "null result");
    return search_host<int32_t>(si, qs, qe, qc, nq, order, false, out, nullptr, nullptr, 0, nullptr);
}
int searchIdxsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe, const int32_t* qc,
                           size_t nq, int order, cCsrResult* out) {
    if (!out) return fail(SI_ERR_INVALID, "null result");
    return search_host<int64_t>(si, qs, qe, qc, nq, order, false, out, nullptr, nullptr, 0, nullptr);
}
int searchValuesBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe, const int32_t* qc,
                         size_t nq, cCsrResult* out) {
    if (!out) return fail(SI_ERR_INVALID, "null result");
    return search_host<int32_t>(si, qs, qe, qc, nq, SI_ORDER_DESC, true, out, nullptr, nullptr, 0, nullptr);
}
int searchValuesBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe, const int32_t* qc,
                             size_t nq, cCsrResult* out) {
    if (!out) return fail(SI_ERR_INVALID, "null result");
    return search_host<int64_t>(si, qs, qe, qc, nq, SI_ORDER_DESC, true, out, nullptr, nullptr, 0, nullptr);
}
int searchBatchIntoGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qc, size_t nq,
                       int order, int values_not_idxs, int64_t* offsets, int32_t* values, size_t capacity,
                       size_t* total) {
    if (!si || !offsets) return fail(SI_ERR_INVALID, "null handle or offsets");
    if (order != SI_ORDER_IDXS_CPP && order != SI_ORDER_DESC) return fail(SI_ERR_INVALID, "unknown order");
    if (si->bits == 64)
        return search_host<int64_t>(si, (const int64_t*)qs, (const int64_t*)qe, qc, nq, order, values_not_idxs != 0,
                                    nullptr, offsets, values, capacity, total);
    return search_host<int32_t>(si, (const int32_t*)qs, (const int32_t*)qe, qc, nq, order, values_not_idxs != 0,
                                nullptr, offsets, values, capacity, total);
}

int countOverlapsDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                           size_t nq, uint32_t* d_counts, void* stream) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64) SI_TRY(run_count<int64_t>(si, q, d_counts, st));
    else SI_TRY(run_count<int32_t>(si, q, d_counts, st));
    return SI_OK;
}

int searchDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc, size_t nq,
                    int order, int values_not_idxs, int64_t* d_offsets, int32_t* d_values, size_t capacity,
                    size_t* total, void* stream) {
    if (!si || !d_offsets) return fail(SI_ERR_INVALID, "null handle or offsets");
    if (order != SI_ORDER_IDXS_CPP && order != SI_ORDER_DESC) return fail(SI_ERR_INVALID, "unknown order");
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64)
        return search_device<int64_t>(si, q, order, values_not_idxs != 0, d_offsets, d_values, capacity, total, st);
    return search_device<int32_t>(si, q, order, values_not_idxs != 0, d_offsets, d_values, capacity, total, st);
}

cCsrResult createCsrResult(void) {
    cCsrResult r;
    memset(&r, 0, sizeof(r));
    return r;
}
void clearCsrResult(cCsrResult* r) {
    if (r) { r->size = 0; r->n_queries = 0; }
}
void destroyCsrResult(cCsrResult* r) {
    if (!r) return;
    free(r->offsets);
    free(r->values);
    memset(r, 0, sizeof(*r));
}

const char* lastErrorGpu(void) { return g_err.c_str(); }
void* getStreamGpu(gSuperIntervals* si) { return si ? (void*)si->st : nullptr; }

int deviceCountGpu(int* count) {
    if (!count) return fail(SI_ERR_INVALID, "null output");
    cudaError_t e = cudaGetDeviceCount(count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *count = 0;
        return fail(SI_ERR_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    }
    return SI_OK;
}
int deviceMallocGpu(void** ptr, size_t bytes) {
    if (!ptr) return fail(SI_ERR_INVALID, "null output");
    const size_t cap = g_budget.load();
    if (cap && g_used.load() + bytes > cap) return fail(SI_ERR_OOM, "device budget exceeded");
    cudaError_t e = cudaMalloc(ptr, std::max<size_t>(bytes, 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(SI_ERR_OOM, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return SI_OK;
}
int deviceFreeGpu(void* ptr) {
    SI_CK(cudaFree(ptr));
    return SI_OK;
}
int hostMallocPinnedGpu(void** ptr, size_t bytes) {
    if (!ptr) return fail(SI_ERR_INVALID, "null output");
    cudaError_t e = cudaMallocHost(ptr, std::max<size_t>(bytes, 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return fail(SI_ERR_OOM, "cudaMallocHost(%zu): %s", bytes, cudaGetErrorString(e));
    }
    return SI_OK;
}
int hostFreePinnedGpu(void* ptr) {
    SI_CK(cudaFreeHost(ptr));
    return SI_OK;
}
int memcpyGpu(void* dst, const void* src, size_t bytes, void* stream) {
    SI_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream));
    return SI_OK;
}
int streamSynchronizeGpu(void* stream) {
    SI_CK(cudaStreamSynchronize((cudaStream_t)stream));
    return SI_OK;
}
int eventCreateGpu(void** ev) {
    SI_CK(cudaEventCreate((cudaEvent_t*)ev));
    return SI_OK;
}
int eventDestroyGpu(void* ev) {
    SI_CK(cudaEventDestroy((cudaEvent_t)ev));
    return SI_OK;
}
int eventRecordGpu(void* ev, void* stream) {
    SI_CK(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream));
    return SI_OK;
}
int eventElapsedMsGpu(void* a, void* b, float* ms) {
    SI_CK(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b));
    return SI_OK;
}
int flushL2Gpu(void* stream) {
    static std::mutex mu;
    static void* buf[64] = {nullptr};
    static int flip = 0;
    int dev = 0;
    SI_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(SI_ERR_INVALID, "device id");
    const size_t bytes = (size_t)512 << 20;  // 4x the 129 MB L2
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!buf[dev]) SI_CK(cudaMalloc(&buf[dev], bytes));
        flip ^= 1;
    }
    SI_CK(cudaMemsetAsync(buf[dev], flip, bytes, (cudaStream_t)stream));
    return SI_OK;
}

}  // extern "C"

extern "C" int upperBoundDeviceGpu(gSuperIntervals* si, const void* d_qe, const int32_t* d_qc, size_t nq, int mode,
                                   int32_t* d_out, void* stream) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (mode != SI_UB_BINARY && mode != si->ub_mode)
        return fail(SI_ERR_INVALID, "upper-bound mode %d is not prepared on this handle (current %d)", mode,
                    si->ub_mode);
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    SI_TRY(si->w_err.reserve(sizeof(int)));
    SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st));
    if (si->n == 0) {
        if (nq) SI_CK(cudaMemsetAsync(d_out, 0xff, sizeof(int32_t) * nq, st));
        return SI_OK;
    }
    sig::QueryBatch q{d_qe, d_qe, d_qc, (int64_t)nq};
    // the batched query path sorts the ends first (same answers): see setQueryPathGpu
    const bool sorted = use_batched(si, (int64_t)nq);
    int r = si->bits == 64
                ? sig::upper_bounds<int64_t>(si->bws, view<int64_t>(si), q, mode, d_out, si->w_err.as<int>(), st,
                                             sorted)
                : sig::upper_bounds<int32_t>(si->bws, view<int32_t>(si), q, mode, d_out, si->w_err.as<int>(), st,
                                             sorted);
    if (r != SI_OK) return fail(r, "upper-bound kernel failed");
    return SI_OK;
}

extern "C" int setBatchedParamsGpu(gSuperIntervals* si, int tile_q, int cap, int64_t long_len, int64_t split_len) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    sig::BatchedParams p = si->bws.prm;
    if (tile_q > 0) {
        p.tile_q = tile_q;
        p.auto_tile = false;
    } else if (tile_q < 0) {
        p.auto_tile = true;
    }
    if (cap) p.cap = cap;
    if (long_len) p.long_len = long_len;
    if (split_len >= 0) p.split_len = split_len;
    if (p.tile_q < 32 || p.tile_q > 1024 || (p.tile_q & 31))
        return fail(SI_ERR_INVALID, "tile_queries must be a multiple of 32 in [32, 1024]");
    if (p.cap < 256 || p.cap > 8192 || (p.cap & 255))
        return fail(SI_ERR_INVALID, "tile_candidates must be a multiple of 256 in [256, 8192]");
    if (p.long_len < 1) return fail(SI_ERR_INVALID, "long_query_len must be positive");
    si->bws.prm = p;
    return SI_OK;
}

extern "C" int getBatchedParamsGpu(const gSuperIntervals* si, int* tile_q, int* cap, int64_t* long_len,
                                   int64_t* split_len) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (tile_q) *tile_q = si->bws.prm.tile_q;
    if (cap) *cap = si->bws.prm.cap;
    if (long_len) *long_len = si->bws.prm.long_len;
    if (split_len) *split_len = si->bws.prm.split_len;
    return SI_OK;
}

extern "C" int setBatchedOptionGpu(gSuperIntervals* si, int option, int64_t value) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (option == SI_OPT_EMIT_COPY) {
        si->bws.prm.emit_copy = value != 0;
        return SI_OK;
    }
    if (option == SI_OPT_EYTZ_DEPTH) {
        if (value < 0 || value > 13) return fail(SI_ERR_INVALID, "Eytzinger depth %lld outside [0, 13]", (long long)value);
        si->bws.prm.eytz_depth = (int)value;
        // the tree is sampled at build time: rebuild it when it is the current provider
        if (si->built && si->ub_mode == SI_UB_EYTZINGER) return setUpperBoundModeGpu(si, SI_UB_EYTZINGER);
        return SI_OK;
    }
    return fail(SI_ERR_INVALID, "unknown option %d", option);
}

extern "C" int getBatchedOptionGpu(const gSuperIntervals* si, int option, int64_t* value) {
    if (!si || !value) return fail(SI_ERR_INVALID, "null argument");
    if (option == SI_OPT_EMIT_COPY) *value = si->bws.prm.emit_copy ? 1 : 0;
    else if (option == SI_OPT_EYTZ_DEPTH) *value = si->bws.ub.eytz_depth > 0 ? si->bws.ub.eytz_depth : si->bws.prm.eytz_depth;
    else return fail(SI_ERR_INVALID, "unknown option %d", option);
    return SI_OK;
}

// =====================================================================================
// Allocation-free search (searchIdxsNoAllocGpu).
//
// Some callers cannot allocate device memory while they query: a host whose device memory is
// owned by another allocator or a fixed pool, a query thread that must not grow its memory
// footprint, or code that is not allowed to call cudaMalloc at that point.  For them this entry
// point runs the count -> scan -> emit search without allocating anything: the caller passes
// device buffers for the queries, the offsets and the results, and the scratch the search needs
// (per-query counts, scan partials, a device error word) lives in one file-scope device array of
// fixed size.  The index must already be built (building allocates).
//
// Limits:
//   * at most kNoAllocMaxQueries queries per call; larger batches are rejected (SI_ERR_TOO_LARGE);
//   * the array is part of the library image, so every device that loads the library holds it
//     (about 16.1 MiB) until the process exits;
//   * every call shares the array and it keeps the last call's contents: calls that overlap on
//     the GPU (other streams, threads or handles) race on it, so the caller serializes them;
//   * the first call on a device looks up the array's device address with that device current;
//     make that first call before any stream capture;
//   * every call reads the result size back into host memory and waits for its stream, so it
//     returns with the search finished.
// =====================================================================================
namespace {

constexpr size_t kNoAllocMaxQueries = (size_t)1 << 22;
constexpr size_t kNoAllocHeader = 256;        // device error word
constexpr size_t kNoAllocScanBytes = 64 << 10;  // scan partials for up to kNoAllocMaxQueries
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocScanBytes + kNoAllocMaxQueries * sizeof(uint32_t);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
int noalloc_scratch(int device, unsigned char** out) {
    if (device < 0 || device >= 64) return fail(SI_ERR_INVALID, "device id %d out of range", device);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(SI_ERR_CUDA, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
        }
        g_noalloc_addr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_addr[device]);
    return SI_OK;
}

template <typename S>
int search_noalloc(gSuperIntervals* si, const sig::QueryBatch& q, int order, int64_t* d_offsets, int32_t* d_out,
                   size_t capacity, size_t* total, cudaStream_t st) {
    unsigned char* base = nullptr;
    SI_TRY(noalloc_scratch(si->device, &base));
    int* d_err = reinterpret_cast<int*>(base);
    void* scan_tmp = base + kNoAllocHeader;
    uint32_t* counts = reinterpret_cast<uint32_t*>(base + kNoAllocHeader + kNoAllocScanBytes);
    if (sig::scan_temp_bytes(q.nq) > kNoAllocScanBytes)
        return fail(SI_ERR_TOO_LARGE, "scan scratch too small for %lld queries", (long long)q.nq);
    SI_CK(cudaMemsetAsync(d_err, 0, sizeof(int), st));  // the error word starts at zero
    if (si->n == 0 || q.nq == 0) {
        SI_CK(cudaMemsetAsync(d_offsets, 0, sizeof(int64_t) * (q.nq + 1), st));
        // an empty index still rejects contig ids outside [0, G), as searchDeviceGpu does
        SI_CK(sig::launch_check_contigs(q.qc, q.nq, si->G, d_err, st));
        int e = 0;
        SI_CK(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        if (total) *total = 0;
        if (e == sig::kDevBadContig) return fail(SI_ERR_INVALID, "a query names a contig outside [0, %d)", si->G);
        if (e != 0) return fail(SI_ERR_CUDA, "device error word %d", e);
        return SI_OK;
    }
    SI_CK(sig::launch_count_plain<S>(view<S>(si), q, counts, d_err, st));
    SI_CK(sig::exclusive_scan_u32_to_i64(counts, d_offsets, q.nq, scan_tmp, st));
    int64_t P = 0;
    SI_CK(cudaMemcpyAsync(&P, d_offsets + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (total) *total = (size_t)P;
    int e = 0;
    if ((size_t)P <= capacity) {
        SI_CK(sig::launch_emit_plain<S>(view<S>(si), q, d_offsets, 0, order, false, d_out, d_err, st));
    }
    SI_CK(cudaMemcpyAsync(&e, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (e == sig::kDevBadContig) return fail(SI_ERR_INVALID, "a query names a contig outside [0, %d)", si->G);
    if (e != 0) return fail(SI_ERR_CUDA, "device error word %d", e);
    if ((size_t)P > capacity) return fail(SI_ERR_CAPACITY, "output needs %lld values, capacity %zu", (long long)P, capacity);
    return SI_OK;
}

}  // namespace

extern "C" int searchIdxsNoAllocGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                                    const int32_t* d_qcontig, size_t nq, int order, int64_t* d_offsets,
                                    int32_t* d_values, size_t capacity, size_t* total, void* stream) {
    SI_TRY(check_built(si));
    if (order != SI_ORDER_IDXS_CPP && order != SI_ORDER_DESC) return fail(SI_ERR_INVALID, "unknown order");
    if (nq > kNoAllocMaxQueries)
        return fail(SI_ERR_TOO_LARGE, "the allocation-free search takes at most %zu queries per call, got %zu",
                    kNoAllocMaxQueries, nq);
    if (!d_offsets || (nq && (!d_qs || !d_qe))) return fail(SI_ERR_INVALID, "null device buffer");
    if (capacity > 0 && !d_values) return fail(SI_ERR_INVALID, "null value buffer with capacity %zu", capacity);
    SI_TRY(set_dev(si));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qcontig, (int64_t)nq};
    if (si->bits == 64) return search_noalloc<int64_t>(si, q, order, d_offsets, d_values, capacity, total, st);
    return search_noalloc<int32_t>(si, q, order, d_offsets, d_values, capacity, total, st);
}

namespace {
std::atomic<long long> g_launches{0};
}
namespace sig {
void note_launch(int n) { g_launches += n; }
}  // namespace sig

extern "C" long long getLaunchCountGpu(void) { return g_launches.load(); }

// =====================================================================================
// Autotuner for the batched path: times full searches (count -> scan -> emit) on a sample of
// the caller's own device-resident queries and keeps the fastest upper-bound provider, tile
// size, candidate capacity and length split, by coordinate descent from the current values.
// The chosen values stay set on the handle; `report` receives them as one JSON object.
// =====================================================================================
extern "C" int autotuneBatchedGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                  size_t nq, size_t sample, int flags, char* report, size_t report_len) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (!d_qs || !d_qe || nq == 0) return fail(SI_ERR_INVALID, "autotune needs a non-empty device query batch");
    const size_t ns = sample == 0 ? nq : std::min(nq, std::max<size_t>(sample, 4096));
    cudaStream_t st = si->st;
    const int saved_path = si->path;
    si->path = SI_PATH_BATCHED;
    DevBuf off, out;
    SI_TRY(off.reserve(sizeof(int64_t) * (ns + 1)));
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)ns};
    size_t P = 0;
    auto run = [&](int& status) -> double {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        double best = 1e30;
        for (int rep = 0; rep < 2; ++rep) {
            size_t t = 0;
            cudaEventRecord(a, st);
            status = si->bits == 64 ? search_device<int64_t>(si, q, SI_ORDER_IDXS_CPP, false, off.as<int64_t>(),
                                                              out.as<int32_t>(), out.bytes / 4, &t, st)
                                    : search_device<int32_t>(si, q, SI_ORDER_IDXS_CPP, false, off.as<int64_t>(),
                                                              out.as<int32_t>(), out.bytes / 4, &t, st);
            cudaEventRecord(b, st);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            if (status != SI_OK) break;
            best = std::min(best, (double)ms);
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        return best;
    };
    // size the output on the sample
    {
        size_t t = 0;
        int r = si->bits == 64 ? search_device<int64_t>(si, q, SI_ORDER_IDXS_CPP, false, off.as<int64_t>(), nullptr, 0,
                                                        &t, st)
                               : search_device<int32_t>(si, q, SI_ORDER_IDXS_CPP, false, off.as<int64_t>(), nullptr, 0,
                                                        &t, st);
        if (r != SI_OK && r != SI_ERR_CAPACITY) {
            si->path = saved_path;
            return r;
        }
        P = t;
        int rr = out.reserve(sizeof(int32_t) * std::max<size_t>(P, 1));
        if (rr != SI_OK) {
            si->path = saved_path;
            return rr;
        }
    }
    sig::BatchedParams best = si->bws.prm;
    int best_ub = si->ub_mode;
    int status = SI_OK;
    double best_ms = run(status);
    if (status != SI_OK) {
        si->path = saved_path;
        return status;
    }
    int trials = 1;
    // set parameters and provider; the provider's structure is rebuilt when the provider or the
    // Eytzinger depth changes
    auto apply = [&](const sig::BatchedParams& p, int ub) -> bool {
        const bool rebuild = ub != si->ub_mode || (ub == SI_UB_EYTZINGER && p.eytz_depth != si->bws.prm.eytz_depth);
        si->bws.prm = p;
        return !rebuild || setUpperBoundModeGpu(si, ub) == SI_OK;
    };
    auto try_params = [&](const sig::BatchedParams& p, int ub) {
        const sig::BatchedParams keep = si->bws.prm;
        const int keep_ub = si->ub_mode;
        if (!apply(p, ub)) {
            apply(keep, keep_ub);
            return;
        }
        int s = SI_OK;
        const double ms = run(s);
        ++trials;
        // a trial replaces the current choice only when 2% faster, so that timing noise does
        // not trade a good setting for one that measured better once
        if (s == SI_OK && ms < 0.98 * best_ms) {
            best_ms = ms;
            best = p;
            best_ub = ub;
        } else {
            apply(keep, keep_ub);
        }
    };
    if (!(flags & SI_TUNE_KEEP_UPPER_BOUND))
        for (int ub : {SI_UB_BINARY, SI_UB_EYTZINGER, SI_UB_LEARNED})
            if (ub != best_ub) try_params(best, ub);
    for (int t : {128, 256, 384, 512})
        if (t != best.tile_q || best.auto_tile) {
            sig::BatchedParams p = best;
            p.tile_q = t;
            p.auto_tile = false;
            try_params(p, best_ub);
        }
    for (int c : {1024, 2048, 3072})
        if (c != best.cap) {
            sig::BatchedParams p = best;
            p.cap = c;
            try_params(p, best_ub);
        }
    for (int64_t x : {(int64_t)512, (int64_t)2048, (int64_t)8192})
        if (x != best.split_len) {
            sig::BatchedParams p = best;
            p.split_len = x;
            try_params(p, best_ub);
        }
    {  // how the emit writes the long-interval list's section of part B
        sig::BatchedParams p = best;
        p.emit_copy = !best.emit_copy;
        try_params(p, best_ub);
    }
    if (best_ub == SI_UB_EYTZINGER)  // depth of the Eytzinger tree (the shared-memory top levels)
        for (int dpt : {7, 10, 13})
            if (dpt != si->bws.ub.eytz_depth) {
                sig::BatchedParams p = best;
                p.eytz_depth = dpt;
                try_params(p, best_ub);
            }
    if (!apply(best, best_ub)) return fail(SI_ERR_CUDA, "autotune: restoring the chosen provider failed");
    si->path = saved_path;
    if (report && report_len) {
        snprintf(report, report_len,
                 "{\"upper_bound\": %d, \"tile_queries\": %d, \"tile_auto\": %d, \"tile_candidates\": %d, "
                 "\"split_len\": %lld, \"long_query_len\": %lld, \"emit_copy\": %d, \"eytz_depth\": %d, "
                 "\"sample_queries\": %zu, \"sample_ms\": %.4f, \"trials\": %d}",
                 best_ub, best.tile_q, best.auto_tile ? 1 : 0, best.cap, (long long)best.split_len,
                 (long long)best.long_len, best.emit_copy ? 1 : 0, best.eytz_depth, ns, best_ms, trials);
    }
    return SI_OK;
}

// =====================================================================================
// Graph-replayed search: the plain path's count -> scan -> emit captured once per call
// shape (buffers, size, order, capacity, stream) as a CUDA graph and replayed afterwards, so
// that repeated small batches (a serving loop) pay one graph launch instead of several kernel
// launches.  The emit kernel never writes past `capacity`; a larger result is reported with
// SI_ERR_CAPACITY and the required size.  The index must not be rebuilt between calls with the
// same shape (a rebuild drops the captured graph).
// =====================================================================================
namespace {

template <typename S>
int capture_plain(gSuperIntervals* si, const sig::QueryBatch& q, int order, int64_t* d_offsets, int32_t* d_values,
                  size_t capacity, cudaStream_t st) {
    cudaGraph_t graph = nullptr;
    const long long k0 = g_launches.load();
    SI_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st);
    if (e == cudaSuccess) e = sig::launch_count_plain<S>(view<S>(si), q, si->w_counts.as<uint32_t>(), si->w_err.as<int>(), st);
    if (e == cudaSuccess)
        e = sig::exclusive_scan_u32_to_i64(si->w_counts.as<uint32_t>(), d_offsets, q.nq, si->w_tmp.p, st, si->w_err.as<int>());
    if (e == cudaSuccess)
        e = sig::launch_emit_plain<S>(view<S>(si), q, d_offsets, 0, order, false, d_values, si->w_err.as<int>(), st,
                                      (int64_t)capacity);
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    si->g_kernels = g_launches.load() - k0;
    g_launches -= si->g_kernels;  // counted when the graph runs, not when it is recorded
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        return fail(SI_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    if (si->gexec) cudaGraphExecDestroy(si->gexec);
    si->gexec = nullptr;
    e = cudaGraphInstantiate(&si->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        si->gexec = nullptr;
        return fail(SI_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    return SI_OK;
}

// The batched path (prepare -> count -> scan -> emit) captured once per call shape: int32
// coordinates and at most 85 contigs, so that the query key packs into 24 bits with the
// packing worked out on the device.  One eager search first sizes every workspace buffer
// (nothing may be allocated while the capture is open).
template <typename S>
int capture_batched(gSuperIntervals* si, const sig::QueryBatch& q, int order, int64_t* d_offsets, int32_t* d_values,
                    size_t capacity, cudaStream_t st) {
    size_t tot = 0;
    const int r0 = search_device<S>(si, q, order, false, d_offsets, d_values, capacity, &tot, st);
    if (r0 != SI_OK && r0 != SI_ERR_CAPACITY) return r0;
    sig::BatchedWorkspace& ws = si->bws;
    const int64_t nq = q.nq;
    SI_TRY(ws.qpair.reserve(2 * sizeof(S) * nq));
    SI_TRY(ws.kw[0].reserve(sizeof(uint32_t) * nq));
    SI_TRY(ws.kalt[0].reserve(sizeof(uint32_t) * nq));
    SI_TRY(ws.sort_tmp.reserve(sig::radix_temp_bytes(nq, 1)));
    SI_TRY(ws.qpack.reserve(2 * sizeof(int)));
    const bool prof = si->prof;
    si->prof = false;  // the phase timers synchronize: none inside the capture
    cudaGraph_t graph = nullptr;
    const long long k0 = g_launches.load();
    SI_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    ws.capturing = true;
    ws.out_cap = (int64_t)capacity;
    int r = run_count<S>(si, q, si->w_counts.as<uint32_t>(), st, true);
    cudaError_t e = cudaSuccess;
    if (r == SI_OK)
        e = sig::exclusive_scan_u32_to_i64(si->w_counts.as<uint32_t>(), d_offsets, nq, si->w_tmp.p, st, si->w_err.as<int>());
    if (r == SI_OK && e == cudaSuccess)
        r = run_emit<S>(si, q, 0, d_offsets, 0, order, false, d_values, st, (int64_t)tot);
    ws.capturing = false;
    ws.out_cap = INT64_MAX;
    si->prof = prof;
    cudaError_t e2 = cudaStreamEndCapture(st, &graph);
    si->g_kernels = g_launches.load() - k0;
    g_launches -= si->g_kernels;  // counted when the graph runs, not when it is recorded
    if (r != SI_OK || e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (r != SI_OK) return r;
        return fail(SI_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    if (si->gexec) cudaGraphExecDestroy(si->gexec);
    si->gexec = nullptr;
    e = cudaGraphInstantiate(&si->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        si->gexec = nullptr;
        return fail(SI_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(e));
    }
    return SI_OK;
}

}  // namespace

extern "C" int searchDeviceGraphGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                    size_t nq, int order, int64_t* d_offsets, int32_t* d_values, size_t capacity,
                                    size_t* total, void* stream) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (order != SI_ORDER_IDXS_CPP && order != SI_ORDER_DESC) return fail(SI_ERR_INVALID, "unknown order");
    if (!d_offsets || (nq && (!d_qs || !d_qe))) return fail(SI_ERR_INVALID, "null device buffer");
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    if (si->n == 0 || nq == 0) {
        SI_CK(cudaMemsetAsync(d_offsets, 0, sizeof(int64_t) * (nq + 1), st));
        SI_CK(cudaStreamSynchronize(st));
        if (total) *total = 0;
        return SI_OK;
    }
    // workspace first: nothing may be allocated while a capture is open
    SI_TRY(si->w_err.reserve(sizeof(int)));
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * nq));
    SI_TRY(si->w_tmp.reserve(sig::scan_temp_bytes((int64_t)nq)));
    // batched when the handle would take it for this batch and the key packs on the device
    const bool batched = use_batched(si, (int64_t)nq, true) && si->bits == 32 && sig::query_code_bits(si->G) <= 8 &&
                         nq < (size_t)INT32_MAX;
    const void* key[8] = {d_qs, d_qe, d_qc, d_offsets, d_values, (const void*)st, si->w_counts.p, si->w_tmp.p};
    const size_t key_n[5] = {nq, capacity, (size_t)order, (size_t)batched, (size_t)g_alloc_gen.load()};
    bool same = si->gexec != nullptr;
    for (int k = 0; k < 8 && same; ++k) same = key[k] == si->gkey[k];
    for (int k = 0; k < 5 && same; ++k) same = key_n[k] == si->gkey_n[k];
    if (!same) {
        sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
        int r;
        if (batched) r = capture_batched<int32_t>(si, q, order, d_offsets, d_values, capacity, st);
        else if (si->bits == 64) r = capture_plain<int64_t>(si, q, order, d_offsets, d_values, capacity, st);
        else r = capture_plain<int32_t>(si, q, order, d_offsets, d_values, capacity, st);
        if (r != SI_OK) return r;
        // every buffer the graph uses is sized now: key it on the allocations as they stand
        si->gkey_n[4] = (size_t)g_alloc_gen.load();
        for (int k = 0; k < 8; ++k) si->gkey[k] = key[k];
        for (int k = 0; k < 4; ++k) si->gkey_n[k] = key_n[k];
        si->gkey[6] = si->w_counts.p;
        si->gkey[7] = si->w_tmp.p;
    }
    SI_CK(cudaGraphLaunch(si->gexec, st));
    int64_t P = 0;
    int e = 0;
    SI_CK(cudaMemcpyAsync(&P, d_offsets + nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(&e, si->w_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (total) *total = (size_t)P;
    if ((size_t)P > capacity) return fail(SI_ERR_CAPACITY, "output needs %lld values, capacity %zu", (long long)P, capacity);
    if (e == sig::kDevBadContig) return fail(SI_ERR_INVALID, "a query names a contig outside [0, %d)", si->G);
    if (e != 0) return fail(SI_ERR_CUDA, "device error word %d", e);
    sig::note_launch((int)si->g_kernels);
    return SI_OK;
}

// =====================================================================================
// Set operations: intersection / difference of a list of intervals (map A, passed as queries)
// against the index (map B).  The hit lists come from the search path (count -> scan -> emit);
// the pieces from a second count -> scan -> emit over those lists (si_setops.cu).
// =====================================================================================
namespace {

// Hit lists of a device-resident batch into so_hoff / so_hits (contig-local positions).
template <typename S>
int hit_lists(gSuperIntervals* si, const sig::QueryBatch& q, int order, cudaStream_t st) {
    SI_TRY(si->so_hoff.reserve(sizeof(int64_t) * (q.nq + 1)));
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * std::max<int64_t>(q.nq, 1)));
    SI_TRY(si->w_tmp.reserve(sig::scan_temp_bytes(q.nq)));
    SI_TRY(run_count<S>(si, q, si->w_counts.as<uint32_t>(), st, true));
    SI_CK(sig::exclusive_scan_u32_to_i64(si->w_counts.as<uint32_t>(), si->so_hoff.as<int64_t>(), q.nq, si->w_tmp.p,
                                         st, si->w_err.as<int>()));
    int64_t P = 0;
    SI_CK(cudaMemcpyAsync(&P, si->so_hoff.as<int64_t>() + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    SI_TRY(si->so_hits.reserve(sizeof(int32_t) * std::max<int64_t>(P, 1)));
    SI_TRY(run_emit<S>(si, q, 0, si->so_hoff.as<int64_t>(), 0, order, false, si->so_hits.as<int32_t>(), st, P));
    return read_dev_err(si, st);
}

// op 0: intersection (order = the hit order), op 1: difference.  Pieces go to caller device
// buffers when they hold `cap` pieces; `total` always receives the piece count.
template <typename S>
int setop_device(gSuperIntervals* si, const sig::QueryBatch& q, int op, int order, int64_t* d_off, S* d_os,
                 S* d_oe, int32_t* d_ob, size_t cap, size_t* total, cudaStream_t st) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (!d_off || (q.nq && (!q.qs || !q.qe))) return fail(SI_ERR_INVALID, "null device buffer");
    if (total) *total = 0;
    if (q.nq == 0) {
        SI_CK(cudaMemsetAsync(d_off, 0, sizeof(int64_t), st));
        SI_CK(cudaStreamSynchronize(st));
        return SI_OK;
    }
    SI_TRY(si->w_err.reserve(sizeof(int)));
    if (si->n > 0) {
        SI_TRY(hit_lists<S>(si, q, op == 0 ? order : SI_ORDER_DESC, st));
    } else {
        SI_TRY(si->so_hoff.reserve(sizeof(int64_t) * (q.nq + 1)));
        SI_TRY(si->so_hits.reserve(sizeof(int32_t)));
        SI_CK(cudaMemsetAsync(si->so_hoff.p, 0, sizeof(int64_t) * (q.nq + 1), st));
        SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st));
    }
    bool sequential = false;
    if (si->n > 0 && si->inverted < 0) {  // does some interval have start > end (once per build)
        SI_TRY(si->so_flag.reserve(2 * sizeof(int)));
        SI_CK(sig::launch_any_inverted<S>(view<S>(si), si->so_flag.as<int>(), st));
        int f = 0;
        SI_CK(cudaMemcpyAsync(&f, si->so_flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        si->inverted = f ? 1 : 0;
    }
    if (op == 1) sequential = si->inverted == 1;
    const int64_t* hoff = si->so_hoff.as<int64_t>();
    const int32_t* hits = si->so_hits.as<int32_t>();
    sig::MapView<S> rv;
    SI_TRY(view_rec<S>(si, st, &rv));
    if (op == 0 && si->inverted == 0) {
        // with start <= end for every interval and every query, each hit gives one piece:
        // the pieces' offsets are the hits' offsets and no counting pass is needed
        SI_TRY(si->so_flag.reserve(2 * sizeof(int)));
        sig::MapView<S> qv = view<S>(si);
        qv.starts = static_cast<const S*>(q.qs);
        qv.ends = static_cast<const S*>(q.qe);
        qv.n = q.nq;
        SI_CK(sig::launch_any_inverted<S>(qv, si->so_flag.as<int>() + 1, st));
        int qinv = 0;
        int64_t P = 0;
        SI_CK(cudaMemcpyAsync(&qinv, si->so_flag.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaMemcpyAsync(&P, hoff + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        if (!qinv) {
            SI_CK(cudaMemcpyAsync(d_off, hoff, sizeof(int64_t) * (q.nq + 1), cudaMemcpyDeviceToDevice, st));
            if (total) *total = (size_t)P;
            if ((size_t)P > cap) {
                SI_CK(cudaStreamSynchronize(st));
                return fail(SI_ERR_CAPACITY, "output needs %lld pieces, capacity %zu", (long long)P, cap);
            }
            if (P > 0 && (!d_os || !d_oe || !d_ob)) return fail(SI_ERR_INVALID, "null output buffer");
            if (P > 0)
                SI_CK(sig::launch_isect<S>(rv, q, hoff, hits, nullptr, d_off, d_os, d_oe, d_ob,
                                           si->w_err.as<int>(), st));
            return read_dev_err(si, st);
        }
    }
    SI_TRY(si->w_counts.reserve(sizeof(uint32_t) * q.nq));
    SI_TRY(si->w_tmp.reserve(sig::scan_temp_bytes(q.nq)));
    uint32_t* cnt = si->w_counts.as<uint32_t>();
    if (op == 0)
        SI_CK(sig::launch_isect<S>(rv, q, hoff, hits, cnt, nullptr, nullptr, nullptr, nullptr, si->w_err.as<int>(), st));
    else
        SI_CK(sig::launch_diff<S>(rv, q, hoff, hits, sequential, cnt, nullptr, nullptr, nullptr, si->w_err.as<int>(), st));
    SI_CK(sig::exclusive_scan_u32_to_i64(cnt, d_off, q.nq, si->w_tmp.p, st, si->w_err.as<int>()));
    int64_t T = 0;
    SI_CK(cudaMemcpyAsync(&T, d_off + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_TRY(read_dev_err(si, st));  // synchronizes
    if (total) *total = (size_t)T;
    if ((size_t)T > cap) return fail(SI_ERR_CAPACITY, "output needs %lld pieces, capacity %zu", (long long)T, cap);
    if (T > 0 && (!d_os || !d_oe || (op == 0 && !d_ob))) return fail(SI_ERR_INVALID, "null output buffer");
    if (T > 0) {
        if (op == 0)
            SI_CK(sig::launch_isect<S>(rv, q, hoff, hits, nullptr, d_off, d_os, d_oe, d_ob, si->w_err.as<int>(), st));
        else
            SI_CK(sig::launch_diff<S>(rv, q, hoff, hits, sequential, nullptr, d_off, d_os, d_oe, si->w_err.as<int>(), st));
    }
    return read_dev_err(si, st);
}

template <typename S>
int setop_host(gSuperIntervals* si, const S* qs, const S* qe, const int32_t* qc, size_t nq, int op, int order,
               int64_t* h_off, S* h_os, S* h_oe, int32_t* h_ob, size_t cap, size_t* total) {
    SI_TRY(check_width<S>(si));
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (!h_off) return fail(SI_ERR_INVALID, "null offsets");
    sig::QueryBatch q;
    SI_TRY(upload_queries<S>(si, qs, qe, qc, nq, q));
    SI_TRY(si->so_off.reserve(sizeof(int64_t) * (nq + 1)));
    size_t T = 0;
    int r = setop_device<S>(si, q, op, order, si->so_off.as<int64_t>(), nullptr, nullptr, nullptr, 0, &T, si->st);
    if (r != SI_OK && r != SI_ERR_CAPACITY) return r;
    if (total) *total = T;
    SI_CK(cudaMemcpyAsync(h_off, si->so_off.p, sizeof(int64_t) * (nq + 1), cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    if (T > cap) return fail(SI_ERR_CAPACITY, "output needs %zu pieces, capacity %zu", T, cap);
    if (T == 0) return SI_OK;
    SI_TRY(si->so_os.reserve(sizeof(S) * T));
    SI_TRY(si->so_oe.reserve(sizeof(S) * T));
    if (op == 0) SI_TRY(si->so_ob.reserve(sizeof(int32_t) * T));
    // the hit lists are still in place: emit the pieces only
    const int64_t* hoff = si->so_hoff.as<int64_t>();
    const int32_t* hits = si->so_hits.as<int32_t>();
    sig::MapView<S> rv;
    SI_TRY(view_rec<S>(si, si->st, &rv));
    if (op == 0)
        SI_CK(sig::launch_isect<S>(rv, q, hoff, hits, nullptr, si->so_off.as<int64_t>(), si->so_os.as<S>(),
                                   si->so_oe.as<S>(), si->so_ob.as<int32_t>(), si->w_err.as<int>(), si->st));
    else
        SI_CK(sig::launch_diff<S>(rv, q, hoff, hits, si->inverted == 1, nullptr, si->so_off.as<int64_t>(),
                                  si->so_os.as<S>(), si->so_oe.as<S>(), si->w_err.as<int>(), si->st));
    if (!h_os || !h_oe || (op == 0 && !h_ob)) return fail(SI_ERR_INVALID, "null output buffer");
    SI_CK(cudaMemcpyAsync(h_os, si->so_os.p, sizeof(S) * T, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaMemcpyAsync(h_oe, si->so_oe.p, sizeof(S) * T, cudaMemcpyDeviceToHost, si->st));
    if (op == 0) SI_CK(cudaMemcpyAsync(h_ob, si->so_ob.p, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    return SI_OK;
}

int check_order(int order) {
    if (order != SI_ORDER_IDXS_CPP && order != SI_ORDER_DESC) return fail(SI_ERR_INVALID, "unknown order %d", order);
    return SI_OK;
}

}  // namespace

extern "C" int intersectDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                  size_t nq, int order, int64_t* d_offsets, void* d_starts, void* d_ends,
                                  int32_t* d_hits, size_t capacity, size_t* total, void* stream) {
    SI_TRY(check_built(si));
    SI_TRY(check_order(order));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64)
        return setop_device<int64_t>(si, q, 0, order, d_offsets, (int64_t*)d_starts, (int64_t*)d_ends, d_hits,
                                     capacity, total, st);
    return setop_device<int32_t>(si, q, 0, order, d_offsets, (int32_t*)d_starts, (int32_t*)d_ends, d_hits,
                                 capacity, total, st);
}

extern "C" int differenceDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                   size_t nq, int64_t* d_offsets, void* d_starts, void* d_ends, size_t capacity,
                                   size_t* total, void* stream) {
    SI_TRY(check_built(si));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64)
        return setop_device<int64_t>(si, q, 1, 0, d_offsets, (int64_t*)d_starts, (int64_t*)d_ends, nullptr, capacity,
                                     total, st);
    return setop_device<int32_t>(si, q, 1, 0, d_offsets, (int32_t*)d_starts, (int32_t*)d_ends, nullptr, capacity,
                                 total, st);
}

extern "C" int intersectBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qc, size_t nq,
                                 int order, int64_t* offsets, void* starts, void* ends, int32_t* hits,
                                 size_t capacity, size_t* total) {
    SI_TRY(check_built(si));
    SI_TRY(check_order(order));
    if (si->bits == 64)
        return setop_host<int64_t>(si, (const int64_t*)qs, (const int64_t*)qe, qc, nq, 0, order, offsets,
                                   (int64_t*)starts, (int64_t*)ends, hits, capacity, total);
    return setop_host<int32_t>(si, (const int32_t*)qs, (const int32_t*)qe, qc, nq, 0, order, offsets,
                               (int32_t*)starts, (int32_t*)ends, hits, capacity, total);
}

extern "C" int differenceBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qc, size_t nq,
                                  int64_t* offsets, void* starts, void* ends, size_t capacity, size_t* total) {
    SI_TRY(check_built(si));
    if (si->bits == 64)
        return setop_host<int64_t>(si, (const int64_t*)qs, (const int64_t*)qe, qc, nq, 1, 0, offsets,
                                   (int64_t*)starts, (int64_t*)ends, nullptr, capacity, total);
    return setop_host<int32_t>(si, (const int32_t*)qs, (const int32_t*)qe, qc, nq, 1, 0, offsets,
                               (int32_t*)starts, (int32_t*)ends, nullptr, capacity, total);
}

// =====================================================================================
// Key gathers and coverage over the hit lists.
// =====================================================================================
namespace {

// Hit lists of a device batch (so_hoff / so_hits); an empty index gives empty lists.
template <typename S>
int lists_or_empty(gSuperIntervals* si, const sig::QueryBatch& q, int order, cudaStream_t st, int64_t* P) {
    SI_TRY(si->w_err.reserve(sizeof(int)));
    if (si->n > 0) {
        SI_TRY(hit_lists<S>(si, q, order, st));
        SI_CK(cudaMemcpyAsync(P, si->so_hoff.as<int64_t>() + q.nq, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
    } else {
        SI_TRY(si->so_hoff.reserve(sizeof(int64_t) * (q.nq + 1)));
        SI_TRY(si->so_hits.reserve(sizeof(int32_t)));
        SI_CK(cudaMemsetAsync(si->so_hoff.p, 0, sizeof(int64_t) * (q.nq + 1), st));
        SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st));
        SI_CK(sig::launch_check_contigs(q.qc, q.nq, si->G, si->w_err.as<int>(), st));
        SI_TRY(read_dev_err(si, st));
        *P = 0;
    }
    return SI_OK;
}

template <typename S>
int keys_device(gSuperIntervals* si, const sig::QueryBatch& q, int order, int64_t* d_off, S* d_s, S* d_e,
                int32_t* d_d, size_t cap, size_t* total, cudaStream_t st) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    SI_TRY(check_order(order));
    if (!d_off || (q.nq && (!q.qs || !q.qe))) return fail(SI_ERR_INVALID, "null device buffer");
    if (total) *total = 0;
    if (q.nq == 0) {
        SI_CK(cudaMemsetAsync(d_off, 0, sizeof(int64_t), st));
        SI_CK(cudaStreamSynchronize(st));
        return SI_OK;
    }
    int64_t P = 0;
    SI_TRY(lists_or_empty<S>(si, q, order, st, &P));
    SI_CK(cudaMemcpyAsync(d_off, si->so_hoff.p, sizeof(int64_t) * (q.nq + 1), cudaMemcpyDeviceToDevice, st));
    if (total) *total = (size_t)P;
    if ((size_t)P > cap) {
        SI_CK(cudaStreamSynchronize(st));
        return fail(SI_ERR_CAPACITY, "output needs %lld keys, capacity %zu", (long long)P, cap);
    }
    if (P > 0) {
        if (!d_s || !d_e) return fail(SI_ERR_INVALID, "null output buffer");
        sig::MapView<S> rv;
        SI_TRY(view_rec<S>(si, st, &rv));
        SI_CK(sig::launch_keys<S>(rv, q, si->so_hoff.as<int64_t>(), si->so_hits.as<int32_t>(), d_s, d_e,
                                  d_d, st));
    }
    SI_CK(cudaStreamSynchronize(st));
    SI_CK(cudaGetLastError());
    return SI_OK;
}

template <typename S>
int coverage_device(gSuperIntervals* si, const sig::QueryBatch& q, uint64_t* d_count, S* d_cov, cudaStream_t st) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (q.nq && (!q.qs || !q.qe || !d_count || !d_cov)) return fail(SI_ERR_INVALID, "null device buffer");
    if (q.nq == 0) return SI_OK;
    if (si->n > 0 && si->inverted == 0 && si->bws.end_sorted) {
        // no interval has start > end: when no query has start > end either, the coverage comes
        // from ranks and prefix sums, without hit lists
        sig::MapView<S> qv = view<S>(si);
        qv.starts = static_cast<const S*>(q.qs);
        qv.ends = static_cast<const S*>(q.qe);
        qv.n = q.nq;
        SI_TRY(si->so_flag.reserve(2 * sizeof(int)));
        SI_CK(sig::launch_any_inverted<S>(qv, si->so_flag.as<int>() + 1, st));
        int inv = 0;
        SI_CK(cudaMemcpyAsync(&inv, si->so_flag.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        if (!inv) {
            if (!si->cov_ready) {
                SI_TRY(si->ps_start.reserve(sizeof(uint64_t) * (si->n + 1)));
                SI_TRY(si->ps_end.reserve(sizeof(uint64_t) * (si->n + 1)));
                DevBuf tmp;
                SI_TRY(tmp.reserve(sig::scan_temp_bytes(si->n)));
                if (sizeof(S) == 4) {
                    SI_CK(sig::exclusive_scan_i32_to_u64((const int32_t*)si->starts.p, si->ps_start.as<uint64_t>(),
                                                         si->n, tmp.p, st));
                    SI_CK(sig::exclusive_scan_i32_to_u64((const int32_t*)si->end_sorted.p,
                                                         si->ps_end.as<uint64_t>(), si->n, tmp.p, st));
                } else {
                    SI_CK(sig::exclusive_scan_i64_to_u64((const int64_t*)si->starts.p, si->ps_start.as<uint64_t>(),
                                                         si->n, tmp.p, st));
                    SI_CK(sig::exclusive_scan_i64_to_u64((const int64_t*)si->end_sorted.p,
                                                         si->ps_end.as<uint64_t>(), si->n, tmp.p, st));
                }
                SI_CK(cudaStreamSynchronize(st));  // tmp is released on scope exit
                si->cov_ready = true;
            }
            SI_TRY(si->w_err.reserve(sizeof(int)));
            SI_CK(cudaMemsetAsync(si->w_err.p, 0, sizeof(int), st));
            const int r = sig::batched_coverage<S>(si->bws, view<S>(si), q, si->ps_start.as<uint64_t>(),
                                                   si->ps_end.as<uint64_t>(), d_count, d_cov, si->w_err.as<int>(),
                                                   si->ub_mode, st);
            if (r != SI_OK) return fail(r, "coverage from ranks failed (status %d)", r);
            return read_dev_err(si, st);
        }
    }
    int64_t P = 0;
    SI_TRY(lists_or_empty<S>(si, q, SI_ORDER_DESC, st, &P));
    sig::MapView<S> rv;
    SI_TRY(view_rec<S>(si, st, &rv));
    SI_CK(sig::launch_coverage<S>(rv, q, si->so_hoff.as<int64_t>(), si->so_hits.as<int32_t>(), d_count,
                                  d_cov, st));
    SI_CK(cudaStreamSynchronize(st));
    SI_CK(cudaGetLastError());
    return SI_OK;
}

}  // namespace

extern "C" int searchKeysDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                   size_t nq, int order, int64_t* d_offsets, void* d_starts, void* d_ends,
                                   int32_t* d_data, size_t capacity, size_t* total, void* stream) {
    SI_TRY(check_built(si));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64)
        return keys_device<int64_t>(si, q, order, d_offsets, (int64_t*)d_starts, (int64_t*)d_ends, d_data, capacity,
                                    total, st);
    return keys_device<int32_t>(si, q, order, d_offsets, (int32_t*)d_starts, (int32_t*)d_ends, d_data, capacity,
                                total, st);
}

extern "C" int searchKeysBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qc, size_t nq,
                                  int order, int64_t* offsets, void* starts, void* ends, int32_t* data,
                                  size_t capacity, size_t* total) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (!offsets) return fail(SI_ERR_INVALID, "null offsets");
    const size_t sb = si->bits / 8;
    sig::QueryBatch q;
    int r = si->bits == 64 ? upload_queries<int64_t>(si, (const int64_t*)qs, (const int64_t*)qe, qc, nq, q)
                           : upload_queries<int32_t>(si, (const int32_t*)qs, (const int32_t*)qe, qc, nq, q);
    SI_TRY(r);
    SI_TRY(si->so_off.reserve(sizeof(int64_t) * (nq + 1)));
    size_t T = 0;
    r = si->bits == 64 ? keys_device<int64_t>(si, q, order, si->so_off.as<int64_t>(), nullptr, nullptr, nullptr, 0,
                                              &T, si->st)
                       : keys_device<int32_t>(si, q, order, si->so_off.as<int64_t>(), nullptr, nullptr, nullptr, 0,
                                              &T, si->st);
    if (r != SI_OK && r != SI_ERR_CAPACITY) return r;
    if (total) *total = T;
    SI_CK(cudaMemcpyAsync(offsets, si->so_off.p, sizeof(int64_t) * (nq + 1), cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    if (T > capacity) return fail(SI_ERR_CAPACITY, "output needs %zu keys, capacity %zu", T, capacity);
    if (T == 0) return SI_OK;
    if (!starts || !ends) return fail(SI_ERR_INVALID, "null output buffer");
    SI_TRY(si->so_os.reserve(sb * T));
    SI_TRY(si->so_oe.reserve(sb * T));
    if (data) SI_TRY(si->so_ob.reserve(sizeof(int32_t) * T));
    // the hit lists are still in place: gather only
    sig::MapView<int64_t> rv64;
    sig::MapView<int32_t> rv32;
    if (si->bits == 64) SI_TRY(view_rec<int64_t>(si, si->st, &rv64));
    else SI_TRY(view_rec<int32_t>(si, si->st, &rv32));
    if (si->bits == 64)
        SI_CK(sig::launch_keys<int64_t>(rv64, q, si->so_hoff.as<int64_t>(), si->so_hits.as<int32_t>(),
                                        si->so_os.as<int64_t>(), si->so_oe.as<int64_t>(),
                                        data ? si->so_ob.as<int32_t>() : nullptr, si->st));
    else
        SI_CK(sig::launch_keys<int32_t>(rv32, q, si->so_hoff.as<int64_t>(), si->so_hits.as<int32_t>(),
                                        si->so_os.as<int32_t>(), si->so_oe.as<int32_t>(),
                                        data ? si->so_ob.as<int32_t>() : nullptr, si->st));
    SI_CK(cudaMemcpyAsync(starts, si->so_os.p, sb * T, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaMemcpyAsync(ends, si->so_oe.p, sb * T, cudaMemcpyDeviceToHost, si->st));
    if (data) SI_CK(cudaMemcpyAsync(data, si->so_ob.p, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    return SI_OK;
}

extern "C" int coverageDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe, const int32_t* d_qc,
                                 size_t nq, uint64_t* d_count, void* d_cov, void* stream) {
    SI_TRY(check_built(si));
    cudaStream_t st = stream ? (cudaStream_t)stream : si->st;
    sig::QueryBatch q{d_qs, d_qe, d_qc, (int64_t)nq};
    if (si->bits == 64) return coverage_device<int64_t>(si, q, d_count, (int64_t*)d_cov, st);
    return coverage_device<int32_t>(si, q, d_count, (int32_t*)d_cov, st);
}

extern "C" int coverageBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qc, size_t nq,
                                uint64_t* count, void* cov) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    if (nq && (!count || !cov)) return fail(SI_ERR_INVALID, "null output");
    const size_t sb = si->bits / 8;
    sig::QueryBatch q;
    int r = si->bits == 64 ? upload_queries<int64_t>(si, (const int64_t*)qs, (const int64_t*)qe, qc, nq, q)
                           : upload_queries<int32_t>(si, (const int32_t*)qs, (const int32_t*)qe, qc, nq, q);
    SI_TRY(r);
    if (nq == 0) return SI_OK;
    SI_TRY(si->so_off.reserve(sizeof(uint64_t) * nq));
    SI_TRY(si->so_os.reserve(sb * nq));
    r = si->bits == 64 ? coverage_device<int64_t>(si, q, si->so_off.as<uint64_t>(), si->so_os.as<int64_t>(), si->st)
                       : coverage_device<int32_t>(si, q, si->so_off.as<uint64_t>(), si->so_os.as<int32_t>(), si->st);
    SI_TRY(r);
    SI_CK(cudaMemcpyAsync(count, si->so_off.p, sizeof(uint64_t) * nq, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaMemcpyAsync(cov, si->so_os.p, sb * nq, cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    return SI_OK;
}

// =====================================================================================
// Index image: the built index as one flat little-endian byte image -- header, contig
// offsets, the sorted starts / ends / payloads and the branch array -- the counterpart of the
// Rust crate's serde derive on IntervalMap (src/superintervals.rs:35-44).  Loading puts the
// image's (already sorted) intervals into staging and indexes them: the sortedness check
// skips the radix sort, the cheap passes (pyramid, branch, long-interval list, upper-bound
// model) run again, and the recomputed branch array must equal the stored one.
// =====================================================================================
namespace {

constexpr char kImageMagic[8] = {'S', 'I', 'G', 'P', 'U', 'I', 'X', '1'};
constexpr uint32_t kImageVersion = 1;

struct ImageHeader {
    char magic[8];
    uint32_t version;
    uint32_t coord_bits;
    uint64_t n;
    uint64_t n_contigs;
};

inline size_t pad8(size_t x) { return (x + 7) & ~(size_t)7; }

// header, seg[G+1], starts, ends, data, branch (each padded to 8 bytes), then the contig names:
// u64 count (0 or G), int64 offsets[count + 1], name bytes (padded to 8)
size_t image_bytes(int bits, uint64_t n, uint64_t G) {
    const size_t sb = (size_t)bits / 8;
    return sizeof(ImageHeader) + 8 * (G + 1) + 2 * pad8(sb * n) + 2 * pad8(4 * n) + 8;
}

size_t names_bytes(const std::vector<std::string>& names) {
    if (names.empty()) return 0;
    size_t b = 0;
    for (const auto& s : names) b += s.size();
    return 8 * (names.size() + 1) + pad8(b);
}

template <typename S>
int deserialize_impl(gSuperIntervals* si, const ImageHeader& h, const unsigned char* p, const unsigned char* end) {
    const uint64_t n = h.n, G = h.n_contigs;
    const int64_t* seg = reinterpret_cast<const int64_t*>(p);
    p += 8 * (G + 1);
    if (seg[0] != 0 || seg[G] != (int64_t)n) return fail(SI_ERR_INVALID, "index image: bad contig offsets");
    for (uint64_t g = 0; g < G; ++g)
        if (seg[g + 1] < seg[g]) return fail(SI_ERR_INVALID, "index image: contig offsets decrease");
    const S* st = reinterpret_cast<const S*>(p);
    p += pad8(sizeof(S) * n);
    const S* en = reinterpret_cast<const S*>(p);
    p += pad8(sizeof(S) * n);
    const int32_t* da = reinterpret_cast<const int32_t*>(p);
    p += pad8(4 * n);
    const int32_t* br = reinterpret_cast<const int32_t*>(p);
    p += pad8(4 * n);
    uint64_t nn = 0;
    memcpy(&nn, p, 8);
    p += 8;
    std::vector<std::string> names;
    if (nn) {
        if (nn != G || (size_t)(end - p) < 8 * (nn + 1)) return fail(SI_ERR_INVALID, "index image: bad name table");
        std::vector<int64_t> at(nn + 1);
        memcpy(at.data(), p, 8 * (nn + 1));
        p += 8 * (nn + 1);
        if (at[0] != 0 || at[nn] < 0 || (size_t)(end - p) < (size_t)at[nn])
            return fail(SI_ERR_INVALID, "index image: bad name table");
        for (uint64_t c = 0; c < nn; ++c) {
            if (at[c + 1] < at[c]) return fail(SI_ERR_INVALID, "index image: bad name table");
            names.emplace_back(reinterpret_cast<const char*>(p) + at[c], (size_t)(at[c + 1] - at[c]));
        }
    }
    hs<S>(si).assign(st, st + n);
    he<S>(si).assign(en, en + n);
    si->hdata.assign(da, da + n);
    si->hseg.clear();
    if (G > 1) si->hseg.assign(seg, seg + G + 1);
    si->contig_names = names;
    si->built = false;
    SI_TRY(build_impl<S>(si));
    if (n == 0) return SI_OK;
    DevBuf tmp, flag;
    SI_TRY(tmp.reserve(4 * n));
    SI_TRY(flag.reserve(sizeof(int)));
    SI_CK(cudaMemcpyAsync(tmp.p, br, 4 * n, cudaMemcpyHostToDevice, si->st));
    SI_CK(sig::launch_differs_i32(tmp.as<int32_t>(), si->branch.as<int32_t>(), (int64_t)n, flag.as<int>(), si->st));
    int differs = 0;
    SI_CK(cudaMemcpyAsync(&differs, flag.p, sizeof(int), cudaMemcpyDeviceToHost, si->st));
    SI_CK(cudaStreamSynchronize(si->st));
    if (!si->input_was_sorted || differs) {
        si->built = false;
        return fail(SI_ERR_INVALID, "index image: intervals are not in index order or the branch array differs");
    }
    return SI_OK;
}

}  // namespace

extern "C" int serializeIndexGpu(const gSuperIntervals* si, void* buf, size_t cap, size_t* size) {
    SI_TRY(check_built(si));
    SI_TRY(set_dev(si));
    const uint64_t n = (uint64_t)si->n, G = (uint64_t)si->G;
    const std::vector<std::string>& names = si->contig_names.size() == G ? si->contig_names
                                                                          : std::vector<std::string>();
    const size_t need = image_bytes(si->bits, n, G) + names_bytes(names);
    if (size) *size = need;
    if (!buf || cap < need) return fail(SI_ERR_CAPACITY, "index image needs %zu bytes, capacity %zu", need, cap);
    unsigned char* p = static_cast<unsigned char*>(buf);
    memset(p, 0, need);
    ImageHeader h;
    memcpy(h.magic, kImageMagic, 8);
    h.version = kImageVersion;
    h.coord_bits = (uint32_t)si->bits;
    h.n = n;
    h.n_contigs = G;
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    std::vector<int64_t> segv = si->hseg;
    if (segv.empty()) segv = {0, (int64_t)n};
    memcpy(p, segv.data(), 8 * (G + 1));
    p += 8 * (G + 1);
    const size_t sb = (size_t)si->bits / 8;
    if (n) {
        SI_CK(cudaMemcpyAsync(p, si->starts.p, sb * n, cudaMemcpyDeviceToHost, si->st));
        p += pad8(sb * n);
        SI_CK(cudaMemcpyAsync(p, si->ends.p, sb * n, cudaMemcpyDeviceToHost, si->st));
        p += pad8(sb * n);
        SI_CK(cudaMemcpyAsync(p, si->data.p, 4 * n, cudaMemcpyDeviceToHost, si->st));
        p += pad8(4 * n);
        SI_CK(cudaMemcpyAsync(p, si->branch.p, 4 * n, cudaMemcpyDeviceToHost, si->st));
        p += pad8(4 * n);
    }
    const uint64_t nn = names.size();
    memcpy(p, &nn, 8);
    p += 8;
    if (nn) {
        int64_t at = 0;
        for (uint64_t c = 0; c <= nn; ++c) {
            memcpy(p + 8 * c, &at, 8);
            if (c < nn) at += (int64_t)names[c].size();
        }
        p += 8 * (nn + 1);
        for (const auto& s : names) {
            memcpy(p, s.data(), s.size());
            p += s.size();
        }
    }
    SI_CK(cudaStreamSynchronize(si->st));
    return SI_OK;
}

extern "C" int deserializeIndexGpu(gSuperIntervals* si, const void* buf, size_t len) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (!buf || len < sizeof(ImageHeader)) return fail(SI_ERR_INVALID, "index image too short");
    ImageHeader h;
    memcpy(&h, buf, sizeof(h));
    if (memcmp(h.magic, kImageMagic, 8) != 0) return fail(SI_ERR_INVALID, "not an index image");
    if (h.version != kImageVersion) return fail(SI_ERR_INVALID, "index image version %u unsupported", h.version);
    if ((int)h.coord_bits != si->bits)
        return fail(SI_ERR_INVALID, "index image has %u-bit coordinates, the handle %d-bit", h.coord_bits, si->bits);
    if (h.n >= ((uint64_t)1 << 31) || h.n_contigs < 1 || h.n_contigs > ((uint64_t)1 << 24))
        return fail(SI_ERR_INVALID, "index image sizes out of range");
    if (len < image_bytes(si->bits, h.n, h.n_contigs)) return fail(SI_ERR_INVALID, "index image truncated");
    SI_TRY(set_dev(si));
    const unsigned char* p = static_cast<const unsigned char*>(buf) + sizeof(h);
    const unsigned char* end = static_cast<const unsigned char*>(buf) + len;
    if (si->bits == 64) return deserialize_impl<int64_t>(si, h, p, end);
    return deserialize_impl<int32_t>(si, h, p, end);
}

extern "C" int saveIndexGpu(const gSuperIntervals* si, const char* path) {
    SI_TRY(check_built(si));
    if (!path) return fail(SI_ERR_INVALID, "null path");
    size_t need = 0;
    serializeIndexGpu(si, nullptr, 0, &need);
    std::vector<unsigned char> img(need);
    SI_TRY(serializeIndexGpu(si, img.data(), img.size(), &need));
    FILE* f = fopen(path, "wb");
    if (!f) return fail(SI_ERR_INVALID, "cannot open %s for writing", path);
    const size_t w = fwrite(img.data(), 1, img.size(), f);
    const int c = fclose(f);
    if (w != img.size() || c != 0) return fail(SI_ERR_INVALID, "writing %s failed", path);
    return SI_OK;
}

extern "C" int loadIndexGpu(gSuperIntervals* si, const char* path) {
    if (!si || !path) return fail(SI_ERR_INVALID, "null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(SI_ERR_INVALID, "cannot open %s", path);
    std::vector<unsigned char> img;
    unsigned char chunk[1 << 16];
    size_t r;
    while ((r = fread(chunk, 1, sizeof(chunk), f)) > 0) img.insert(img.end(), chunk, chunk + r);
    const bool bad = ferror(f) != 0;
    fclose(f);
    if (bad) return fail(SI_ERR_INVALID, "reading %s failed", path);
    return deserializeIndexGpu(si, img.data(), img.size());
}

// =====================================================================================
// BED ingest (examples/bed-intersect-si.rs:63-120, test/bench.cpp:67-102): the text is parsed
// on the GPU (si_bed.cu); the contig dictionary and the per-contig bucketing are radix sorts.
// =====================================================================================
namespace {

struct BedRecords {
    DevBuf text, nl, status, valid, hash, start, end, noff, nlen, voffs, tmp;
    DevBuf h_lo, h_hi, rec, r_start, r_end, r_noff, r_nlen, r_line;
    int64_t n_lines = 0, m = 0;
};

uint64_t fnv1a64(const char* p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t k = 0; k < n; ++k) h = (h ^ (unsigned char)p[k]) * 1099511628211ull;
    return h;
}

// Parse the text into interval records (file order) on the device.
int bed_records(gSuperIntervals* si, const char* text, size_t len, int options, BedRecords& B, cBedStats* stats) {
    cudaStream_t st = si->st;
    const int64_t L = (int64_t)len;
    if (len && !text) return fail(SI_ERR_INVALID, "null text");
    SI_TRY(B.text.reserve(len + 16));
    if (len) SI_CK(cudaMemcpyAsync(B.text.p, text, len, cudaMemcpyHostToDevice, st));
    const int64_t chunks = sig::bed_chunks(L);
    DevBuf counts, offs;
    SI_TRY(counts.reserve(sizeof(uint32_t) * chunks));
    SI_TRY(offs.reserve(sizeof(int64_t) * (chunks + 1)));
    SI_TRY(B.tmp.reserve(sig::scan_temp_bytes(chunks)));
    const unsigned char* t = B.text.as<unsigned char>();
    SI_CK(sig::launch_nl_count(t, L, counts.as<uint32_t>(), st));
    SI_CK(sig::exclusive_scan_u32_to_i64(counts.as<uint32_t>(), offs.as<int64_t>(), chunks, B.tmp.p, st));
    int64_t n_nl = 0;
    SI_CK(cudaMemcpyAsync(&n_nl, offs.as<int64_t>() + chunks, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    SI_TRY(B.nl.reserve(sizeof(int64_t) * std::max<int64_t>(n_nl, 1)));
    if (n_nl) SI_CK(sig::launch_nl_write(t, L, offs.as<int64_t>(), B.nl.as<int64_t>(), st));
    const int64_t n = n_nl + ((len > 0 && text[len - 1] != '\n') ? 1 : 0);
    B.n_lines = n;
    const int64_t nn = std::max<int64_t>(n, 1);
    SI_TRY(B.status.reserve(nn));
    SI_TRY(B.valid.reserve(4 * nn));
    SI_TRY(B.hash.reserve(8 * nn));
    SI_TRY(B.start.reserve(8 * nn));
    SI_TRY(B.end.reserve(8 * nn));
    SI_TRY(B.noff.reserve(8 * nn));
    SI_TRY(B.nlen.reserve(4 * nn));
    const int64_t lo = si->bits == 64 ? INT64_MIN : INT32_MIN, hi = si->bits == 64 ? INT64_MAX : INT32_MAX;
    SI_CK(sig::launch_bed_parse(t, L, B.nl.as<int64_t>(), n_nl, n, (options & SI_BED_HALF_OPEN) ? 1 : 0, lo, hi,
                                B.status.as<uint8_t>(), B.valid.as<uint32_t>(), B.hash.as<uint64_t>(),
                                B.start.as<int64_t>(), B.end.as<int64_t>(), B.noff.as<int64_t>(),
                                B.nlen.as<int32_t>(), st));
    if (stats) {
        std::vector<uint8_t> hs_(n);
        if (n) SI_CK(cudaMemcpyAsync(hs_.data(), B.status.p, n, cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        size_t c[5] = {0, 0, 0, 0, 0};
        for (uint8_t v : hs_) ++c[v < 5 ? v : 2];
        stats->lines = (size_t)n;
        stats->intervals = c[0];
        stats->skipped_headers = c[1];
        stats->malformed = c[2];
        stats->filtered = c[3];
        stats->out_of_range = c[4];
        stats->unknown_contig = 0;
    }
    SI_TRY(B.voffs.reserve(sizeof(int64_t) * (n + 1)));
    SI_TRY(B.tmp.reserve(sig::scan_temp_bytes(nn)));
    SI_CK(sig::exclusive_scan_u32_to_i64(B.valid.as<uint32_t>(), B.voffs.as<int64_t>(), n, B.tmp.p, st));
    int64_t m = 0;
    SI_CK(cudaMemcpyAsync(&m, B.voffs.as<int64_t>() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (m >= ((int64_t)1 << 31) - 1) return fail(SI_ERR_TOO_LARGE, "%lld intervals exceed the position space", (long long)m);
    B.m = m;
    const int64_t mm = std::max<int64_t>(m, 1);
    SI_TRY(B.h_lo.reserve(4 * mm));
    SI_TRY(B.h_hi.reserve(4 * mm));
    SI_TRY(B.rec.reserve(4 * mm));
    SI_TRY(B.r_start.reserve(8 * mm));
    SI_TRY(B.r_end.reserve(8 * mm));
    SI_TRY(B.r_noff.reserve(8 * mm));
    SI_TRY(B.r_nlen.reserve(4 * mm));
    SI_TRY(B.r_line.reserve(8 * mm));
    SI_CK(sig::launch_bed_compact(B.valid.as<uint32_t>(), B.voffs.as<int64_t>(), n, B.hash.as<uint64_t>(),
                                  B.start.as<int64_t>(), B.end.as<int64_t>(), B.noff.as<int64_t>(),
                                  B.nlen.as<int32_t>(), B.h_lo.as<uint32_t>(), B.h_hi.as<uint32_t>(),
                                  B.rec.as<uint32_t>(), B.r_start.as<int64_t>(), B.r_end.as<int64_t>(),
                                  B.r_noff.as<int64_t>(), B.r_nlen.as<int32_t>(), B.r_line.as<int64_t>(), st));
    return SI_OK;
}

template <typename S>
int bed_ingest(gSuperIntervals* si, const char* text, size_t len, int options, cBedStats* stats) {
    cudaStream_t st = si->st;
    BedRecords B;
    SI_TRY(bed_records(si, text, len, options, B, stats));
    const int64_t m = B.m;
    hs<S>(si).clear();
    he<S>(si).clear();
    si->hdata.clear();
    si->hseg.clear();
    si->contig_names.clear();
    si->built = false;
    if (m == 0) return SI_OK;
    // 1. dictionary: sort records by name hash (stable: file order inside a hash group)
    DevBuf serr;  // the one-sweep sorts' error word (a bounded wait that gave up)
    SI_TRY(serr.reserve(sizeof(int)));
    SI_CK(cudaMemsetAsync(serr.p, 0, sizeof(int), st));
    DevBuf lo2, hi2, rec2, stmp;
    SI_TRY(lo2.reserve(4 * m));
    SI_TRY(hi2.reserve(4 * m));
    SI_TRY(rec2.reserve(4 * m));
    SI_TRY(stmp.reserve(sig::radix_temp_bytes(m, 2)));
    uint32_t* kp[2] = {B.h_lo.as<uint32_t>(), B.h_hi.as<uint32_t>()};
    uint32_t* ka[2] = {lo2.as<uint32_t>(), hi2.as<uint32_t>()};
    bool alt = false;
    SI_CK(sig::radix_sort(kp, ka, B.rec.as<uint32_t>(), rec2.as<uint32_t>(), 2, m, stmp.p, stmp.bytes, &alt, nullptr,
                          st, 0, serr.as<int>()));
    const uint32_t* slo = alt ? ka[0] : kp[0];
    const uint32_t* shi = alt ? ka[1] : kp[1];
    const uint32_t* perm = alt ? rec2.as<uint32_t>() : B.rec.as<uint32_t>();
    DevBuf head, ex, gid;
    SI_TRY(head.reserve(4 * m));
    SI_TRY(ex.reserve(4 * (m + 1)));
    SI_TRY(gid.reserve(4 * m));
    SI_TRY(B.tmp.reserve(sig::scan_temp_bytes(m)));
    SI_CK(sig::launch_hash_heads(slo, shi, m, head.as<uint32_t>(), st));
    SI_CK(sig::exclusive_scan_u32_to_u32(head.as<uint32_t>(), ex.as<uint32_t>(), m, B.tmp.p, st));
    uint32_t G32 = 0;
    SI_CK(cudaMemcpyAsync(&G32, ex.as<uint32_t>() + m, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    const int64_t G = G32;
    DevBuf first, gkey, coll;
    SI_TRY(first.reserve(4 * G));
    SI_TRY(gkey.reserve(4 * G));
    SI_TRY(coll.reserve(sizeof(int)));
    SI_CK(cudaMemsetAsync(coll.p, 0, sizeof(int), st));
    SI_CK(sig::launch_hash_groups(B.text.as<unsigned char>(), head.as<uint32_t>(), ex.as<uint32_t>(), perm, m,
                                  B.r_noff.as<int64_t>(), B.r_nlen.as<int32_t>(), gid.as<uint32_t>(),
                                  first.as<uint32_t>(), gkey.as<uint32_t>(), coll.as<int>(), st));
    int collision = 0;
    SI_CK(cudaMemcpyAsync(&collision, coll.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (collision) return fail(SI_ERR_INVALID, "two contig names share a 64-bit name hash");
    // 2. contig ids in order of first appearance
    DevBuf gk2, gp, gp2, gtmp;
    SI_TRY(gk2.reserve(4 * G));
    SI_TRY(gp.reserve(4 * G));
    SI_TRY(gp2.reserve(4 * G));
    SI_TRY(gtmp.reserve(sig::radix_temp_bytes(G, 1)));
    SI_CK(sig::launch_iota_u32(gp.as<uint32_t>(), G, st));
    uint32_t* gkp[1] = {gkey.as<uint32_t>()};
    uint32_t* gka[1] = {gk2.as<uint32_t>()};
    bool galt = false;
    SI_CK(sig::radix_sort(gkp, gka, gp.as<uint32_t>(), gp2.as<uint32_t>(), 1, G, gtmp.p, gtmp.bytes, &galt, nullptr,
                          st, 0, serr.as<int>()));
    const uint32_t* sorted_groups = galt ? gp2.as<uint32_t>() : gp.as<uint32_t>();
    // the sorted keys are each contig's first record, in contig order
    const uint32_t* first_rec = galt ? gka[0] : gkp[0];
    DevBuf rank, cid;
    SI_TRY(rank.reserve(4 * G));
    SI_TRY(cid.reserve(4 * m));
    SI_CK(sig::launch_record_contig(sorted_groups, G, rank.as<uint32_t>(), gid.as<uint32_t>(), perm, m,
                                    cid.as<uint32_t>(), st));
    // 3. per-contig buckets, file order inside a contig
    DevBuf cid2, ord, ord2, otmp;
    SI_TRY(cid2.reserve(4 * m));
    SI_TRY(ord.reserve(4 * m));
    SI_TRY(ord2.reserve(4 * m));
    SI_TRY(otmp.reserve(sig::radix_temp_bytes(m, 1)));
    SI_CK(sig::launch_iota_u32(ord.as<uint32_t>(), m, st));
    uint32_t* ckp[1] = {cid.as<uint32_t>()};
    uint32_t* cka[1] = {cid2.as<uint32_t>()};
    bool calt = false;
    SI_CK(sig::radix_sort(ckp, cka, ord.as<uint32_t>(), ord2.as<uint32_t>(), 1, m, otmp.p, otmp.bytes, &calt, nullptr,
                          st, 0, serr.as<int>()));
    {
        int se = 0;
        SI_CK(cudaMemcpyAsync(&se, serr.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        SI_CK(cudaStreamSynchronize(st));
        if (se != 0) return fail(SI_ERR_CUDA, "a bounded wait in the BED sorts gave up (device error word %d)", se);
    }
    const uint32_t* cid_sorted = calt ? cka[0] : ckp[0];
    const uint32_t* order = calt ? ord2.as<uint32_t>() : ord.as<uint32_t>();
    DevBuf os, oe, ol, seg, noff, nlen;
    SI_TRY(os.reserve(sizeof(S) * m));
    SI_TRY(oe.reserve(sizeof(S) * m));
    SI_TRY(ol.reserve(4 * m));
    SI_TRY(seg.reserve(8 * (G + 1)));
    SI_TRY(noff.reserve(8 * G));
    SI_TRY(nlen.reserve(4 * G));
    SI_CK(sig::launch_bed_out<S>(cid_sorted, order, m, B.r_start.as<int64_t>(), B.r_end.as<int64_t>(),
                                 B.r_line.as<int64_t>(), os.as<S>(), oe.as<S>(), ol.as<int32_t>(),
                                 seg.as<int64_t>(), st));
    SI_CK(sig::launch_contig_names(first_rec, B.r_noff.as<int64_t>(), B.r_nlen.as<int32_t>(), G, noff.as<int64_t>(),
                                   nlen.as<int32_t>(), st));
    hs<S>(si).resize(m);
    he<S>(si).resize(m);
    si->hdata.resize(m);
    std::vector<int64_t> segv(G + 1);
    std::vector<int64_t> hoff(G);
    std::vector<int32_t> hlen(G);
    SI_CK(cudaMemcpyAsync(hs<S>(si).data(), os.p, sizeof(S) * m, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(he<S>(si).data(), oe.p, sizeof(S) * m, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(si->hdata.data(), ol.p, 4 * m, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(segv.data(), seg.p, 8 * G, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(hoff.data(), noff.p, 8 * G, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(hlen.data(), nlen.p, 4 * G, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    segv[G] = m;
    if (G > 1) si->hseg = segv;
    si->contig_names.resize(G);
    for (int64_t c = 0; c < G; ++c) si->contig_names[c].assign(text + hoff[c], (size_t)hlen[c]);
    return SI_OK;
}

template <typename S>
int bed_queries(gSuperIntervals* si, const char* text, size_t len, int options, S* qs, S* qe, int32_t* qc,
                int64_t* line, size_t cap, size_t* n_out, cBedStats* stats) {
    cudaStream_t st = si->st;
    const int G = (int)si->contig_names.size();
    if (G == 0) return fail(SI_ERR_INVALID, "the handle has no contig names: ingest a BED file first");
    BedRecords B;
    SI_TRY(bed_records(si, text, len, options, B, stats));
    const int64_t m = B.m;
    if (n_out) *n_out = 0;
    // contig table: (hash, id) sorted by hash, and the names as one blob
    std::vector<std::pair<uint64_t, int32_t>> tab(G);
    std::vector<int64_t> at(G + 1, 0);
    std::string blob;
    for (int c = 0; c < G; ++c) {
        const std::string& nm = si->contig_names[c];
        tab[c] = {fnv1a64(nm.data(), nm.size()), c};
        at[c] = (int64_t)blob.size();
        blob += nm;
    }
    at[G] = (int64_t)blob.size();
    std::sort(tab.begin(), tab.end());
    for (int c = 1; c < G; ++c)
        if (tab[c].first == tab[c - 1].first) return fail(SI_ERR_INVALID, "two contig names share a 64-bit name hash");
    std::vector<uint64_t> th(G);
    std::vector<int32_t> tid(G);
    for (int c = 0; c < G; ++c) {
        th[c] = tab[c].first;
        tid[c] = tab[c].second;
    }
    DevBuf dh, did, dnames, dat, dqc, flag, offs;
    SI_TRY(dh.reserve(8 * G));
    SI_TRY(did.reserve(4 * G));
    SI_TRY(dnames.reserve(std::max<size_t>(blob.size(), 1)));
    SI_TRY(dat.reserve(8 * (G + 1)));
    SI_CK(cudaMemcpyAsync(dh.p, th.data(), 8 * G, cudaMemcpyHostToDevice, st));
    SI_CK(cudaMemcpyAsync(did.p, tid.data(), 4 * G, cudaMemcpyHostToDevice, st));
    if (!blob.empty()) SI_CK(cudaMemcpyAsync(dnames.p, blob.data(), blob.size(), cudaMemcpyHostToDevice, st));
    SI_CK(cudaMemcpyAsync(dat.p, at.data(), 8 * (G + 1), cudaMemcpyHostToDevice, st));
    const int64_t mm = std::max<int64_t>(m, 1);
    SI_TRY(dqc.reserve(4 * mm));
    SI_TRY(flag.reserve(4 * mm));
    SI_TRY(offs.reserve(8 * (m + 1)));
    SI_CK(sig::launch_bed_lookup(B.text.as<unsigned char>(), B.h_lo.as<uint32_t>(), B.h_hi.as<uint32_t>(),
                                 B.r_noff.as<int64_t>(), B.r_nlen.as<int32_t>(), m, dh.as<uint64_t>(),
                                 did.as<int32_t>(), G, dnames.as<unsigned char>(), dat.as<int64_t>(),
                                 dqc.as<int32_t>(), st));
    SI_CK(sig::launch_known(dqc.as<int32_t>(), m, flag.as<uint32_t>(), st));
    SI_TRY(B.tmp.reserve(sig::scan_temp_bytes(mm)));
    SI_CK(sig::exclusive_scan_u32_to_i64(flag.as<uint32_t>(), offs.as<int64_t>(), m, B.tmp.p, st));
    int64_t k = 0;
    SI_CK(cudaMemcpyAsync(&k, offs.as<int64_t>() + m, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    if (stats) stats->unknown_contig = (size_t)(m - k);
    if (n_out) *n_out = (size_t)k;
    if ((size_t)k > cap) return fail(SI_ERR_CAPACITY, "%lld queries, capacity %zu", (long long)k, cap);
    if (k == 0) return SI_OK;
    if (!qs || !qe || !qc) return fail(SI_ERR_INVALID, "null output buffer");
    DevBuf dqs, dqe, dqc2, dl;
    SI_TRY(dqs.reserve(sizeof(S) * k));
    SI_TRY(dqe.reserve(sizeof(S) * k));
    SI_TRY(dqc2.reserve(4 * k));
    SI_TRY(dl.reserve(8 * k));
    SI_CK(sig::launch_query_out<S>(dqc.as<int32_t>(), offs.as<int64_t>(), m, B.r_start.as<int64_t>(),
                                   B.r_end.as<int64_t>(), B.r_line.as<int64_t>(), dqs.as<S>(), dqe.as<S>(),
                                   dqc2.as<int32_t>(), dl.as<int64_t>(), st));
    SI_CK(cudaMemcpyAsync(qs, dqs.p, sizeof(S) * k, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(qe, dqe.p, sizeof(S) * k, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaMemcpyAsync(qc, dqc2.p, 4 * k, cudaMemcpyDeviceToHost, st));
    if (line) SI_CK(cudaMemcpyAsync(line, dl.p, 8 * k, cudaMemcpyDeviceToHost, st));
    SI_CK(cudaStreamSynchronize(st));
    return SI_OK;
}

}  // namespace

extern "C" int ingestBedGpu(gSuperIntervals* si, const char* text, size_t len, int options, cBedStats* stats) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    SI_TRY(set_dev(si));
    if (si->bits == 64) return bed_ingest<int64_t>(si, text, len, options, stats);
    return bed_ingest<int32_t>(si, text, len, options, stats);
}

extern "C" int bedQueriesGpu(gSuperIntervals* si, const char* text, size_t len, int options, void* qs, void* qe,
                             int32_t* qcontig, int64_t* line, size_t capacity, size_t* n, cBedStats* stats) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    SI_TRY(set_dev(si));
    if (si->bits == 64)
        return bed_queries<int64_t>(si, text, len, options, (int64_t*)qs, (int64_t*)qe, qcontig, line, capacity, n,
                                    stats);
    return bed_queries<int32_t>(si, text, len, options, (int32_t*)qs, (int32_t*)qe, qcontig, line, capacity, n,
                                stats);
}

extern "C" int contigNameGpu(const gSuperIntervals* si, size_t contig, char* buf, size_t cap, size_t* len) {
    if (!si) return fail(SI_ERR_INVALID, "null handle");
    if (contig >= si->contig_names.size())
        return fail(SI_ERR_INVALID, "contig %zu has no name (%zu named)", contig, si->contig_names.size());
    const std::string& nm = si->contig_names[contig];
    if (len) *len = nm.size();
    if (!buf || cap < nm.size() + 1) return fail(SI_ERR_CAPACITY, "name needs %zu bytes", nm.size() + 1);
    memcpy(buf, nm.data(), nm.size());
    buf[nm.size()] = 0;
    return SI_OK;
}
