// interval_map.hpp -- C++ drop-in for si::IntervalMap<S, T> (kcleal/superintervals,
// src/superintervals.hpp:46-1390, the build / query part), answered by the GPU through the
// C-ABI in c_api.h.
//
// Include this header instead of superintervals.hpp and link libsi_gpu.so.  Kept:
//   * the public members starts, ends, branch (size_t, SIZE_MAX = none), data,
//     start_sorted, end_sorted (hpp:49-61), filled by build();
//   * add (hpp:95-105), reserve, clear, size, build (hpp:112-130), at;
//   * count (hpp:651-825), has_overlaps (hpp:865-871), search_idxs (hpp:879-905, appends in the
//     C++ order), search_values (hpp:551-579, appends, descending), search_keys (hpp:913-938),
//     coverage (hpp:979-1006), upper_bound (hpp:501-516);
//   * batch forms modelled on the Cython ones (intervalmap.pyx:363-494): count_batch,
//     search_idxs_batch, search_values_batch, search_keys_batch (CSR: offsets + flat values) and
//     coverage_batch.
// S is int32_t or int64_t; T is any copyable payload, kept on the host and permuted with the
// intervals exactly as the reference permutes its data vector (stable order inside exact
// (start, end) duplicates, where the reference's std::sort order is unspecified).
// Queries before build() are undefined in the reference; here they throw.  Device failures
// throw std::runtime_error with the library's message.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "c_api.h"

namespace si {

template <typename S, typename T>
struct Interval {
    S start, end;
    T data;
    Interval() = default;
    Interval(S s, S e, T d) : start(s), end(e), data(d) {}
};

template <typename S, typename T>
class IntervalMap {
    static_assert(std::is_same<S, int32_t>::value || std::is_same<S, int64_t>::value,
                  "the GPU index takes int32_t or int64_t coordinates");

public:
    std::vector<S> starts;
    std::vector<S> ends;
    std::vector<size_t> branch;
    std::vector<T> data;
    bool start_sorted = true, end_sorted = true;

    explicit IntervalMap(int device = 0) : device_(device) {}
    IntervalMap(const IntervalMap&) = delete;
    IntervalMap& operator=(const IntervalMap&) = delete;
    virtual ~IntervalMap() { release(); }

    void clear() noexcept {
        data.clear();
        starts.clear();
        ends.clear();
        branch.clear();
        built_ = false;
    }
    void reserve(size_t n) {
        data.reserve(n);
        starts.reserve(n);
        ends.reserve(n);
    }
    size_t size() const { return starts.size(); }

    // hpp:95-105, including the sortedness flags the reference keeps
    void add(S start, S end, const T& value) {
        if (start_sorted && !starts.empty()) {
            start_sorted = !(start < starts.back());
            if (start_sorted && start == starts.back() && end > ends.back()) end_sorted = false;
        }
        starts.push_back(start);
        ends.push_back(end);
        data.push_back(value);
        built_ = false;
    }

    // hpp:112-130: sorts (start asc, end desc) and builds the branch array -- on the GPU
    virtual void build() {
        release();
        check(createSuperIntervalsGpu(&h_, sizeof(S) * 8, device_));
        const size_t n = starts.size();
        std::vector<int32_t> order(n);
        for (size_t i = 0; i < n; ++i) order[i] = (int32_t)i;
        if (n) {
            if (sizeof(S) == 4)
                check(addIntervalsGpu(h_, reinterpret_cast<const int32_t*>(starts.data()),
                                      reinterpret_cast<const int32_t*>(ends.data()), order.data(), n));
            else
                check(addIntervalsGpu_i64(h_, reinterpret_cast<const int64_t*>(starts.data()),
                                          reinterpret_cast<const int64_t*>(ends.data()), order.data(), n));
        }
        check(indexSuperIntervalsGpu(h_));
        std::vector<int64_t> br(n);
        std::vector<int32_t> perm(n);
        if (n) check(getIndexArraysGpu(h_, starts.data(), ends.data(), perm.data(), br.data()));
        std::vector<T> d2;
        d2.reserve(n);
        for (size_t i = 0; i < n; ++i) d2.push_back(data[(size_t)perm[i]]);
        data.swap(d2);
        branch.resize(n);
        for (size_t i = 0; i < n; ++i) branch[i] = br[i] < 0 ? SIZE_MAX : (size_t)br[i];
        start_sorted = end_sorted = true;
        built_ = true;
    }

    Interval<S, T> at(size_t index) const { return Interval<S, T>(starts[index], ends[index], data[index]); }

    // ---- single queries (the reference's per-query methods), as one-query batches ----------
    // count and has_overlaps are noexcept as in the reference (hpp:651, 865): a device failure
    // inside them ends the process through std::terminate instead of throwing.
    size_t count(S start, S end) const noexcept {
        if (starts.empty()) return 0;
        uint32_t c = 0;
        count_into(&start, &end, 1, &c);
        return c;
    }
    bool has_overlaps(S start, S end) const noexcept {
        if (starts.empty()) return false;
        uint8_t r = 0;
        need();
        if (sizeof(S) == 4)
            check(anyOverlapsBatchGpu(h_, reinterpret_cast<const int32_t*>(&start),
                                      reinterpret_cast<const int32_t*>(&end), nullptr, 1, &r));
        else
            check(anyOverlapsBatchGpu_i64(h_, reinterpret_cast<const int64_t*>(&start),
                                          reinterpret_cast<const int64_t*>(&end), nullptr, 1, &r));
        return r != 0;
    }
    void search_idxs(S start, S end, std::vector<size_t>& found) const {
        if (starts.empty()) return;
        std::vector<int64_t> off;
        std::vector<int32_t> val;
        search_into(&start, &end, 1, SI_ORDER_IDXS_CPP, off, val);
        for (int32_t v : val) found.push_back((size_t)v);
    }
    void search_values(S start, S end, std::vector<T>& found) const {
        if (starts.empty()) return;
        std::vector<int64_t> off;
        std::vector<int32_t> val;
        search_into(&start, &end, 1, SI_ORDER_DESC, off, val);
        for (int32_t v : val) found.push_back(data[(size_t)v]);
    }
    void search_keys(S start, S end, std::vector<std::pair<S, S>>& found) const {
        if (starts.empty()) return;
        std::vector<int64_t> off;
        std::vector<S> ks, ke;
        keys_into(&start, &end, 1, SI_ORDER_DESC, off, ks, ke);
        for (size_t k = 0; k < ks.size(); ++k) found.emplace_back(ks[k], ke[k]);
    }
    // hpp:979-1006: adds the number of overlaps and the sum of min(end) - max(start) (no +1)
    void coverage(S start, S end, std::pair<size_t, S>& cov_result) const {
        if (starts.empty()) return;
        uint64_t c = 0;
        S v = 0;
        need();
        check(coverageBatchGpu(h_, &start, &end, nullptr, 1, &c, &v));
        cov_result.first += (size_t)c;
        cov_result.second += v;
    }
    // hpp:501-516: last index with starts[idx] <= value, SIZE_MAX when none
    size_t upper_bound(S value) const {
        size_t length = starts.size(), idx = 0;
        if (!length) return SIZE_MAX;
        while (length > 1) {
            const size_t half = length / 2;
            idx += (starts[idx + half] <= value) * (length - half);
            length = half;
        }
        return starts[idx] > value ? idx - 1 : idx;
    }

    // ---- batch forms (intervalmap.pyx:363-494), one GPU pass per call ----------------------
    std::vector<uint32_t> count_batch(const S* qs, const S* qe, size_t nq) const {
        std::vector<uint32_t> out(nq, 0);
        if (!starts.empty() && nq) count_into(qs, qe, nq, out.data());
        return out;
    }
    // CSR: query i's indices are values[offsets[i] .. offsets[i+1]) in the C++ order
    void search_idxs_batch(const S* qs, const S* qe, size_t nq, std::vector<int64_t>& offsets,
                           std::vector<int32_t>& values) const {
        search_into(qs, qe, nq, SI_ORDER_IDXS_CPP, offsets, values);
    }
    // CSR of each hit's (start, end), in the order of search_keys (fully descending)
    void search_keys_batch(const S* qs, const S* qe, size_t nq, std::vector<int64_t>& offsets,
                           std::vector<S>& key_starts, std::vector<S>& key_ends) const {
        keys_into(qs, qe, nq, SI_ORDER_DESC, offsets, key_starts, key_ends);
    }
    // per query: number of overlaps and the sum of overlapping lengths (coverage, no +1)
    void coverage_batch(const S* qs, const S* qe, size_t nq, std::vector<uint64_t>& counts,
                        std::vector<S>& covered) const {
        counts.assign(nq, 0);
        covered.assign(nq, 0);
        if (starts.empty() || nq == 0) return;
        need();
        check(coverageBatchGpu(h_, qs, qe, nullptr, nq, counts.data(), covered.data()));
    }
    void search_values_batch(const S* qs, const S* qe, size_t nq, std::vector<int64_t>& offsets,
                             std::vector<T>& values) const {
        std::vector<int32_t> pos;
        search_into(qs, qe, nq, SI_ORDER_DESC, offsets, pos);
        values.clear();
        values.reserve(pos.size());
        for (int32_t p : pos) values.push_back(data[(size_t)p]);
    }

    gSuperIntervals* handle() const { return h_; }

private:
    int device_;
    gSuperIntervals* h_ = nullptr;
    bool built_ = false;

    static void check(int status) {
        if (status != SI_OK) throw std::runtime_error(std::string("superintervals GPU: ") + lastErrorGpu());
    }
    void need() const {
        if (!built_ || !h_) throw std::logic_error("IntervalMap: build() must be called before queries");
    }
    void release() {
        if (h_) destroySuperIntervalsGpu(h_);
        h_ = nullptr;
        built_ = false;
    }
    void count_into(const S* qs, const S* qe, size_t nq, uint32_t* out) const {
        need();
        if (sizeof(S) == 4)
            check(countOverlapsBatchGpu(h_, reinterpret_cast<const int32_t*>(qs),
                                        reinterpret_cast<const int32_t*>(qe), nullptr, nq, out));
        else
            check(countOverlapsBatchGpu_i64(h_, reinterpret_cast<const int64_t*>(qs),
                                            reinterpret_cast<const int64_t*>(qe), nullptr, nq, out));
    }
    void keys_into(const S* qs, const S* qe, size_t nq, int order, std::vector<int64_t>& offsets,
                   std::vector<S>& ks, std::vector<S>& ke) const {
        offsets.assign(nq + 1, 0);
        ks.clear();
        ke.clear();
        if (starts.empty() || nq == 0) return;
        need();
        size_t total = 0;
        int st = searchKeysBatchGpu(h_, qs, qe, nullptr, nq, order, offsets.data(), nullptr, nullptr, nullptr, 0,
                                    &total);
        if (st == SI_ERR_CAPACITY) {
            ks.resize(total);
            ke.resize(total);
            st = searchKeysBatchGpu(h_, qs, qe, nullptr, nq, order, offsets.data(), ks.data(), ke.data(), nullptr,
                                    total, &total);
        }
        check(st);
    }
    void search_into(const S* qs, const S* qe, size_t nq, int order, std::vector<int64_t>& offsets,
                     std::vector<int32_t>& values) const {
        offsets.assign(nq + 1, 0);
        values.clear();
        if (starts.empty() || nq == 0) return;
        need();
        size_t total = 0;
        int st = searchBatchIntoGpu(h_, qs, qe, nullptr, nq, order, 0, offsets.data(), nullptr, 0, &total);
        if (st == SI_ERR_CAPACITY) {
            values.resize(total);
            st = searchBatchIntoGpu(h_, qs, qe, nullptr, nq, order, 0, offsets.data(), values.data(), total,
                                    &total);
        }
        check(st);
    }
};

}  // namespace si
