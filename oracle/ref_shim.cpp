// ref_shim.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A thin extern "C" shim around the UNMODIFIED reference header
// src/superintervals.hpp (kcleal/superintervals).  The header is found by
// include path at build time (oracle/Makefile, REF_SRC); no reference source
// is copied into this repository.  The shared library built from this file
// (oracle/_ref/libsi_ref.so) is used only to produce the golden fixtures under
// tests/golden/ and to check the oracle restatement in oracle/si_oracle.c.
#include <cstdint>
#include <cstring>
#include <vector>
#include "superintervals.hpp"

namespace {

template <typename S>
struct RefMap {
    si::IntervalMap<S, int32_t> m;
};

template <typename S>
void* map_new(int64_t n, const S* s, const S* e, const int32_t* d) {
    auto* h = new RefMap<S>();
    h->m.reserve((size_t)n);
    for (int64_t i = 0; i < n; ++i) h->m.add(s[i], e[i], d ? d[i] : (int32_t)i);
    h->m.build();
    return h;
}

template <typename S>
void map_arrays(void* hp, S* s, S* e, int32_t* d, int64_t* br) {
    auto* h = static_cast<RefMap<S>*>(hp);
    size_t n = h->m.starts.size();
    for (size_t i = 0; i < n; ++i) {
        if (s) s[i] = h->m.starts[i];
        if (e) e[i] = h->m.ends[i];
        if (d) d[i] = h->m.data[i];
        if (br) br[i] = (h->m.branch[i] == SIZE_MAX) ? -1 : (int64_t)h->m.branch[i];
    }
}

// mode: 0 count, 1 count_linear, 2 count_large, 3 has_overlaps
template <typename S>
void map_scalar(void* hp, int mode, int64_t nq, const S* qs, const S* qe, int64_t* out) {
    auto* h = static_cast<RefMap<S>*>(hp);
    for (int64_t q = 0; q < nq; ++q) {
        switch (mode) {
            case 0: out[q] = (int64_t)h->m.count(qs[q], qe[q]); break;
            case 1: out[q] = (int64_t)h->m.count_linear(qs[q], qe[q]); break;
            case 2: out[q] = (int64_t)h->m.count_large(qs[q], qe[q]); break;
            case 3: out[q] = h->m.has_overlaps(qs[q], qe[q]) ? 1 : 0; break;
            default: out[q] = -1;
        }
    }
}

// mode: 0 search_idxs, 1 search_values, 2 search_values_large, 3 search_keys (start only)
template <typename S>
int64_t map_search(void* hp, int mode, int64_t nq, const S* qs, const S* qe,
                   int64_t* offsets, int64_t* out, int64_t cap) {
    auto* h = static_cast<RefMap<S>*>(hp);
    std::vector<size_t> idx;
    std::vector<int32_t> val;
    std::vector<std::pair<S, S>> keys;
    int64_t total = 0;
    offsets[0] = 0;
    for (int64_t q = 0; q < nq; ++q) {
        idx.clear(); val.clear(); keys.clear();
        int64_t k = 0;
        if (mode == 0) { h->m.search_idxs(qs[q], qe[q], idx); k = (int64_t)idx.size(); }
        else if (mode == 1) { h->m.search_values(qs[q], qe[q], val); k = (int64_t)val.size(); }
        else if (mode == 2) { h->m.search_values_large(qs[q], qe[q], val); k = (int64_t)val.size(); }
        else { h->m.search_keys(qs[q], qe[q], keys); k = (int64_t)keys.size(); }
        if (total + k <= cap) {
            for (int64_t j = 0; j < k; ++j) {
                if (mode == 0) out[total + j] = (int64_t)idx[j];
                else if (mode == 3) out[total + j] = (int64_t)keys[j].first;
                else out[total + j] = (int64_t)val[j];
            }
        }
        total += k;
        offsets[q + 1] = total;
    }
    return total;
}

template <typename S>
void map_coverage(void* hp, int64_t nq, const S* qs, const S* qe, int64_t* cnt, S* cov) {
    auto* h = static_cast<RefMap<S>*>(hp);
    for (int64_t q = 0; q < nq; ++q) {
        std::pair<size_t, S> r{0, 0};
        h->m.coverage(qs[q], qe[q], r);
        cnt[q] = (int64_t)r.first;
        cov[q] = r.second;
    }
}

// Set operations of map a against map b (hpp:1158-1211).  op 0: a.intersection(b) keeping a's
// data, op 1: a.intersection(b) keeping b's data, op 2: a.difference(b).  The result map is not
// built, so its arrays are in the order the reference adds pieces.  Returns the piece count;
// writes at most cap pieces.
template <typename S>
int64_t map_setop(void* ap, void* bp, int op, S* os, S* oe, int32_t* od, int64_t cap) {
    auto* a = static_cast<RefMap<S>*>(ap);
    auto* b = static_cast<RefMap<S>*>(bp);
    si::IntervalMap<S, int32_t> r;
    if (op == 0) r = a->m.intersection(b->m);
    else if (op == 1) r = a->m.intersection(b->m, [](const int32_t&, const int32_t& y) { return y; });
    else r = a->m.difference(b->m);
    const int64_t k = (int64_t)r.starts.size();
    for (int64_t i = 0; i < k && i < cap; ++i) {
        os[i] = r.starts[i];
        oe[i] = r.ends[i];
        od[i] = r.data[i];
    }
    return k;
}

}  // namespace

extern "C" {

int64_t ref_map_i32_setop(void* a, void* b, int op, int32_t* os, int32_t* oe, int32_t* od, int64_t cap) { return map_setop<int32_t>(a, b, op, os, oe, od, cap); }
int64_t ref_map_i64_setop(void* a, void* b, int op, int64_t* os, int64_t* oe, int32_t* od, int64_t cap) { return map_setop<int64_t>(a, b, op, os, oe, od, cap); }

void* ref_map_i32_new(int64_t n, const int32_t* s, const int32_t* e, const int32_t* d) { return map_new<int32_t>(n, s, e, d); }
void* ref_map_i64_new(int64_t n, const int64_t* s, const int64_t* e, const int32_t* d) { return map_new<int64_t>(n, s, e, d); }
void ref_map_i32_free(void* h) { delete static_cast<RefMap<int32_t>*>(h); }
void ref_map_i64_free(void* h) { delete static_cast<RefMap<int64_t>*>(h); }
int64_t ref_map_i32_size(void* h) { return (int64_t)static_cast<RefMap<int32_t>*>(h)->m.starts.size(); }
int64_t ref_map_i64_size(void* h) { return (int64_t)static_cast<RefMap<int64_t>*>(h)->m.starts.size(); }
void ref_map_i32_arrays(void* h, int32_t* s, int32_t* e, int32_t* d, int64_t* br) { map_arrays<int32_t>(h, s, e, d, br); }
void ref_map_i64_arrays(void* h, int64_t* s, int64_t* e, int32_t* d, int64_t* br) { map_arrays<int64_t>(h, s, e, d, br); }
void ref_map_i32_scalar(void* h, int mode, int64_t nq, const int32_t* qs, const int32_t* qe, int64_t* out) { map_scalar<int32_t>(h, mode, nq, qs, qe, out); }
void ref_map_i64_scalar(void* h, int mode, int64_t nq, const int64_t* qs, const int64_t* qe, int64_t* out) { map_scalar<int64_t>(h, mode, nq, qs, qe, out); }
int64_t ref_map_i32_search(void* h, int mode, int64_t nq, const int32_t* qs, const int32_t* qe, int64_t* off, int64_t* out, int64_t cap) { return map_search<int32_t>(h, mode, nq, qs, qe, off, out, cap); }
int64_t ref_map_i64_search(void* h, int mode, int64_t nq, const int64_t* qs, const int64_t* qe, int64_t* off, int64_t* out, int64_t cap) { return map_search<int64_t>(h, mode, nq, qs, qe, off, out, cap); }
void ref_map_i32_coverage(void* h, int64_t nq, const int32_t* qs, const int32_t* qe, int64_t* cnt, int32_t* cov) { map_coverage<int32_t>(h, nq, qs, qe, cnt, cov); }
void ref_map_i64_coverage(void* h, int64_t nq, const int64_t* qs, const int64_t* qe, int64_t* cnt, int64_t* cov) { map_coverage<int64_t>(h, nq, qs, qe, cnt, cov); }

}  // extern "C"
