// C++ drop-in check: the known answers of the reference's unit tests (test/tests.cpp:63-238)
// and of its Python README batch example (src/superintervals/README.md:16-27), asserted
// against si::IntervalMap from include/si_gpu/interval_map.hpp (answered by the GPU).
#include <cstdio>
#include <utility>
#include <vector>

#include "si_gpu/interval_map.hpp"

// the reference declares these two noexcept (superintervals.hpp:651, 865)
static_assert(noexcept(std::declval<const si::IntervalMap<int, int>&>().count(0, 0)), "count is noexcept");
static_assert(noexcept(std::declval<const si::IntervalMap<int64_t, int>&>().has_overlaps(0, 0)),
              "has_overlaps is noexcept");

#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "FAIL %s:%d: %s\n", __FILE__, __LINE__, #c); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

template <typename S>
int basics() {  // tests.cpp:63-107
    si::IntervalMap<S, int> itv;
    CHECK(!itv.has_overlaps(0, 1));
    itv.add(10, 20, 0);
    itv.add(11, 12, -1);
    itv.add(13, 14, -1);
    itv.add(15, 16, -1);
    itv.add(25, 29, 4);
    itv.build();
    CHECK(itv.has_overlaps(17, 30));
    CHECK(!itv.has_overlaps(1, 3));
    std::vector<int> values;
    itv.search_values(17, 30, values);
    CHECK(values.size() == 2 && values[0] == 4 && values[1] == 0);
    CHECK(itv.count(17, 30) == 2);
    std::vector<size_t> idxs;
    itv.search_idxs(17, 30, idxs);
    CHECK(idxs.size() == 2 && idxs[0] == 4 && idxs[1] == 0);
    std::vector<std::pair<S, S>> keys;
    itv.search_keys(17, 30, keys);
    CHECK(keys[0].first == 25 && keys[1].second == 20);
    std::pair<size_t, S> cov{0, 0};
    itv.coverage(10, 29, cov);
    CHECK(cov.second == 17);
    return 0;
}

template <typename S>
int overlaps() {  // tests.cpp:140-188
    std::vector<int> a;
    {
        si::IntervalMap<S, int> itv;
        itv.add(0, 250000, 0);
        for (int s : {55, 115, 130, 281, 639, 842, 999, 1094, 1157, 1161, 1265, 1532, 1590, 1665, 1945, 2384, 2515})
            itv.add(s, s + 1000, -1);
        itv.build();
        itv.search_values(1377, 2377, a);
        CHECK(a.back() == 0 && a.size() == 12);
        a.clear();
    }
    {
        si::IntervalMap<S, int> itv;
        itv.add(3, 40, 0);
        itv.add(4, 5, 4);
        itv.add(6, 7, 4);
        itv.add(10, 31, 5);
        itv.add(31, 32, 5);
        itv.build();
        itv.search_values(31, 32, a);
        CHECK(a.size() == 3);
        a.clear();
        itv.search_values(10, 11, a);
        CHECK(a.size() == 2);
        a.clear();
        itv.search_values(4, 7, a);
        CHECK(a.size() == 3);
        a.clear();
    }
    {
        si::IntervalMap<S, int> itv;
        itv.add(3, 40, 0);
        itv.add(3, 40, 4);
        itv.add(3, 40, 4);
        itv.add(3, 4, 4);
        itv.add(35, 50, 4);
        itv.add(40, 400, 5);
        itv.add(40, 400, 4);
        itv.build();
        itv.search_values(38, 41, a);
        CHECK(a.size() == 6);
        a.clear();
        itv.search_values(41, 42, a);
        CHECK(a.size() == 3);
        a.clear();
    }
    return 0;
}

template <typename S>
int coverage_and_edges() {  // tests.cpp:194-238
    si::IntervalMap<S, int> itv;
    itv.add(1, 100, 0);
    itv.add(30, 200, 7);
    itv.add(40, 50, 6);
    itv.add(60, 70, 7);
    itv.build();
    std::vector<int> a;
    itv.search_values(55, 65, a);
    CHECK(a.size() == 3);
    std::pair<size_t, S> cov{0, 0};
    itv.coverage(55, 65, cov);
    CHECK(cov.first == 3 && cov.second == 25);
    si::IntervalMap<S, int> empty;
    empty.build();
    CHECK(empty.count(1, 5) == 0);
    CHECK(!empty.has_overlaps(1, 5));
    si::IntervalMap<S, int> one;
    one.add(1, 10, 1);
    one.build();
    CHECK(one.count(1, 5) == 1);
    CHECK(one.count(11, 20) == 0);
    return 0;
}

int batch_readme() {  // src/superintervals/README.md:16-27
    si::IntervalMap<int32_t, const char*> imap;
    imap.add(10, 20, "A");
    imap.add(15, 25, "B");
    imap.add(30, 40, "C");
    imap.build();
    const int32_t qs[] = {5, 18, 35}, qe[] = {12, 22, 45};
    std::vector<uint32_t> c = imap.count_batch(qs, qe, 3);
    CHECK(c[0] == 1 && c[1] == 2 && c[2] == 1);
    std::vector<int64_t> off;
    std::vector<int32_t> idx;
    imap.search_idxs_batch(qs, qe, 3, off, idx);
    CHECK(off[1] == 1 && off[2] == 3 && off[3] == 4);
    CHECK(idx[0] == 0 && idx[1] == 0 && idx[2] == 1 && idx[3] == 2);
    std::vector<const char*> vals;
    imap.search_values_batch(qs, qe, 3, off, vals);
    CHECK(vals[1][0] == 'B' && vals[2][0] == 'A');
    // keys in search_keys order (descending) and coverage (no +1), batch and single
    std::vector<int32_t> ks, ke;
    imap.search_keys_batch(qs, qe, 3, off, ks, ke);
    CHECK(off[3] == 4 && ks[1] == 15 && ke[1] == 25 && ks[2] == 10 && ke[3] == 40);
    std::vector<uint64_t> cc;
    std::vector<int32_t> cv;
    imap.coverage_batch(qs, qe, 3, cc, cv);
    CHECK(cc[0] == 1 && cv[0] == 2 && cc[1] == 2 && cv[1] == 2 + 4 && cc[2] == 1 && cv[2] == 5);
    std::pair<size_t, int32_t> one{0, 0};
    imap.coverage(18, 22, one);
    CHECK(one.first == 2 && one.second == 6);
    return 0;
}

int main() {
    int rc = basics<int32_t>() | basics<int64_t>() | overlaps<int32_t>() | overlaps<int64_t>() |
             coverage_and_edges<int32_t>() | coverage_and_edges<int64_t>() | batch_readme();
    if (rc == 0) std::printf("drop-in ok\n");
    return rc;
}
