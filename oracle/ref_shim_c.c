/* ref_shim_c.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A thin shim around the UNMODIFIED reference C API src/c_superintervals.h
 * (kcleal/superintervals), found by include path at build time (oracle/Makefile,
 * REF_SRC).  Used only to produce golden fixtures for the C-API order
 * (fully descending searchIdxs / searchValues, c_superintervals.h:575-643).
 */
#include <stdint.h>
#include "c_superintervals.h"

void* ref_c_new(int64_t n, const int32_t* s, const int32_t* e, const int32_t* d) {
    cSuperIntervals* si = createSuperIntervals();
    reserveSuperIntervals(si, (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) addInterval(si, s[i], e[i], d ? d[i] : (int32_t)i);
    indexSuperIntervals(si);
    return si;
}

void ref_c_free(void* h) { destroySuperIntervals((cSuperIntervals*)h); }

/* op 0: intersection(a, b, NULL) (keeps a's data), op 2: difference(a, b)
 * (c_superintervals.h:921-974).  Returns the piece count; writes at most cap. */
int64_t ref_c_setop(void* a, void* b, int op, int32_t* os, int32_t* oe, int32_t* od, int64_t cap) {
    cSuperIntervals* r = op == 0 ? intersection((cSuperIntervals*)a, (cSuperIntervals*)b, NULL)
                                 : difference((cSuperIntervals*)a, (cSuperIntervals*)b);
    int64_t k = (int64_t)r->size;
    for (int64_t i = 0; i < k && i < cap; ++i) {
        os[i] = r->starts[i];
        oe[i] = r->ends[i];
        od[i] = r->data[i];
    }
    destroySuperIntervals(r);
    return k;
}

void ref_c_arrays(void* h, int32_t* s, int32_t* e, int32_t* d, int64_t* br) {
    cSuperIntervals* si = (cSuperIntervals*)h;
    for (size_t i = 0; i < si->size; ++i) {
        if (s) s[i] = si->starts[i];
        if (e) e[i] = si->ends[i];
        if (d) d[i] = si->data[i];
        if (br) br[i] = (si->branch[i] == SI_NONE) ? -1 : (int64_t)si->branch[i];
    }
}

/* mode 0 searchIdxs, 1 searchValues, 2 countOverlaps (offsets only), 3 anyOverlaps */
int64_t ref_c_search(void* h, int mode, int64_t nq, const int32_t* qs, const int32_t* qe,
                     int64_t* off, int64_t* out, int64_t cap) {
    cSuperIntervals* si = (cSuperIntervals*)h;
    cIndexResult r = createIndexResult();
    int64_t total = 0;
    off[0] = 0;
    for (int64_t q = 0; q < nq; ++q) {
        int64_t k = 0;
        if (mode == 0 || mode == 1) {
            clearIndexResult(&r);
            if (mode == 0) searchIdxs(si, qs[q], qe[q], &r);
            else searchValues(si, qs[q], qe[q], &r);
            k = (int64_t)r.size;
            if (total + k <= cap)
                for (int64_t j = 0; j < k; ++j) out[total + j] = r.data[j];
        } else if (mode == 2) {
            k = (int64_t)countOverlaps(si, qs[q], qe[q]);
        } else {
            k = anyOverlaps(si, qs[q], qe[q]) ? 1 : 0;
        }
        total += k;
        off[q + 1] = total;
    }
    destroyIndexResult(&r);
    return total;
}
