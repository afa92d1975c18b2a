/*
 * si_oracle.c -- the ORACLE for the SuperIntervals batch overlap-query path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference algorithm (kcleal/superintervals, src/superintervals.hpp and
 * src/c_superintervals.h).  It is used by the test-suite as the checker, and
 * by bench.py as the timed CPU baseline ("port").  No product code path links,
 * loads or calls it.
 *
 * Parity pin: this restatement is checked against fixtures produced by the
 * reference itself (oracle/ref_shim.cpp compiled against the reference header,
 * see tests/golden/make_golden.py) and against the known answers of the
 * reference's own unit tests (test/tests.cpp).
 *
 * What is restated, with the reference line each part follows:
 *   - add() sortedness flags ........ src/superintervals.hpp:95-105
 *   - sort_intervals / sort_block ... src/superintervals.hpp:1396-1439
 *       The reference sorts with std::sort (unstable).  This restatement uses
 *       a STABLE merge sort on the same key (start asc, end desc).  Starts and
 *       ends come out identical; the payload order can only differ inside runs
 *       of exact (start, end) duplicates, where std::sort's order is an
 *       artefact of libstdc++ introsort.
 *   - build() branch pass ........... src/superintervals.hpp:112-130
 *   - upper_bound ................... src/superintervals.hpp:501-516
 *   - count (count_linear form) ..... src/superintervals.hpp:623-649, 651-825
 *   - search_idxs (ascending head) .. src/superintervals.hpp:879-905
 *   - search_values (descending) .... src/superintervals.hpp:551-579
 *   - searchIdxs C API (descending) . src/c_superintervals.h:610-643
 *   - has_overlaps .................. src/superintervals.hpp:865-871
 *   - coverage ...................... src/superintervals.hpp:979-1006
 *   - per-query batch loops ......... src/superintervals/intervalmap.pyx:363-494
 *
 * Index sentinel: the reference uses SIZE_MAX; this file uses -1 (int64).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define SIO_NONE ((int64_t)-1)

/* order codes for the search family */
#define SIO_ORDER_IDXS_CPP 0   /* C++ search_idxs: head run ascending, rest descending */
#define SIO_ORDER_DESC 1       /* search_values / C searchIdxs: fully descending */

typedef struct {
    int64_t begin, end;   /* query range handled by one worker claim */
} sio_range;

/* ------------------------------------------------------------------------- */
/* A tiny dynamic work queue over [0, n) for the multi-threaded batch loops.  */
/* ------------------------------------------------------------------------- */
typedef struct {
    int64_t n;
    int64_t chunk;
    int64_t next;   /* accessed with __atomic builtins */
} sio_queue;

static int sio_claim(sio_queue* q, sio_range* r) {
    int64_t b = __atomic_fetch_add(&q->next, q->chunk, __ATOMIC_RELAXED);
    if (b >= q->n) return 0;
    r->begin = b;
    r->end = (b + q->chunk < q->n) ? b + q->chunk : q->n;
    return 1;
}

typedef void (*sio_worker_fn)(void* ctx, int64_t begin, int64_t end);

typedef struct {
    sio_queue* q;
    sio_worker_fn fn;
    void* ctx;
} sio_thread_arg;

static void* sio_thread_main(void* p) {
    sio_thread_arg* a = (sio_thread_arg*)p;
    sio_range r;
    while (sio_claim(a->q, &r)) a->fn(a->ctx, r.begin, r.end);
    return NULL;
}

static void sio_parallel_for_chunk(int64_t n, int nthreads, void (*fn)(void*, int64_t, int64_t), void* ctx,
                                   int64_t chunk) {
    if (n <= 0) return;
    if (nthreads <= 1) {
        fn(ctx, 0, n);
        return;
    }
    sio_queue q;
    q.n = n;
    q.chunk = chunk;
    q.next = 0;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    sio_thread_arg arg = {&q, fn, ctx};
    int started = 0;
    for (int t = 0; t < nthreads; ++t) {
        if (pthread_create(&th[t], NULL, sio_thread_main, &arg) == 0) ++started;
        else break;
    }
    if (started == 0) fn(ctx, 0, n);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
    free(th);
}

static void sio_parallel_for(int64_t n, int nthreads, void (*fn)(void*, int64_t, int64_t), void* ctx) {
    sio_parallel_for_chunk(n, nthreads, fn, ctx, 2048);
}

/* ------------------------------------------------------------------------- */
/* Single-pass batch search: each worker walks its queries once and appends   */
/* the hits to a growable buffer per chunk of queries, as the reference's    */
/* per-query search_idxs appends to a std::vector (hpp:879-905) and its batch */
/* loop builds one list per query (intervalmap.pyx:402-446).  The chunks are  */
/* then copied into one CSR array.                                            */
/* ------------------------------------------------------------------------- */
#define SIO_LIST_CHUNK 2048
typedef struct {
    int32_t* vals;
    int64_t n, cap;
} sio_list_chunk;

typedef struct {
    int64_t nq, n_chunks;
    sio_list_chunk* chunks;
} sio_lists;

static int sio_list_reserve(sio_list_chunk* c, int64_t need) {
    if (c->n + need <= c->cap) return 1;
    int64_t cap = c->cap ? c->cap : 4096;
    while (cap < c->n + need) cap *= 2;
    int32_t* p = (int32_t*)realloc(c->vals, sizeof(int32_t) * (size_t)cap);
    if (!p) return 0;
    c->vals = p;
    c->cap = cap;
    return 1;
}

int64_t sio_lists_total(const void* h) {
    const sio_lists* L = (const sio_lists*)h;
    int64_t t = 0;
    for (int64_t k = 0; k < L->n_chunks; ++k) t += L->chunks[k].n;
    return t;
}

typedef struct {
    const sio_lists* L;
    const int64_t* offsets;
    int32_t* out;
} sio_copy_ctx;

static void sio_copy_worker(void* p, int64_t b, int64_t e) {
    sio_copy_ctx* c = (sio_copy_ctx*)p;
    for (int64_t k = b; k < e; ++k) {
        const sio_list_chunk* ch = &c->L->chunks[k];
        if (ch->n) memcpy(c->out + c->offsets[k * SIO_LIST_CHUNK], ch->vals, sizeof(int32_t) * (size_t)ch->n);
    }
}

static void sio_parallel_for_chunk(int64_t n, int nthreads, void (*fn)(void*, int64_t, int64_t), void* ctx,
                                   int64_t chunk);

/* Copy the chunk buffers into out at the query offsets (offsets[nq + 1] = exclusive sums of
   the counts the search wrote). */
void sio_lists_copy(const void* h, const int64_t* offsets, int32_t* out, int nthreads) {
    sio_copy_ctx c = {(const sio_lists*)h, offsets, out};
    sio_parallel_for_chunk(((const sio_lists*)h)->n_chunks, nthreads, sio_copy_worker, &c, 1);
}

void sio_lists_free(void* h) {
    sio_lists* L = (sio_lists*)h;
    if (!L) return;
    for (int64_t k = 0; k < L->n_chunks; ++k) free(L->chunks[k].vals);
    free(L->chunks);
    free(L);
}

static sio_lists* sio_lists_new(int64_t nq) {
    sio_lists* L = (sio_lists*)calloc(1, sizeof(sio_lists));
    if (!L) return NULL;
    L->nq = nq;
    L->n_chunks = (nq + SIO_LIST_CHUNK - 1) / SIO_LIST_CHUNK;
    L->chunks = (sio_list_chunk*)calloc((size_t)(L->n_chunks ? L->n_chunks : 1), sizeof(sio_list_chunk));
    if (!L->chunks) {
        free(L);
        return NULL;
    }
    return L;
}

/* ------------------------------------------------------------------------- */
/* Type-generic body, instantiated for int32 and int64 coordinates.          */
/* ------------------------------------------------------------------------- */
#define SIO_DEFINE(SFX, S)                                                              \
                                                                                        \
/* Key order of sort_intervals (hpp:1418): start ascending, then end descending.   */   \
static int sio_less_##SFX(const S* s, const S* e, int64_t a, int64_t b) {               \
    if (s[a] != s[b]) return s[a] < s[b];                                               \
    return e[a] > e[b];                                                                 \
}                                                                                       \
                                                                                        \
static void sio_msort_##SFX(const S* s, const S* e, int64_t* idx, int64_t* tmp,         \
                            int64_t n) {                                                \
    /* bottom-up stable merge sort of idx by (start asc, end desc) */                   \
    for (int64_t w = 1; w < n; w *= 2) {                                                \
        for (int64_t lo = 0; lo < n; lo += 2 * w) {                                     \
            int64_t mid = lo + w < n ? lo + w : n;                                      \
            int64_t hi = lo + 2 * w < n ? lo + 2 * w : n;                               \
            int64_t i = lo, j = mid, k = lo;                                            \
            while (i < mid && j < hi) {                                                 \
                /* take from the right only if strictly less: keeps stability */        \
                if (sio_less_##SFX(s, e, idx[j], idx[i])) tmp[k++] = idx[j++];          \
                else tmp[k++] = idx[i++];                                               \
            }                                                                           \
            while (i < mid) tmp[k++] = idx[i++];                                        \
            while (j < hi) tmp[k++] = idx[j++];                                         \
        }                                                                               \
        memcpy(idx, tmp, sizeof(int64_t) * (size_t)n);                                  \
    }                                                                                   \
}                                                                                       \
                                                                                        \
/* Sort + branch build for one map.  Follows build() (hpp:112-130) and           */     \
/* sort_intervals (hpp:1415-1439) with the stable-sort substitution noted above.  */    \
/* perm (optional) receives the input position of each sorted slot.              */     \
/* Returns 1 when the input was already in canonical order (no sort performed).  */     \
int sio_build_##SFX(int64_t n, const S* s_in, const S* e_in, const int32_t* d_in,      \
                    S* s_out, S* e_out, int32_t* d_out, int64_t* perm,                 \
                    int64_t* branch) {                                                  \
    if (n <= 0) return 1;                                                               \
    /* replay of add()'s flag maintenance (hpp:95-105) */                               \
    int start_sorted = 1, end_sorted = 1;                                               \
    for (int64_t i = 1; i < n && start_sorted; ++i) {                                   \
        start_sorted = (s_in[i] < s_in[i - 1]) ? 0 : 1;                                 \
        if (start_sorted && s_in[i] == s_in[i - 1] && e_in[i] > e_in[i - 1])            \
            end_sorted = 0;                                                             \
    }                                                                                   \
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);                       \
    for (int64_t i = 0; i < n; ++i) idx[i] = i;                                         \
    int sorted = start_sorted && end_sorted;                                            \
    if (!sorted) {                                                                      \
        int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);                   \
        sio_msort_##SFX(s_in, e_in, idx, tmp, n);                                       \
        free(tmp);                                                                      \
    }                                                                                   \
    for (int64_t i = 0; i < n; ++i) {                                                   \
        s_out[i] = s_in[idx[i]];                                                        \
        e_out[i] = e_in[idx[i]];                                                        \
        if (d_in && d_out) d_out[i] = d_in[idx[i]];                                     \
        if (perm) perm[i] = idx[i];                                                     \
    }                                                                                   \
    free(idx);                                                                          \
    /* monotonic stack: branch[i] = nearest j < i with ends[j] >= ends[i] */            \
    if (branch) {                                                                       \
        int64_t* st = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);                    \
        int64_t top = 0;                                                                \
        branch[0] = SIO_NONE;                                                           \
        st[top++] = 0;                                                                  \
        for (int64_t i = 1; i < n; ++i) {                                               \
            while (top > 0 && e_out[st[top - 1]] < e_out[i]) --top;                     \
            branch[i] = top > 0 ? st[top - 1] : SIO_NONE;                               \
            st[top++] = i;                                                              \
        }                                                                               \
        free(st);                                                                       \
    }                                                                                   \
    return sorted;                                                                      \
}                                                                                       \
                                                                                        \
/* upper_bound (hpp:501-516): last k with starts[k] <= v, else -1.               */     \
int64_t sio_upper_bound_##SFX(int64_t n, const S* starts, S v) {                        \
    if (n <= 0) return SIO_NONE;                                                        \
    int64_t length = n, idx = 0;                                                        \
    while (length > 1) {                                                                \
        int64_t half = length / 2;                                                      \
        idx += (starts[idx + half] <= v) * (length - half);                             \
        length = half;                                                                  \
    }                                                                                   \
    if (starts[idx] > v) --idx;                                                         \
    return idx;                                                                         \
}                                                                                       \
                                                                                        \
/* count (hpp:623-649): size of { k <= ub(qe) : ends[k] >= qs }.                 */     \
int64_t sio_count_##SFX(int64_t n, const S* starts, const S* ends,                      \
                        const int64_t* branch, S qs, S qe) {                            \
    int64_t i = sio_upper_bound_##SFX(n, starts, qe);                                   \
    if (i == SIO_NONE) return 0;                                                        \
    int64_t top = i;                                                                    \
    while (i != SIO_NONE && qs <= ends[i]) --i;                                         \
    int64_t c = top - i;                                                                \
    if (i == SIO_NONE) return c;                                                        \
    i = branch[i];                                                                      \
    while (i != SIO_NONE) {                                                             \
        if (qs <= ends[i]) { ++c; --i; }                                                \
        else i = branch[i];                                                             \
    }                                                                                   \
    return c;                                                                           \
}                                                                                       \
                                                                                        \
/* has_overlaps (hpp:865-871) */                                                        \
int sio_has_overlaps_##SFX(int64_t n, const S* starts, const S* ends, S qs, S qe) {     \
    int64_t i = sio_upper_bound_##SFX(n, starts, qe);                                   \
    return i != SIO_NONE && qs <= ends[i];                                              \
}                                                                                       \
                                                                                        \
/* search_idxs (hpp:879-905, order 0) / search_values + C searchIdxs             */     \
/* (hpp:551-579, c:610-643, order 1).  Writes positions (or data[pos] when       */     \
/* data != NULL) to out and returns how many were written.                       */     \
int64_t sio_search_##SFX(int64_t n, const S* starts, const S* ends,                     \
                         const int64_t* branch, const int32_t* data, S qs, S qe,        \
                         int order, int64_t* out) {                                     \
    int64_t idx = sio_upper_bound_##SFX(n, starts, qe);                                 \
    if (idx == SIO_NONE) return 0;                                                      \
    int64_t i = idx, w = 0;                                                             \
    while (i != SIO_NONE && qs <= ends[i]) --i;                                         \
    /* head run i+1 .. idx */                                                           \
    if (order == SIO_ORDER_IDXS_CPP) {                                                  \
        for (int64_t k = i + 1; k <= idx; ++k) out[w++] = data ? data[k] : k;           \
    } else {                                                                            \
        for (int64_t k = idx; k > i; --k) out[w++] = data ? data[k] : k;               \
    }                                                                                   \
    if (i == SIO_NONE) return w;                                                        \
    i = branch[i];                                                                      \
    while (i != SIO_NONE) {                                                             \
        if (qs <= ends[i]) { out[w++] = data ? data[i] : i; --i; }                      \
        else i = branch[i];                                                             \
    }                                                                                   \
    return w;                                                                           \
}                                                                                       \
                                                                                        \
/* ---- set operations of a list of intervals (map A) against this map (B) ----- */     \
typedef struct { S s, e; } sio_key_##SFX;                                               \
static int sio_keycmp_##SFX(const void* x, const void* y) {                             \
    const sio_key_##SFX* a = (const sio_key_##SFX*)x;                                   \
    const sio_key_##SFX* b = (const sio_key_##SFX*)y;                                   \
    if (a->s != b->s) return a->s < b->s ? -1 : 1;                                      \
    return (a->e > b->e) - (a->e < b->e);                                               \
}                                                                                       \
                                                                                        \
/* intersection (hpp:1158-1177, c:921-940): for each A interval k, in order, one */     \
/* piece [max(as, starts[h]), min(ae, ends[h])] per hit h of search (order), kept */    \
/* when start <= end.  ob receives h.  Returns the piece count (writes <= cap).   */     \
int64_t sio_intersection_##SFX(int64_t n, const S* starts, const S* ends,              \
                               const int64_t* branch, int64_t na, const S* as,          \
                               const S* ae, int order, int64_t* off, S* os, S* oe,      \
                               int64_t* ob, int64_t cap) {                              \
    int64_t total = 0, bcap = 0;                                                        \
    int64_t* buf = NULL;                                                                \
    if (off) off[0] = 0;                                                                \
    for (int64_t k = 0; k < na; ++k) {                                                  \
        int64_t c = sio_count_##SFX(n, starts, ends, branch, as[k], ae[k]);            \
        if (c > bcap) { bcap = 2 * c; buf = (int64_t*)realloc(buf, 8 * (size_t)bcap); } \
        int64_t w = c ? sio_search_##SFX(n, starts, ends, branch, NULL, as[k], ae[k],   \
                                         order, buf) : 0;                               \
        for (int64_t j = 0; j < w; ++j) {                                               \
            int64_t h = buf[j];                                                         \
            S s = as[k] > starts[h] ? as[k] : starts[h];                                \
            S e = ae[k] < ends[h] ? ae[k] : ends[h];                                    \
            if (s <= e) {                                                               \
                if (total < cap) { os[total] = s; oe[total] = e; ob[total] = h; }       \
                ++total;                                                                \
            }                                                                           \
        }                                                                               \
        if (off) off[k + 1] = total;                                                    \
    }                                                                                   \
    free(buf);                                                                          \
    return total;                                                                       \
}                                                                                       \
                                                                                        \
/* difference (hpp:1186-1211, c:951-974): per A interval, the hits' (start, end) */     \
/* keys sorted ascending and swept with a cursor from as; every uncovered piece   */    \
/* is emitted.  A covered piece reaching the type's maximum ends the sweep (the  */     \
/* reference's cursor = end + 1 overflows there).                                */     \
int64_t sio_difference_##SFX(int64_t n, const S* starts, const S* ends,                \
                             const int64_t* branch, int64_t na, const S* as,            \
                             const S* ae, int64_t* off, S* os, S* oe, int64_t cap) {    \
    const S smax = (S)((((uint64_t)1) << (sizeof(S) * 8 - 1)) - 1);                     \
    int64_t total = 0, bcap = 0;                                                        \
    int64_t* buf = NULL;                                                                \
    sio_key_##SFX* keys = NULL;                                                         \
    if (off) off[0] = 0;                                                                \
    for (int64_t k = 0; k < na; ++k) {                                                  \
        int64_t c = sio_count_##SFX(n, starts, ends, branch, as[k], ae[k]);            \
        if (c > bcap) {                                                                 \
            bcap = 2 * c;                                                               \
            buf = (int64_t*)realloc(buf, 8 * (size_t)bcap);                             \
            keys = (sio_key_##SFX*)realloc(keys, sizeof(sio_key_##SFX) * (size_t)bcap); \
        }                                                                               \
        int64_t w = c ? sio_search_##SFX(n, starts, ends, branch, NULL, as[k], ae[k],   \
                                         SIO_ORDER_DESC, buf) : 0;                      \
        for (int64_t j = 0; j < w; ++j) { keys[j].s = starts[buf[j]]; keys[j].e = ends[buf[j]]; } \
        if (w > 1) qsort(keys, (size_t)w, sizeof(sio_key_##SFX), sio_keycmp_##SFX);    \
        S cursor = as[k];                                                               \
        int closed = 0;                                                                 \
        for (int64_t j = 0; j < w; ++j) {                                               \
            S cs = keys[j].s > as[k] ? keys[j].s : as[k];                               \
            S ce = keys[j].e < ae[k] ? keys[j].e : ae[k];                               \
            if (!closed && cs > cursor) {                                               \
                if (total < cap) { os[total] = cursor; oe[total] = cs - 1; }            \
                ++total;                                                                \
            }                                                                           \
            if (ce == smax) closed = 1;                                                 \
            else if (ce + 1 > cursor) cursor = ce + 1;                                  \
        }                                                                               \
        if (!closed && cursor <= ae[k]) {                                               \
            if (total < cap) { os[total] = cursor; oe[total] = ae[k]; }                 \
            ++total;                                                                    \
        }                                                                               \
        if (off) off[k + 1] = total;                                                    \
    }                                                                                   \
    free(buf);                                                                          \
    free(keys);                                                                         \
    return total;                                                                       \
}                                                                                       \
                                                                                        \
/* coverage (hpp:979-1006): count and sum of min(e)-max(s) (no +1).              */     \
void sio_coverage_##SFX(int64_t n, const S* starts, const S* ends,                      \
                        const int64_t* branch, S qs, S qe, int64_t* cnt, S* cov) {      \
    *cnt = 0; *cov = 0;                                                                 \
    int64_t i = sio_upper_bound_##SFX(n, starts, qe);                                   \
    if (i == SIO_NONE) return;                                                          \
    while (i != SIO_NONE && qs <= ends[i]) {                                            \
        ++*cnt;                                                                         \
        *cov += (ends[i] < qe ? ends[i] : qe) - (starts[i] > qs ? starts[i] : qs);      \
        --i;                                                                            \
    }                                                                                   \
    if (i == SIO_NONE) return;                                                          \
    i = branch[i];                                                                      \
    while (i != SIO_NONE) {                                                             \
        if (qs <= ends[i]) {                                                            \
            ++*cnt;                                                                     \
            *cov += (ends[i] < qe ? ends[i] : qe) - (starts[i] > qs ? starts[i] : qs);  \
            --i;                                                                        \
        } else i = branch[i];                                                           \
    }                                                                                   \
}                                                                                       \
                                                                                        \
/* ---- batch loops over many queries (intervalmap.pyx:363-494), optionally    */       \
/* against a set of per-contig maps concatenated with segment offsets.         */       \
typedef struct {                                                                        \
    const int64_t* seg; /* n_seg+1 offsets into the concatenated arrays */              \
    const S* starts; const S* ends; const int64_t* branch; const int32_t* data;         \
    const int32_t* qc; const S* qs; const S* qe;                                        \
    int order;                                                                          \
    uint32_t* counts; const int64_t* offsets; int32_t* out32; int64_t* scratch;         \
} sio_batch_ctx_##SFX;                                                                  \
                                                                                        \
static void sio_ub_worker_##SFX(void* p, int64_t b, int64_t e) {                        \
    sio_batch_ctx_##SFX* c = (sio_batch_ctx_##SFX*)p;                                   \
    for (int64_t q = b; q < e; ++q) {                                                   \
        int32_t g = c->qc ? c->qc[q] : 0;                                               \
        int64_t lo = c->seg[g], n = c->seg[g + 1] - lo;                                 \
        c->scratch[q] = sio_upper_bound_##SFX(n, c->starts + lo, c->qe[q]);            \
    }                                                                                   \
}                                                                                       \
                                                                                        \
static void sio_count_worker_##SFX(void* p, int64_t b, int64_t e) {                     \
    sio_batch_ctx_##SFX* c = (sio_batch_ctx_##SFX*)p;                                   \
    for (int64_t q = b; q < e; ++q) {                                                   \
        int32_t g = c->qc ? c->qc[q] : 0;                                               \
        int64_t lo = c->seg[g], n = c->seg[g + 1] - lo;                                 \
        c->counts[q] = (uint32_t)sio_count_##SFX(n, c->starts + lo, c->ends + lo,      \
                                                 c->branch + lo, c->qs[q], c->qe[q]);   \
    }                                                                                   \
}                                                                                       \
                                                                                        \
static void sio_search_worker_##SFX(void* p, int64_t b, int64_t e) {                    \
    sio_batch_ctx_##SFX* c = (sio_batch_ctx_##SFX*)p;                                   \
    int64_t cap = 0; int64_t* buf = NULL;                                               \
    for (int64_t q = b; q < e; ++q) {                                                   \
        int32_t g = c->qc ? c->qc[q] : 0;                                               \
        int64_t lo = c->seg[g], n = c->seg[g + 1] - lo;                                 \
        int64_t need = c->offsets[q + 1] - c->offsets[q];                               \
        if (need > cap) { cap = need * 2; buf = (int64_t*)realloc(buf, 8 * (size_t)cap); } \
        int64_t w = sio_search_##SFX(n, c->starts + lo, c->ends + lo, c->branch + lo,   \
                                     c->data ? c->data + lo : NULL, c->qs[q], c->qe[q], \
                                     c->order, buf);                                    \
        int32_t* dst = c->out32 + c->offsets[q];                                        \
        for (int64_t k = 0; k < w && k < need; ++k) dst[k] = (int32_t)buf[k];           \
    }                                                                                   \
    free(buf);                                                                          \
}                                                                                       \
                                                                                        \
void sio_count_batch_##SFX(const int64_t* seg, const S* starts, const S* ends,          \
                           const int64_t* branch, int64_t nq, const int32_t* qc,        \
                           const S* qs, const S* qe, uint32_t* counts, int nthreads) {  \
    sio_batch_ctx_##SFX c;                                                              \
    memset(&c, 0, sizeof(c));                                                           \
    c.seg = seg; c.starts = starts; c.ends = ends; c.branch = branch;                   \
    c.qc = qc; c.qs = qs; c.qe = qe; c.counts = counts;                                 \
    sio_parallel_for(nq, nthreads, sio_count_worker_##SFX, &c);                         \
}                                                                                       \
                                                                                        \
/* upper_bound of every query end in its contig's map (hpp:501-516), -1 when none. */ \
void sio_upper_bound_batch_##SFX(const int64_t* seg, const S* starts, int64_t nq,       \
                                 const int32_t* qc, const S* qe, int64_t* out,          \
                                 int nthreads) {                                        \
    sio_batch_ctx_##SFX c;                                                              \
    memset(&c, 0, sizeof(c));                                                           \
    c.seg = seg; c.starts = starts; c.qc = qc; c.qe = qe; c.scratch = out;              \
    sio_parallel_for(nq, nthreads, sio_ub_worker_##SFX, &c);                            \
}                                                                                       \
                                                                                        \
void sio_search_batch_##SFX(const int64_t* seg, const S* starts, const S* ends,         \
                            const int64_t* branch, const int32_t* data, int64_t nq,     \
                            const int32_t* qc, const S* qs, const S* qe, int order,     \
                            const int64_t* offsets, int32_t* out, int nthreads) {       \
    sio_batch_ctx_##SFX c;                                                              \
    memset(&c, 0, sizeof(c));                                                           \
    c.seg = seg; c.starts = starts; c.ends = ends; c.branch = branch; c.data = data;    \
    c.qc = qc; c.qs = qs; c.qe = qe; c.order = order; c.offsets = offsets;              \
    c.out32 = out;                                                                      \
    sio_parallel_for(nq, nthreads, sio_search_worker_##SFX, &c);                        \
}                                                                                       \
                                                                                        \
/* Single-pass batch search (see sio_lists above): counts[q] = hits of query q;  */     \
/* returns the chunk lists (sio_lists_total / sio_lists_copy / sio_lists_free).  */     \
typedef struct {                                                                        \
    sio_batch_ctx_##SFX b; sio_lists* L; int failed;                                    \
} sio_lists_ctx_##SFX;                                                                  \
                                                                                        \
static void sio_lists_worker_##SFX(void* p, int64_t cb, int64_t ce) {                   \
    sio_lists_ctx_##SFX* x = (sio_lists_ctx_##SFX*)p;                                   \
    const sio_batch_ctx_##SFX* c = &x->b;                                               \
    for (int64_t k = cb; k < ce; ++k) {                                                 \
        sio_list_chunk* ch = &x->L->chunks[k];                                          \
        /* the chunk's buffer in locals: stores through vals cannot alias them */       \
        int32_t* vals = ch->vals; int64_t w = ch->n, cap = ch->cap;                     \
        const int64_t q1 = (k + 1) * SIO_LIST_CHUNK < x->L->nq ? (k + 1) * SIO_LIST_CHUNK \
                                                               : x->L->nq;              \
        for (int64_t q = k * SIO_LIST_CHUNK; q < q1; ++q) {                             \
            int32_t g = c->qc ? c->qc[q] : 0;                                           \
            int64_t lo = c->seg[g], n = c->seg[g + 1] - lo;                             \
            const S* st = c->starts + lo; const S* en = c->ends + lo;                   \
            const int64_t* br = c->branch + lo;                                         \
            const int32_t* dd = c->data ? c->data + lo : NULL;                          \
            const S qs = c->qs[q], qe = c->qe[q];                                       \
            const int64_t w0 = w;                                                       \
            int64_t idx = sio_upper_bound_##SFX(n, st, qe);                             \
            if (idx != SIO_NONE) {                                                      \
                int64_t i = idx;                                                        \
                while (i != SIO_NONE && qs <= en[i]) --i;                               \
                if (w + (idx - i) + 64 > cap) {                                         \
                    ch->vals = vals; ch->n = w; ch->cap = cap;                          \
                    if (!sio_list_reserve(ch, idx - i + 64)) { x->failed = 1; return; } \
                    vals = ch->vals; cap = ch->cap;                                     \
                }                                                                       \
                if (c->order == SIO_ORDER_IDXS_CPP) {                                   \
                    for (int64_t t = i + 1; t <= idx; ++t) vals[w++] = dd ? dd[t] : (int32_t)t; \
                } else {                                                                \
                    for (int64_t t = idx; t > i; --t) vals[w++] = dd ? dd[t] : (int32_t)t; \
                }                                                                       \
                if (i != SIO_NONE) {                                                    \
                    i = br[i];                                                          \
                    while (i != SIO_NONE) {                                             \
                        if (qs <= en[i]) {                                              \
                            if (w == cap) {                                             \
                                ch->vals = vals; ch->n = w; ch->cap = cap;              \
                                if (!sio_list_reserve(ch, 64)) { x->failed = 1; return; } \
                                vals = ch->vals; cap = ch->cap;                         \
                            }                                                           \
                            vals[w++] = dd ? dd[i] : (int32_t)i;                        \
                            --i;                                                        \
                        } else {                                                        \
                            i = br[i];                                                  \
                        }                                                               \
                    }                                                                   \
                }                                                                       \
            }                                                                           \
            c->counts[q] = (uint32_t)(w - w0);                                          \
        }                                                                               \
        ch->vals = vals; ch->n = w; ch->cap = cap;                                      \
    }                                                                                   \
}                                                                                       \
                                                                                        \
void* sio_search_lists_##SFX(const int64_t* seg, const S* starts, const S* ends,        \
                             const int64_t* branch, const int32_t* data, int64_t nq,    \
                             const int32_t* qc, const S* qs, const S* qe, int order,    \
                             uint32_t* counts, int nthreads) {                          \
    sio_lists_ctx_##SFX x;                                                              \
    memset(&x, 0, sizeof(x));                                                           \
    x.b.seg = seg; x.b.starts = starts; x.b.ends = ends; x.b.branch = branch;           \
    x.b.data = data; x.b.qc = qc; x.b.qs = qs; x.b.qe = qe; x.b.order = order;          \
    x.b.counts = counts;                                                                \
    x.L = sio_lists_new(nq);                                                            \
    if (!x.L) return NULL;                                                              \
    sio_parallel_for_chunk(x.L->n_chunks, nthreads, sio_lists_worker_##SFX, &x, 1);              \
    if (x.failed) { sio_lists_free(x.L); return NULL; }                                 \
    return x.L;                                                                         \
}                                                                                       \
                                                                                        \
/* Per-contig build over concatenated input segments (each segment is one map). */     \
void sio_build_segments_##SFX(int64_t n_seg, const int64_t* seg, const S* s_in,         \
                              const S* e_in, const int32_t* d_in, S* s_out, S* e_out,   \
                              int32_t* d_out, int64_t* perm, int64_t* branch) {         \
    for (int64_t g = 0; g < n_seg; ++g) {                                               \
        int64_t lo = seg[g], n = seg[g + 1] - lo;                                       \
        sio_build_##SFX(n, s_in + lo, e_in + lo, d_in ? d_in + lo : NULL, s_out + lo,   \
                        e_out + lo, d_out ? d_out + lo : NULL, perm ? perm + lo : NULL, \
                        branch + lo);                                                   \
    }                                                                                   \
}

SIO_DEFINE(i32, int32_t)
SIO_DEFINE(i64, int64_t)
