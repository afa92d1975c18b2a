/*
 * c_api.h -- C-ABI of the GB300 SuperIntervals overlap-query library (libsi_gpu.so).
 *
 * Drop-in for the batch overlap-query path of kcleal/superintervals.  Every
 * entry point below names the reference interface it replaces (file:line in
 * the reference project).  Semantics follow the reference exactly:
 *   - intervals are END-INCLUSIVE [start, end];
 *   - indexSuperIntervalsGpu sorts by (start asc, end desc) and builds the
 *     branch array (nearest preceding interval with end >= this end);
 *   - searchIdxs results use the C++ order (ascending head run, then the
 *     descending branch walk) or the fully descending order of the C API;
 *   - results are per-query lists, returned in CSR form (offsets + values).
 * Differences, all deliberate:
 *   - every call returns an int status (SI_OK = 0) because device work can fail;
 *     the reference's void returns cannot report that;
 *   - the sort is stable: payloads of exact (start, end) duplicates keep their
 *     insertion order (the reference's std::sort / qsort leave it unspecified);
 *   - a handle may hold several contigs (one independent map per contig, the
 *     per-chromosome pattern of examples/bed-intersect-si.rs:98-120); queries
 *     then carry a contig id and results carry contig-local indices.
 *
 * Threading: one CUDA stream per handle; calls on one handle must not overlap.
 * Ownership: the handle owns its device buffers; result buffers belong to the
 * caller (cCsrResult buffers grown by the library are freed by destroyCsrResult).
 */
#ifndef SI_GPU_C_API_H
#define SI_GPU_C_API_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SI_GPU_VERSION "1.0.0"

/* ---- status codes ------------------------------------------------------ */
#define SI_OK 0
#define SI_ERR_INVALID 1      /* bad argument (null pointer, wrong coordinate width, bad contig) */
#define SI_ERR_OOM 2          /* device allocation failed or exceeded the device budget */
#define SI_ERR_NOT_BUILT 3    /* query before indexSuperIntervalsGpu (or after a later add) */
#define SI_ERR_CUDA 4         /* a CUDA call failed; see lastErrorGpu() */
#define SI_ERR_CAPACITY 5     /* caller-provided output too small; the needed size is reported */
#define SI_ERR_UNSUPPORTED 6  /* option not available for this handle */
#define SI_ERR_TOO_LARGE 7    /* more intervals than the 32-bit position space allows */

/* ---- query orders ------------------------------------------------------ */
#define SI_ORDER_IDXS_CPP 0   /* si::IntervalMap::search_idxs (superintervals.hpp:879-905) */
#define SI_ORDER_DESC 1       /* search_values (hpp:551-579) and C searchIdxs (c_superintervals.h:610-643) */

/* ---- query paths -------------------------------------------------------- */
#define SI_PATH_AUTO 0        /* library choice */
#define SI_PATH_PLAIN 1       /* one query per thread, reference walk */
#define SI_PATH_BATCHED 2     /* sorted-query tiles sharing one candidate walk */

/* ---- upper-bound search modes -------------------------------------------- */
#define SI_UB_BINARY 0        /* branch-free halving search (superintervals.hpp:501-516) */
#define SI_UB_EYTZINGER 1     /* shared-memory Eytzinger top levels + bounded global search */
#define SI_UB_LEARNED 2       /* two-stage piecewise-linear model + max-error window */

/* Opaque handle: replaces cSuperIntervals (c_superintervals.h:81-91). */
typedef struct gSuperIntervals gSuperIntervals;

/* CSR result: offsets[n_queries + 1] and values[offsets[n_queries]].
 * Replaces the per-query cIndexResult buffers (c_superintervals.h:98-102) and the
 * list-of-lists of the batch methods (intervalmap.pyx:402-494). */
typedef struct {
    int64_t* offsets;
    int32_t* values;
    size_t n_queries;
    size_t size;              /* number of values */
    size_t capacity;          /* allocated values */
    size_t offsets_capacity;  /* allocated offsets */
} cCsrResult;

/* ---- lifecycle: createSuperIntervals / destroySuperIntervals /
 *      clearSuperIntervals / reserveSuperIntervals (c_superintervals.h:135-144) ---- */
int createSuperIntervalsGpu(gSuperIntervals** out, int coord_bits /* 32 or 64 */, int device);
void destroySuperIntervalsGpu(gSuperIntervals* si);
int clearSuperIntervalsGpu(gSuperIntervals* si);
int reserveSuperIntervalsGpu(gSuperIntervals* si, size_t n);

/* ---- staging: addInterval (c_superintervals.h:153, 402-419; hpp:95-105);
 *      the array forms replace IntervalMap.from_arrays (intervalmap.pyx:63-131) -- */
int addIntervalGpu(gSuperIntervals* si, int32_t start, int32_t end, int32_t value);
int addIntervalGpu_i64(gSuperIntervals* si, int64_t start, int64_t end, int32_t value);
int addIntervalsGpu(gSuperIntervals* si, const int32_t* starts, const int32_t* ends,
                    const int32_t* values /* may be NULL: insertion index */, size_t n);
int addIntervalsGpu_i64(gSuperIntervals* si, const int64_t* starts, const int64_t* ends,
                        const int32_t* values, size_t n);
/* Declare that the staged intervals form n_contigs consecutive groups:
 * contig g holds staged intervals [offsets[g], offsets[g+1]).  No reference
 * counterpart (one IntervalMap per contig there). */
int setContigsGpu(gSuperIntervals* si, size_t n_contigs, const int64_t* offsets);
size_t sizeSuperIntervalsGpu(const gSuperIntervals* si);          /* c_superintervals.h:156 */
size_t numContigsGpu(const gSuperIntervals* si);

/* ---- index: indexSuperIntervals (c_superintervals.h:169, 487-521);
 *      IntervalMap::build (superintervals.hpp:112-130) ---------------------- */
int indexSuperIntervalsGpu(gSuperIntervals* si);
/* Sorted arrays after indexing (starts/ends as the handle's coordinate width;
 * branch is contig-local, -1 where the reference holds SIZE_MAX).  Any pointer
 * may be NULL.  Replaces intervalAt/startAt/endAt/dataAt (c_superintervals.h:176-185) and
 * the public vectors starts/ends/branch/data (superintervals.hpp:49-61). */
int getIndexArraysGpu(const gSuperIntervals* si, void* starts, void* ends, int32_t* data,
                      int64_t* branch);

/* ---- BED ingest: the format step in front of the index
 *      (examples/bed-intersect-si.rs:63-120 read_bed_file / parse_bed_line,
 *      test/bench.cpp:67-102 load_intervals), parsed on the GPU ------------
 * Columns: chrom, start, end (tab-separated; further columns ignored).  Lines
 * that are empty or start with '#', "track" or "browser" are skipped; lines with
 * fewer than three columns or a non-integer start / end are counted as
 * malformed and skipped; with SI_BED_HALF_OPEN the stored end is column 3 - 1
 * (BED ends are exclusive, the index is end-inclusive, as bed-intersect-si.rs
 * does); lines with end < 0 or end < start are skipped (as there); coordinates
 * outside the handle's width are counted and skipped. */
#define SI_BED_HALF_OPEN 1
typedef struct {
    size_t lines, intervals, skipped_headers, malformed, filtered, out_of_range, unknown_contig;
} cBedStats;
/* Replaces the staged intervals with the file's: one contig per distinct chrom
 * name, ids in order of first appearance, intervals of a contig in file order,
 * payload = 0-based line number.  Call indexSuperIntervalsGpu afterwards. */
int ingestBedGpu(gSuperIntervals* si, const char* text, size_t len, int options, cBedStats* stats);
/* Queries from BED text against the handle's contig names: lines on chroms the
 * index does not hold are skipped (counted in unknown_contig); output in file
 * order with each query's contig id and 0-based line number (line may be NULL).
 * SI_ERR_CAPACITY with *n set when capacity is too small. */
int bedQueriesGpu(gSuperIntervals* si, const char* text, size_t len, int options, void* qs, void* qe,
                  int32_t* qcontig, int64_t* line, size_t capacity, size_t* n, cBedStats* stats);
/* Name of contig `contig` after ingestBedGpu (NUL-terminated; *len = length). */
int contigNameGpu(const gSuperIntervals* si, size_t contig, char* buf, size_t cap, size_t* len);

/* ---- index image: the counterpart of the Rust crate's serde derive on
 *      IntervalMap (superintervals.rs:35-44) ---------------------------------
 * One flat little-endian byte image of a built index: header, contig offsets,
 * sorted starts / ends / payloads, branch array, contig names (when known).  serializeIndexGpu writes it
 * into buf (SI_ERR_CAPACITY with the size in *size when cap is too small);
 * deserializeIndexGpu replaces the handle's intervals with the image's and
 * indexes them without sorting (the coordinate width must match the handle's;
 * a corrupt image is rejected with SI_ERR_INVALID).  save/load do the same
 * through a file. */
int serializeIndexGpu(const gSuperIntervals* si, void* buf, size_t cap, size_t* size);
int deserializeIndexGpu(gSuperIntervals* si, const void* buf, size_t len);
int saveIndexGpu(const gSuperIntervals* si, const char* path);
int loadIndexGpu(gSuperIntervals* si, const char* path);

/* ---- options (no reference counterpart) ------------------------------- */
int setQueryPathGpu(gSuperIntervals* si, int path);
int setUpperBoundModeGpu(gSuperIntervals* si, int mode);
/* Tunables of the batched path: sorted queries per tile, candidate slots per
 * tile (shared memory), the query length above which a query takes the
 * per-query walk, and the interval length from which a tile's candidate goes
 * to its "long" list (scanned for every query) instead of being scanned only
 * near each query.  0 keeps the current value (split_len: -1 keeps it, 0 is a
 * valid length).  tile_queries -1 (the default) picks the tile size per batch
 * from its intervals and hits per query; a positive value fixes it.  Results
 * do not depend on these values. */
int setBatchedParamsGpu(gSuperIntervals* si, int tile_queries, int tile_candidates,
                        int64_t long_query_len, int64_t split_len);
int getBatchedParamsGpu(const gSuperIntervals* si, int* tile_queries, int* tile_candidates,
                        int64_t* long_query_len, int64_t* split_len);
/* Further tunables of the batched path (no reference counterpart); results never depend on
 * them.  SI_OPT_EMIT_COPY: 1 writes the section of a tile's long candidates that comes from
 * the long-interval list (intervals at least 32768 long) as copied runs between its few
 * misses, 0 (default) checks every candidate.  SI_OPT_EYTZ_DEPTH: levels of the Eytzinger
 * tree (1-13, 0 automatic), resampled at once when it is the current provider.
 * getBatchedOptionGpu reports the depth in use. */
#define SI_OPT_EMIT_COPY 1
#define SI_OPT_EYTZ_DEPTH 2
int setBatchedOptionGpu(gSuperIntervals* si, int option, int64_t value);
int getBatchedOptionGpu(const gSuperIntervals* si, int option, int64_t* value);
/* Autotuner of the batched path: times full searches on the first `sample`
 * queries of a device-resident batch (sample = 0 or >= nq: the whole batch; a
 * prefix of an unsorted batch is sparser along the genome than the batch, so it
 * stands for the batch's tile shapes only when it keeps the batch's density)
 * and keeps the fastest upper-bound provider,
 * tile size, candidate capacity and length split (coordinate descent from the
 * current values).  flags & SI_TUNE_KEEP_UPPER_BOUND keeps the current upper-bound
 * provider.  The choice stays set on the handle and is also written to `report`
 * as a JSON object (may be NULL).  Results never depend on it. */
#define SI_TUNE_KEEP_UPPER_BOUND 1
int autotuneBatchedGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                       const int32_t* d_qcontig, size_t nq, size_t sample, int flags, char* report,
                       size_t report_len);
/* Device bytes one host-buffer search call may use for a result chunk (by default
 * 1/16 of the device's memory, at least 4 GiB); larger results are emitted in
 * query chunks against it, two chunk buffers alternating so that emit and
 * device-to-host copy overlap.  Each chunk's emit visits every tile of the batch,
 * so fewer, larger chunks cost less GPU time. */
int setOutputBudgetGpu(gSuperIntervals* si, size_t bytes);
/* Per-phase device time of the query pipeline, measured with CUDA events on
 * the stream the phase runs on while profiling is on (it synchronizes after
 * each phase).  Phases: 0 count, 1 scan, 2 emit, 3 query preparation (query
 * sort and upper-bound search of the batched path).  ms and calls hold 4 values. */
int setProfilingGpu(gSuperIntervals* si, int on);
int getPhaseTimesGpu(const gSuperIntervals* si, double* ms, int64_t* calls);
/* Process-wide cap on device bytes the library allocates (0 = no cap). */
int setDeviceBudgetGpu(size_t bytes);
size_t deviceBytesInUseGpu(void);
/* Free and total device memory of `device` (admission control of a serving loop). */
int deviceMemInfoGpu(int device, size_t* free_bytes, size_t* total_bytes);

/* ---- batch queries with HOST buffers.  coordinates: int32 (handle made with
 *      32) or the _i64 forms; qcontig may be NULL (all contig 0). ---------- */
/* countOverlaps (c_superintervals.h:205, 729-756) / count (hpp:651-825) /
 * count_batch (intervalmap.pyx:363-400) */
int countOverlapsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe,
                          const int32_t* qcontig, size_t nq, uint32_t* counts);
int countOverlapsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe,
                              const int32_t* qcontig, size_t nq, uint32_t* counts);
/* anyOverlaps (c_superintervals.h:202, 570-573) / has_overlaps (hpp:865-871):
 * true iff the interval at upper_bound(qe) reaches qs */
int anyOverlapsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe,
                        const int32_t* qcontig, size_t nq, uint8_t* out);
int anyOverlapsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe,
                            const int32_t* qcontig, size_t nq, uint8_t* out);
/* searchIdxs (c_superintervals.h:214, 610-643) / search_idxs (hpp:879-905) /
 * search_idxs_batch (intervalmap.pyx:402-446) */
int searchIdxsBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe,
                       const int32_t* qcontig, size_t nq, int order, cCsrResult* out);
int searchIdxsBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe,
                           const int32_t* qcontig, size_t nq, int order, cCsrResult* out);
/* searchValues (c_superintervals.h:211, 575-608) / search_values (hpp:551-579) /
 * search_values_batch (intervalmap.pyx:448-494): payloads, fully descending */
int searchValuesBatchGpu(gSuperIntervals* si, const int32_t* qs, const int32_t* qe,
                         const int32_t* qcontig, size_t nq, cCsrResult* out);
int searchValuesBatchGpu_i64(gSuperIntervals* si, const int64_t* qs, const int64_t* qe,
                             const int32_t* qcontig, size_t nq, cCsrResult* out);
/* Same, into caller-owned host buffers (e.g. pinned): offsets needs nq+1
 * slots; returns SI_ERR_CAPACITY with *total set when values is too small. */
int searchBatchIntoGpu(gSuperIntervals* si, const void* qs, const void* qe,
                       const int32_t* qcontig, size_t nq, int order, int values_not_idxs,
                       int64_t* offsets, int32_t* values, size_t capacity, size_t* total);

/* ---- batch queries with DEVICE buffers (inputs already in HBM).  stream
 *      may be NULL (the handle's stream).  Same semantics as above. ---------- */
int countOverlapsDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                           const int32_t* d_qcontig, size_t nq, uint32_t* d_counts, void* stream);
int searchDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                    const int32_t* d_qcontig, size_t nq, int order, int values_not_idxs,
                    int64_t* d_offsets, int32_t* d_values, size_t capacity, size_t* total,
                    void* stream);

/* Allocation-free search.  No counterpart in the reference: it exists for callers
 * that cannot allocate device memory while they query (a host whose device memory
 * belongs to another allocator or a fixed pool, or a query thread that must not
 * call cudaMalloc).  Same result as searchDeviceGpu with values_not_idxs = 0 (on
 * the plain path: one warp per query up to 32,768 queries, one thread per query
 * above), into caller-provided device buffers; the
 * scratch it needs sits in one fixed device array inside the library (about
 * 16.1 MiB, held on every device that loads the library until exit), so the call
 * performs no cudaMalloc / cudaFree.  Limit: at most 4,194,304 queries per call
 * (larger batches return SI_ERR_TOO_LARGE).  All calls share that array: calls
 * that overlap on the GPU race and must be serialized by the caller.  The first
 * call on a device looks the array up on that device; make it before any stream
 * capture.  Every call reads the result size back into host memory and waits for
 * `stream`, so it returns with the search finished (and no call can be captured
 * into a graph).  A result larger than
 * `capacity` returns SI_ERR_CAPACITY with the offsets and *total filled and
 * nothing written to d_values, which may be NULL only with capacity 0.  The index
 * must already be built. */
int searchIdxsNoAllocGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                         const int32_t* d_qcontig, size_t nq, int order, int64_t* d_offsets,
                         int32_t* d_values, size_t capacity, size_t* total, void* stream);

/* Upper bound of every query end: contig-local position of the last interval
 * whose start <= qe, or -1.  upperBound (c_superintervals.h:195, 537-568) /
 * IntervalMap::upper_bound (superintervals.hpp:501-516), computed with the
 * provider `mode` (SI_UB_*), which must be the handle's current mode or
 * SI_UB_BINARY.  Device buffers. */
int upperBoundDeviceGpu(gSuperIntervals* si, const void* d_qe, const int32_t* d_qcontig, size_t nq,
                        int mode, int32_t* d_out, void* stream);

/* Same result as searchDeviceGpu (values_not_idxs = 0, plain path), replayed from a CUDA
 * graph: count -> scan -> emit are captured on the first call of a given shape (buffers,
 * size, order, capacity, stream) and replayed by later calls with that shape -- for
 * repeated small batches, where launch overhead dominates.  Never writes past `capacity`;
 * a larger result returns SI_ERR_CAPACITY with *total set. */
int searchDeviceGraphGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                         const int32_t* d_qcontig, size_t nq, int order, int64_t* d_offsets,
                         int32_t* d_values, size_t capacity, size_t* total, void* stream);

/* ---- set operations: intersection / difference of a list of intervals
 *      (the other map A, passed as queries, one per interval of A in the
 *      order A iterates them) against this handle (map B, built).  CSR over the
 *      queries: query i's pieces are [offsets[i], offsets[i+1]).  Coordinates
 *      have the handle's width.  With too small a capacity the call returns
 *      SI_ERR_CAPACITY, sets *total and (host forms) fills offsets. -------- */
/* intersection (c_superintervals.h:286, 921-940; superintervals.hpp:1158-1177
 * IntervalMap::intersection): for each hit h of query i in `order`
 * (SI_ORDER_IDXS_CPP = the C++ class, SI_ORDER_DESC = the C API), the piece
 * [max(qs, starts[h]), min(qe, ends[h])], kept when start <= end; hits[]
 * receives h (contig-local position in the built index) so that the caller
 * applies its combine function (the reference's default keeps A's data). */
int intersectBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qcontig,
                      size_t nq, int order, int64_t* offsets, void* starts, void* ends, int32_t* hits,
                      size_t capacity, size_t* total);
int intersectDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                       const int32_t* d_qcontig, size_t nq, int order, int64_t* d_offsets,
                       void* d_starts, void* d_ends, int32_t* d_hits, size_t capacity, size_t* total,
                       void* stream);
/* difference (c_superintervals.h:292, 950-974; superintervals.hpp:1186-1211):
 * the pieces of each query interval not covered by this map, ascending; each
 * inherits the query's data.  A covered piece reaching the coordinate type's
 * maximum ends the sweep (the reference's end + 1 overflows there). */
int differenceBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qcontig,
                       size_t nq, int64_t* offsets, void* starts, void* ends, size_t capacity,
                       size_t* total);
int differenceDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                        const int32_t* d_qcontig, size_t nq, int64_t* d_offsets, void* d_starts,
                        void* d_ends, size_t capacity, size_t* total, void* stream);

/* ---- keys and coverage ------------------------------------------------- */
/* search_keys (superintervals.hpp:913-938; order SI_ORDER_DESC) / searchKeys
 * (c_superintervals.h:217) and the Python search_keys / search_items
 * (intervalmap.pyx:302-345; order SI_ORDER_IDXS_CPP): each hit's start and end
 * (and payload when data is not NULL), CSR over the queries.  With too small a
 * capacity: SI_ERR_CAPACITY, *total set, offsets filled. */
int searchKeysBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qcontig,
                       size_t nq, int order, int64_t* offsets, void* starts, void* ends, int32_t* data,
                       size_t capacity, size_t* total);
int searchKeysDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                        const int32_t* d_qcontig, size_t nq, int order, int64_t* d_offsets,
                        void* d_starts, void* d_ends, int32_t* d_data, size_t capacity,
                        size_t* total, void* stream);
/* coverage (superintervals.hpp:979-1006, intervalmap.pyx:347-361): per query the
 * number of overlapping intervals and the sum of min(end, qe) - max(start, qs)
 * over them (no +1), in the coordinate type (wrapping on overflow). */
int coverageBatchGpu(gSuperIntervals* si, const void* qs, const void* qe, const int32_t* qcontig,
                     size_t nq, uint64_t* count, void* covered);
int coverageDeviceGpu(gSuperIntervals* si, const void* d_qs, const void* d_qe,
                      const int32_t* d_qcontig, size_t nq, uint64_t* d_count, void* d_covered,
                      void* stream);

/* ---- result helpers: createIndexResult / clearIndexResult /
 *      destroyIndexResult (c_superintervals.h:339-343, 1070-1075) --------- */
cCsrResult createCsrResult(void);
void clearCsrResult(cCsrResult* r);
void destroyCsrResult(cCsrResult* r);

/* ---- small runtime helpers so that hosts need no CUDA headers ---------- */
const char* lastErrorGpu(void);           /* message of the last failing call on this thread */
void* getStreamGpu(gSuperIntervals* si);  /* the handle's cudaStream_t */
int deviceCountGpu(int* count);
int deviceMallocGpu(void** ptr, size_t bytes);
int deviceFreeGpu(void* ptr);
int hostMallocPinnedGpu(void** ptr, size_t bytes);
int hostFreePinnedGpu(void* ptr);
int memcpyGpu(void* dst, const void* src, size_t bytes, void* stream); /* any direction, async */
int streamSynchronizeGpu(void* stream);
int eventCreateGpu(void** ev);
int eventDestroyGpu(void* ev);
int eventRecordGpu(void* ev, void* stream);
int eventElapsedMsGpu(void* start, void* stop, float* ms);
/* Number of kernels this library has launched in this process. */
long long getLaunchCountGpu(void);
/* L2 flush: writes a device buffer larger than L2 on the stream. */
int flushL2Gpu(void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SI_GPU_C_API_H */
