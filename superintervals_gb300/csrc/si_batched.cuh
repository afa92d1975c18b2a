// si_batched.cuh -- the BATCHED query path (sorted-query tiles).
#pragma once
#include "si_internal.cuh"

namespace sig {

// Per-handle state of the batched path: query-sort buffers and the per-contig
// upper-bound accelerators.  Grown on demand, released with the handle.
struct BatchedWorkspace {
    void* blocks[16] = {nullptr};
    size_t bytes[16] = {0};
    ~BatchedWorkspace();
};

template <typename S>
int batched_prepare(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const int64_t* lvl_sizes,
                    int ub_mode, cudaStream_t st);
template <typename S>
int batched_count(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q,
                  uint32_t* counts, int* d_err, int ub_mode, cudaStream_t st);
template <typename S>
int batched_emit(BatchedWorkspace& ws, MapView<S> m, Levels<S> L, int H, const QueryBatch& q,
                 const int64_t* offsets, int64_t out_base, int order, bool values, int32_t* out,
                 int* d_err, int ub_mode, cudaStream_t st);

}  // namespace sig
