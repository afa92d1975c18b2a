// si_batched.cu -- the BATCHED query path (sorted-query tiles).
#include "si_batched.cuh"
#include "si_gpu/c_api.h"

namespace sig {

BatchedWorkspace::~BatchedWorkspace() {
    for (int i = 0; i < 16; ++i)
        if (blocks[i]) cudaFree(blocks[i]);
}

template <typename S>
int batched_prepare(BatchedWorkspace&, MapView<S>, Levels<S>, int, const int64_t*, int, cudaStream_t) {
    return SI_OK;
}

template <typename S>
int batched_count(BatchedWorkspace&, MapView<S> m, Levels<S>, int, const QueryBatch& q, uint32_t* counts,
                  int* d_err, int, cudaStream_t st) {
    return launch_count_plain<S>(m, q, counts, d_err, st) == cudaSuccess ? SI_OK : SI_ERR_CUDA;
}

template <typename S>
int batched_emit(BatchedWorkspace&, MapView<S> m, Levels<S>, int, const QueryBatch& q, const int64_t* offsets,
                 int64_t out_base, int order, bool values, int32_t* out, int* d_err, int, cudaStream_t st) {
    return launch_emit_plain<S>(m, q, offsets, out_base, order, values, out, d_err, st) == cudaSuccess
               ? SI_OK
               : SI_ERR_CUDA;
}

#define SIG_BINST(S)                                                                                  \
    template int batched_prepare<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const int64_t*, int, \
                                    cudaStream_t);                                                   \
    template int batched_count<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const QueryBatch&,    \
                                  uint32_t*, int*, int, cudaStream_t);                               \
    template int batched_emit<S>(BatchedWorkspace&, MapView<S>, Levels<S>, int, const QueryBatch&,     \
                                 const int64_t*, int64_t, int, bool, int32_t*, int*, int, cudaStream_t);
SIG_BINST(int32_t)
SIG_BINST(int64_t)

}  // namespace sig
