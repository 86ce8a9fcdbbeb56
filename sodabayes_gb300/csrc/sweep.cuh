// sweep.cuh — host-side entry points of the sweep kernels (sweep.cu).
#pragma once
#include <cuda_runtime.h>
#include "state.cuh"

namespace soda {

int sweep_chain_count_supported(int chains);
cudaError_t sweep_prepare(int bs);
// Enqueues one Gibbs iteration of every chain on `st` (graph-capturable).
cudaError_t sweep_enqueue_iteration(const Dev &D, const int *blk_sizes, int sm_count, cudaStream_t st);
cudaError_t sweep_enqueue_init(const Dev &D, double vara0, double scale_va0, int sm_count, cudaStream_t st);
cudaError_t sweep_enqueue_recal(const Dev &D, double unused, cudaStream_t st);

}  // namespace soda
