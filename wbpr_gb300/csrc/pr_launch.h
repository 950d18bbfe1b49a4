// Launch entry points of the persistent solver, one translation unit per
// residual layout so the instantiations compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "pr_kernel.cuh"

namespace wbpr_dev {

cudaError_t launch_pr(const Params<TopoB>& p, int tile, int blocks, int threads, cudaStream_t st);
cudaError_t launch_pr(const Params<TopoR>& p, int tile, int blocks, int threads, cudaStream_t st);
int occupancy_pr(const Params<TopoB>*, int tile, int threads);
int occupancy_pr(const Params<TopoR>*, int tile, int threads);
cudaError_t launch_stranded(const Params<TopoB>& p, int blocks, int threads, cudaStream_t st);
cudaError_t launch_stranded(const Params<TopoR>& p, int blocks, int threads, cudaStream_t st);

}  // namespace wbpr_dev
