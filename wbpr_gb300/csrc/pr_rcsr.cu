// Persistent solver instantiations for the RCSR layout.
#include "pr_launch.h"

namespace wbpr_dev {

template <int W>
static cudaError_t launch_w(const Params<TopoR>& p, int blocks, int threads, cudaStream_t st) {
  void* args[] = {(void*)&p};
  return cudaLaunchCooperativeKernel((const void*)pr_persistent<TopoR, W>, dim3(blocks), dim3(threads),
                                     args, 0, st);
}

cudaError_t launch_pr(const Params<TopoR>& p, int tile, int blocks, int threads, cudaStream_t st) {
  switch (tile) {
    case 1: return launch_w<1>(p, blocks, threads, st);
    case 8: return launch_w<8>(p, blocks, threads, st);
    case 16: return launch_w<16>(p, blocks, threads, st);
    case 32: return launch_w<32>(p, blocks, threads, st);
  }
  return cudaErrorInvalidValue;
}

int occupancy_pr(const Params<TopoR>*, int tile, int threads) {
  int nb = 0;
  cudaError_t e = cudaErrorInvalidValue;
  switch (tile) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pr_persistent<TopoR, 1>, threads, 0); break;
    case 8: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pr_persistent<TopoR, 8>, threads, 0); break;
    case 16: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pr_persistent<TopoR, 16>, threads, 0); break;
    case 32: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pr_persistent<TopoR, 32>, threads, 0); break;
  }
  return e == cudaSuccess ? nb : 0;
}

cudaError_t launch_stranded(const Params<TopoR>& p, int blocks, int threads, cudaStream_t st) {
  count_stranded<TopoR><<<blocks, threads, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace wbpr_dev
