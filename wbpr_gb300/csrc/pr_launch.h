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

// Blocks of the persistent grid for a graph of `units` = n + residual arcs,
// with `full` = SMs x resident blocks per SM.  Smaller graphs run on fewer
// blocks: their rounds and BFS levels are latency-bound, and fewer blocks make
// every phase's barrier and idle block cheaper.  Bands measured on GB300
// (GENRMF, layered, grids, R-MAT); at most 16,384 units one block, whose
// phases are then separated by block barriers only.
constexpr long long kOneBlockUnits = 16384;
inline int grid_blocks_for(long long units, int sms, int full) {
  if (units <= kOneBlockUnits) return 1;
  if (units <= (1LL << 21)) return full < sms / 2 ? full : (sms / 2 > 1 ? sms / 2 : 1);
  if (units <= (1LL << 22)) return full < sms ? full : sms;
  if (units <= (1LL << 24)) return full < 2 * sms ? full : 2 * sms;
  return full;
}

// Global relabel after this many times (n + residual arcs) units of scan work
// (measured on GB300 with the greedy routing on: R-MAT scale 20 and 22 and
// layered networks gain 4-18% over 0.75, R-MAT scale 16 and the 2M x 2M
// matching lose 5-13%; the matching's best is 0.5, which wbpr_autotune finds).
constexpr double kDefaultGrAlpha = 1.0;
// Also relabel globally when the active set shrank by less than 10% over
// this many rounds (0: off).  Measured on GB300 at 4 rounds: the 2M x 2M
// unit-capacity matching 9.7 -> 7.7 ms and R-MAT scale 16 1.26 -> 0.98 ms,
// but R-MAT scale 20/22, layered networks, GENRMF and 512 x 512 grids lose
// 5-50% to extra relabels, so it is off by default and wbpr_autotune tries it.
constexpr int kDefaultPlateau = 0;

// Default of the no-flow-into-t global-relabel trigger (rounds in a row, 0:
// off).  On R-MAT scale 20/22 and the 2M x 2M bipartite graph it cut 5-18%
// of the solve, one round a little more than two after the greedy routing;
// on graphs of at most 2^22 units (GENRMF, layered networks, 512 x 512 grids)
// it ran extra global relabels and cost 0-25%.
inline int default_gr_stall(long long units) { return units > (1LL << 22) ? 1 : 0; }

}  // namespace wbpr_dev
