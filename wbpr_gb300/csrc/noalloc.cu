// wbpr_solve_bcsr_noalloc: a maximum-flow solve for callers that cannot
// allocate device memory -- code running under a caller-owned memory pool or
// arena, inside a framework that forbids cudaMalloc on its hot path, or in a
// process whose allocator is not CUDA's.  The caller brings the residual
// graph in device buffers it already owns; every scratch array the solver
// needs (labels, excess, active lists, BFS frontiers, control block) lives in
// one file-scope __device__ array of fixed size, so this entry point calls no
// cudaMalloc, cudaFree or other allocating routine.
//
// Limits: at most kNoAllocMaxVertices vertices and kNoAllocMaxArcs residual
// arcs (two per input arc); larger graphs are refused with
// WBPR_ERR_INVALID_ARG.  The array occupies about 5.6 MB on every device that
// loads the library, until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and caches it; make that
// first call before any stream capture.  All calls share the one array and it
// keeps the last call's contents: each call clears the control block it needs
// zeroed, and calls whose work overlaps on the GPU (different streams or host
// threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "pr_launch.h"
#include "wbpr_internal.h"

using namespace wbpr_dev;

namespace {

constexpr int kNoAllocMaxVertices = 1 << 16;
constexpr long long kNoAllocMaxArcs = 1 << 20;

constexpr long long align_ints(long long x) { return (x + 63) & ~63LL; }
// layout of the scratch array, in 4-byte words
constexpr long long kCtlWords = align_ints((sizeof(Ctl) + 3) / 4);
constexpr long long kStatWords = align_ints((sizeof(Stats) + 3) / 4);
constexpr long long kCountWords = 64;  // classification counters
constexpr int kVertexArrays = 15;      // per-vertex int arrays, indexed as in wbpr_solve_bcsr_noalloc
constexpr long long kTdItems = kNoAllocMaxArcs / kTdChunk + kNoAllocMaxVertices;
// deep entries are rows longer than kFirst, each filed at most once a round
constexpr long long kChunkItems = kNoAllocMaxArcs / kChunk + kNoAllocMaxArcs / (kFirst + 1) + 1;
constexpr long long kBchItems = kNoAllocMaxArcs / kChunk + kNoAllocMaxArcs / (kHeavyDeg + 1) + 1;
constexpr long long kOffStat = kCtlWords;
constexpr long long kOffCount = kOffStat + kStatWords;
constexpr long long kOffVert = kOffCount + kCountWords;
constexpr long long kOffFrh = kOffVert + (long long)kVertexArrays * kNoAllocMaxVertices;
constexpr long long kOffChunk = kOffFrh + 3 * 2 * kTdItems;
constexpr long long kOffBch = kOffChunk + 14 * kChunkItems;  // hrec (3 x int4), hsum, hmin per item
constexpr long long kScratchWords = align_ints(kOffBch + 4 * kBchItems);

static __device__ __align__(256) int g_noalloc_scratch[kScratchWords];

std::mutex g_mu;
int* g_ptr[128] = {nullptr};

// per-device address of the scratch array (looked up once per device)
cudaError_t scratch_ptr(int dev, int** out) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (dev < 0 || dev >= 128) return cudaErrorInvalidDevice;
  if (!g_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = (int*)p;
  }
  *out = g_ptr[dev];
  return cudaSuccess;
}

__global__ void na_reset(int2* arc, const int2* arx, long long na) {
  for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < na;
       a += (long long)gridDim.x * blockDim.x)
    arc[a].y = __ldg(&arx[a].y);
}

// counts: [0] light, [1] medium, [2] heavy, [3] long-row chunks,
//         [4..7] fill cursors of the second pass
__global__ void na_count(const int* row, int n, int* counts) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int d = row[v + 1] - row[v];
    if (d == 0) continue;
    if (d <= kLightDeg) atomicAdd(counts + 0, 1);
    else if (d <= kHeavyDeg) atomicAdd(counts + 1, 1);
    else {
      atomicAdd(counts + 2, 1);
      atomicAdd(counts + 3, (d + kChunk - 1) / kChunk);
    }
  }
}

__global__ void na_fill(const int* row, int n, int* counts, int* cls, int4* bch) {
  const int nl = counts[0], nm = counts[1];
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = row[v], d = row[v + 1] - b;
    if (d == 0) continue;
    if (d <= kLightDeg) {
      cls[atomicAdd(counts + 4, 1)] = v;
    } else if (d <= kHeavyDeg) {
      cls[nl + atomicAdd(counts + 5, 1)] = v;
    } else {
      cls[nl + nm + atomicAdd(counts + 6, 1)] = v;
      const int nch = (d + kChunk - 1) / kChunk;
      const int base = atomicAdd(counts + 7, nch);
      for (int j = 0; j < nch; ++j) bch[base + j] = make_int4(v, 0, b + j * kChunk, min(b + d, b + (j + 1) * kChunk));
    }
  }
}

#define NA_CK(call)                                                          \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess) {                                                 \
      wbpr::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
      return WBPR_ERR_CUDA;                                                  \
    }                                                                        \
  } while (0)

}  // namespace

extern "C" wbpr_status wbpr_solve_bcsr_noalloc(int32_t n, int64_t num_residual_arcs, const int32_t* d_row,
                                               int32_t* d_arc, const int32_t* d_arx, int32_t s, int32_t t,
                                               int32_t algo, void* stream, int64_t* flow) {
  if (n < 2 || n > kNoAllocMaxVertices) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: n must be in [2, 65536]");
    return WBPR_ERR_INVALID_ARG;
  }
  if (num_residual_arcs < 0 || num_residual_arcs > kNoAllocMaxArcs) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: at most 1048576 residual arcs");
    return WBPR_ERR_INVALID_ARG;
  }
  if (!d_row || !flow || (num_residual_arcs > 0 && (!d_arc || !d_arx)) || s < 0 || t < 0 || s >= n ||
      t >= n || s == t || (algo != WBPR_ALGO_TC && algo != WBPR_ALGO_VC))
    return WBPR_ERR_INVALID_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  NA_CK(cudaGetDevice(&dev));
  NA_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int* base = nullptr;
  NA_CK(scratch_ptr(dev, &base));
  Ctl* ctl = (Ctl*)base;
  Stats* stats = (Stats*)(base + kOffStat);
  int* counts = base + kOffCount;
  NA_CK(cudaMemsetAsync(base, 0, sizeof(int) * (size_t)kOffVert, st));
  int2* arc = (int2*)d_arc;
  const int2* arx = (const int2*)d_arx;
  if (num_residual_arcs > 0) na_reset<<<sms * 4, 256, 0, st>>>(arc, arx, num_residual_arcs);
  int* vert = base + kOffVert;
  auto va = [&](int i) { return vert + (long long)i * kNoAllocMaxVertices; };
  int* cls = va(14);
  int4* bch = (int4*)(base + kOffBch);
  na_count<<<sms * 2, 256, 0, st>>>(d_row, n, counts);
  na_fill<<<sms * 2, 256, 0, st>>>(d_row, n, counts, cls, bch);
  NA_CK(cudaGetLastError());
  int hc[4];
  NA_CK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));

  Params<TopoB> p{};  // every field zero unless it has its own initializer
  p.g.row = d_row;
  p.g.arc = arc;
  p.g.arx = arx;
  p.n = n;
  p.s = s;
  p.t = t;
  p.lab = va(0);
  p.e = va(1);
  p.rl_min = va(2);
  p.rl_left = va(3);
  p.lq[0] = va(4);
  p.lq[1] = va(5);
  p.hq[0] = va(6);
  p.hq[1] = va(7);
  p.esnap = va(8);
  p.qraw = va(9);
  p.fr[0] = va(10);
  p.fr[1] = va(11);
  p.fr[2] = va(12);
  p.dmin0 = va(13);
  p.cls = cls;
  for (int k = 0; k < 3; ++k) p.frh[k] = (int2*)(base + kOffFrh) + (long long)k * kTdItems;
  p.hrec = (int4*)(base + kOffChunk);
  p.hsum = base + kOffChunk + 12 * kChunkItems;
  p.hmin = p.hsum + kChunkItems;
  p.bch = bch;
  p.n_light = hc[0];
  p.n_medium = hc[1];
  p.n_heavy = hc[2];
  p.n_bch = hc[3];
  p.ctl = ctl;
  p.st = stats;
  p.total_deg = num_residual_arcs;
  p.gr_threshold = (unsigned long long)(0.75 * ((double)n + (double)num_residual_arcs)) + 1;
  p.gr_rounds = 48;
  p.budget_ns = 120ull * 1000 * 1000 * 1000;
  p.bar_timeout_ns = 10ull * 1000 * 1000 * 1000;
  p.heavy_deg = 32;
  p.mode = kModeFresh;
  p.bfs_excl = s;
  const int tile = algo == WBPR_ALGO_TC ? 1 : 32;
  const int occ = occupancy_pr(&p, tile, 256);
  if (occ <= 0) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: solver kernel does not fit on an SM");
    return WBPR_ERR_CUDA;
  }
  NA_CK(launch_pr(p, tile, sms * occ, 256, st));
  int err = 0, et = 0;
  NA_CK(cudaMemcpyAsync(&err, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(&et, p.e + t, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (err) return (wbpr_status)err;
  *flow = et;
  return WBPR_OK;
}
