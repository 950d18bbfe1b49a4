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
// deep parts: rows longer than kFirst, each filed at most once a round, cut
// into kPart-arc parts beyond their first kFirst arcs
constexpr long long kChunkItems = kNoAllocMaxArcs / kPart + kNoAllocMaxArcs / (kFirst + 1) + 1;
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
//         [4..7] fill cursors of the second pass, [8] malformed rows,
//         [9] malformed arcs, [10] vertices whose incoming capacity passes int32
__global__ void na_count(const int* row, int n, long long na, int* counts) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && (row[0] != 0 || (long long)row[n] != na)) atomicAdd(counts + 8, 1);
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int d = row[v + 1] - row[v];
    if (d < 0) atomicAdd(counts + 8, 1);
    if (d <= 0) continue;
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

// The caller's arcs, read before any solver kernel indexes with them: heads
// in [0, n), twins in [0, na) and paired (twin of twin is the arc itself),
// capacities >= 0; and each vertex's incoming capacity (the capacities of the
// twins of its row's arcs, which bound its excess) summed in 64 bits and
// compared with int32.  Rows of up to kHeavyDeg arcs are summed by a warp
// each, longer rows by a block per kChunk-arc chunk (the bch items).
__global__ void na_check(const int* row, const int2* arc, const int2* arx, int n, long long na, const int* cls,
                         int n_short, const int4* bch, int n_bch, unsigned long long* insum, int* counts) {
  const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x, gs = (long long)gridDim.x * blockDim.x;
  int bad = 0;
  for (long long a = gt; a < na; a += gs) {
    const int2 r = arc[a], x = arx[a];
    bool ok = r.x >= 0 && r.x < n && x.x >= 0 && (long long)x.x < na && x.y >= 0;
    if (ok) ok = arx[x.x].x == (int)a;
    bad += !ok;
  }
  if (bad) atomicAdd(counts + 9, bad);
  const int lane = threadIdx.x & 31;
  for (long long w = gt >> 5; w < n_short; w += gs >> 5) {
    const int v = cls[w];
    const int b = row[v], e = row[v + 1];
    unsigned long long sum = 0;
    for (int a = b + lane; a < e; a += 32) {
      const int tw = arx[a].x;
      if (tw >= 0 && (long long)tw < na) sum += (unsigned long long)max(arx[tw].y, 0);
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane == 0 && sum > 0x7fffffffull) atomicAdd(counts + 10, 1);
  }
  __shared__ unsigned long long s_sum;
  for (int it = blockIdx.x; it < n_bch; it += gridDim.x) {
    const int4 ch = bch[it];  // {vertex, 0, begin, end}
    if (threadIdx.x == 0) s_sum = 0;
    __syncthreads();
    unsigned long long sum = 0;
    for (int a = ch.z + threadIdx.x; a < ch.w; a += blockDim.x) {
      const int tw = arx[a].x;
      if (tw >= 0 && (long long)tw < na) sum += (unsigned long long)max(arx[tw].y, 0);
    }
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if (lane == 0 && sum) atomicAdd(&s_sum, sum);
    __syncthreads();
    if (threadIdx.x == 0 && s_sum) atomicAdd(insum + ch.x, s_sum);
    __syncthreads();
  }
}

__global__ void na_check_heavy(const int* cls, int first, int nh, const unsigned long long* insum, int* counts) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nh; i += gridDim.x * blockDim.x)
    if (insum[cls[first + i]] > 0x7fffffffull) atomicAdd(counts + 10, 1);
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
      t >= n || s == t || (algo != WBPR_ALGO_TC && algo != WBPR_ALGO_VC)) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: null buffer, terminal out of range or bad algo");
    return WBPR_ERR_INVALID_ARG;
  }
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
  int* vert = base + kOffVert;
  auto va = [&](int i) { return vert + (long long)i * kNoAllocMaxVertices; };
  int* cls = va(14);
  int4* bch = (int4*)(base + kOffBch);
  // The rows are checked before anything sizes work by them: the class list
  // and the chunk items are bounded by the declared arc count only when
  // row[0] == 0, row[n] == num_residual_arcs and no row is negative.
  na_count<<<sms * 2, 256, 0, st>>>(d_row, n, num_residual_arcs, counts);
  NA_CK(cudaGetLastError());
  int hc[11];
  NA_CK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (hc[8]) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: d_row must start at 0, end at num_residual_arcs and never "
                         "decrease");
    return WBPR_ERR_INVALID_ARG;
  }
  na_fill<<<sms * 2, 256, 0, st>>>(d_row, n, counts, cls, bch);
  // the per-vertex incoming-capacity sums borrow two vertex arrays (active
  // lists the solver fills before it reads them)
  unsigned long long* insum = (unsigned long long*)va(4);
  NA_CK(cudaMemsetAsync(insum, 0, sizeof(unsigned long long) * (size_t)n, st));
  na_check<<<sms * 2, 256, 0, st>>>(d_row, arc, arx, n, num_residual_arcs, cls, hc[0] + hc[1], bch, hc[3], insum,
                                    counts);
  na_check_heavy<<<sms, 256, 0, st>>>(cls, hc[0] + hc[1], hc[2], insum, counts);
  NA_CK(cudaGetLastError());
  NA_CK(cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (hc[9]) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: " + std::to_string(hc[9]) +
                         " residual arcs with a head outside [0, n), an unpaired twin or a negative capacity");
    return WBPR_ERR_INVALID_ARG;
  }
  if (hc[10]) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: a vertex's incoming capacities sum past int32");
    return WBPR_ERR_OVERFLOW;
  }
  if (num_residual_arcs > 0) na_reset<<<sms * 4, 256, 0, st>>>(arc, arx, num_residual_arcs);

  Params<TopoB> p{};  // every field zero unless it has its own initializer
  p.g.row = d_row;
  p.g.arc = arc;
  p.g.arx = arx;
  p.g.bd.viol = &ctl->viol;  // bounds counted in the checked build only
  p.g.bd.na = num_residual_arcs;
  p.g.bd.n = n;
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
  p.gr_threshold = (unsigned long long)(kDefaultGrAlpha * ((double)n + (double)num_residual_arcs)) + 1;
  p.gr_rounds = 48;
  p.gr_stall = default_gr_stall((long long)n + num_residual_arcs);
  p.greedy = 1;
  p.gr_plateau = kDefaultPlateau;
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
  NA_CK(launch_pr(p, tile, grid_blocks_for((long long)n + num_residual_arcs, sms, sms * occ), 256, st));
  int res[3] = {0, 0, 0};  // err, viol, excess(t)
  NA_CK(cudaMemcpyAsync(res, &ctl->err, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(res + 1, &ctl->viol, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaMemcpyAsync(res + 2, p.e + t, sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  if (res[0]) {
    wbpr::set_last_error(res[0] == WBPR_ERR_TIMEOUT ? "wbpr_solve_bcsr_noalloc: a grid-barrier wait timed out"
                                                    : "wbpr_solve_bcsr_noalloc: round or time budget exhausted");
    return (wbpr_status)res[0];
  }
  if (res[1]) {
    wbpr::set_last_error("wbpr_solve_bcsr_noalloc: bounds check: " + std::to_string(res[1]) +
                         " out-of-range arc or vertex indices");
    return WBPR_ERR_VERIFY;
  }
  *flow = res[2];
  return WBPR_OK;
}
