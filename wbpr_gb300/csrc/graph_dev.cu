// Device graph handle, solve orchestration, certificate check, min-cut
// adjoint and the reference drop-ins of libwbpr.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "devmem.h"
#include "match.h"
#include "pr_launch.h"
#include "wbpr_internal.h"

using namespace wbpr_dev;

// NVTX range around an entry point (a no-op unless a profiler is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

static thread_local std::string g_last_error;

namespace wbpr {
void set_last_error(const std::string& msg) { g_last_error = msg; }

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxDevices] = {};
unsigned long long g_cache_bytes = 16ull << 30;  // release threshold of new pools
}  // namespace

cudaMemPool_t device_pool(int device) {
  if (device < 0 || device >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pools[device]) {
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    unsigned long long thr = g_cache_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    g_pools[device] = pool;
  }
  return g_pools[device];
}

cudaError_t pool_alloc_on(void** p, size_t bytes, cudaStream_t stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = device_pool(dev);
  if (!pool) return cudaErrorMemoryAllocation;
  e = cudaMallocFromPoolAsync(p, bytes, pool, stream);
  if (e == cudaErrorMemoryAllocation) {
    // the free blocks the pool keeps may be of other sizes: hand them back
    // to the driver (blocks in use stay) and map the request anew
    cudaGetLastError();
    cudaStreamSynchronize(stream);
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(p, bytes, pool, stream);
  }
  return e;
}

cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t stream) {
  cudaError_t e = pool_alloc_on(p, bytes, stream);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    cudaFreeAsync(*p, stream);
    *p = nullptr;
  }
  return e;
}
}  // namespace wbpr

#define CK(call)                                                            \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      g_last_error = std::string(#call) + ": " + cudaGetErrorString(e_);    \
      return WBPR_ERR_CUDA;                                                 \
    }                                                                       \
  } while (0)

struct wbpr_graph {
  int device = 0;
  int sms = 0;
  int l2_bytes = 0;
  wbpr_layout layout = WBPR_LAYOUT_BCSR;
  int32_t n = 0;
  int64_t m = 0;
  int32_t s = -1, t = -1;
  cudaStream_t stream = nullptr;  // the stream all of the handle's work goes to
  cudaStream_t own_stream = nullptr;  // the handle's own stream (destroyed with it)
  // terminal sets of the last multi-pair solve
  signed char* term = nullptr;
  int* pairs = nullptr;  // sources then sinks
  int64_t pairs_cap = 0;
  long long* pair_flow = nullptr;
  int* cap_tmp = nullptr;  // staging for wbpr_graph_set_capacities
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
  // BCSR16
  int* row = nullptr;
  int2* arc = nullptr;
  int2* arx = nullptr;
  // RCSR
  int* frow = nullptr;
  int2* farc = nullptr;
  int* fcb = nullptr;
  int* fcap = nullptr;
  int* rrow = nullptr;
  int2* rarc = nullptr;
  // input row offsets (maps input arc i of u to its residual slot)
  int* ioff = nullptr;
  // BCSR16 undo log (pr_kernel.cuh): arcs pushed since the residuals were
  // last restored; `full_reset` asks the next fresh solve to rewrite them all
  int* ulog = nullptr;
  int* ulog_n = nullptr;
  int ulog_cap = 0;
  bool full_reset = false;
  // per-vertex state and scratch
  int* h = nullptr;
  int* e = nullptr;
  int* rl_min = nullptr;
  int* rl_left = nullptr;
  int* lq[2] = {nullptr, nullptr};
  int* hq[2] = {nullptr, nullptr};
  int* esnap = nullptr;
  int* dmin0 = nullptr;
  int4* hrec = nullptr;
  int* hsum = nullptr;
  int* hmin = nullptr;
  int4* bch = nullptr;
  int n_bch = 0;
  int n_td_heavy = 0;
  int* qraw = nullptr;
  int* fr[3] = {nullptr, nullptr, nullptr};
  int2* frh[3] = {nullptr, nullptr, nullptr};
  int64_t n_td_items = 0;
  int* cls = nullptr;
  int* vlab = nullptr;
  int8_t* ind = nullptr;
  int* flow_tmp = nullptr;
  long long* trace = nullptr;
  unsigned long long* bt = nullptr;
  unsigned long long* bt2 = nullptr;
  int trace_cap = 0;
  int trace_n = 0;
  int n_light = 0, n_medium = 0, n_heavy = 0;
  long long total_deg = 0;
  double avg_deg = 0;
  Ctl* ctl = nullptr;
  Stats* st = nullptr;
  // unit-capacity bipartite shape of the terminal pair (mt_s, mt_t), and the
  // matching kernel's arrays (allocated at the first check)
  int mt_s = -1, mt_t = -1;
  bool mt_ok = false;
  int mt_nl = 0, mt_nl_light = 0, mt_nr = 0;
  long long mt_larcs = 0;
  int* mt_lv = nullptr;
  int* mt_rv = nullptr;
  unsigned long long* mt_mate = nullptr;
  int* mt_claim = nullptr;
  int* mt_cy = nullptr;
  int* mt_lmin = nullptr;
  MCtl* mt_ctl = nullptr;
  int64_t bytes = 0;
  std::vector<void*> allocs;
};

namespace {

template <class T>
wbpr_status dalloc(wbpr_graph* g, T** p, size_t count) {
  void* q = nullptr;
  size_t bytes = sizeof(T) * std::max<size_t>(count, 1);
  cudaError_t e = wbpr::pool_alloc(&q, bytes, g->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    g_last_error = std::string("device allocation: ") + cudaGetErrorString(e);
    return WBPR_ERR_CUDA;
  }
  g->allocs.push_back(q);
  g->bytes += (int64_t)bytes;
  *p = (T*)q;
  return WBPR_OK;
}

void release(wbpr_graph* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) {
    // back into the library's pool, in stream order after the handle's work
    cudaStreamSynchronize(g->stream);
    for (void* q : g->allocs) cudaFreeAsync(q, g->stream);
    cudaStreamSynchronize(g->stream);
  }
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->ev2) cudaEventDestroy(g->ev2);
  if (g->ev3) cudaEventDestroy(g->ev3);
  if (g->own_stream) cudaStreamDestroy(g->own_stream);
  delete g;
}

// ---------------------------------------------------------------------------
// small kernels
__global__ void reset_bcsr(int2* arc, const int2* arx, long long na) {
  for (long long a = blockIdx.x * (long long)blockDim.x + threadIdx.x; a < na;
       a += (long long)gridDim.x * blockDim.x)
    arc[a].y = __ldg(&arx[a].y);
}
// Restore the residuals a BCSR16 solve changed: every logged arc and its twin
// get their capacity back, a block per log slot (slot k to block k mod
// blocks).  A slot that overflowed (or `full`) makes it a rewrite of all
// `na` arcs, as reset_bcsr.  The overflow words are read by the block's
// threads together.
__global__ void reset_logged(int2* arc, const int2* arx, long long na, const int* ulog, const int* ulog_n,
                             int cap, int full) {
  int f = full;
  for (int k = threadIdx.x; k < kLogSlots; k += blockDim.x) f |= ulog_n[k * kLogStride + 1];
  if (__syncthreads_or(f)) {
    const long long gt = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long gs = (long long)gridDim.x * blockDim.x;
    for (long long a = gt; a < na; a += gs) arc[a].y = __ldg(&arx[a].y);
    return;
  }
  for (int k = blockIdx.x; k < kLogSlots; k += gridDim.x) {
    const int cnt = min(ulog_n[k * kLogStride], cap);
    const int* lg = ulog + (long long)k * cap;
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
      const int a = lg[i];
      const int2 x = __ldg(arx + a);
      arc[a].y = x.y;
      arc[x.x].y = __ldg(&arx[x.x].y);
    }
  }
}
__global__ void reset_rcsr(int2* farc, int* fcb, const int* fcap, long long m) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m;
       i += (long long)gridDim.x * blockDim.x) {
    farc[i].y = __ldg(fcap + i);
    fcb[i] = 0;
  }
}

struct VerifyAcc {
  int cap_viol;
  int cons_viol;
  int excess_reach;
  int label_viol;
  long long cut;
};

// Arc-parallel walks over a CSR: every warp takes tiles of kTile consecutive
// entries (kTile / 32 per lane, striped so a load instruction is coalesced).
// Lanes 0 and 1 find the rows of the tile's first and last entries by binary
// search over the offsets; each entry then searches between those two rows.
// Rows of any length cost the same per entry (a 262,144-arc row is spread
// over 1,024 warps instead of walked by one).
constexpr int kTile = 256;
struct TileRows {
  int lo, hi;  // off[lo] <= first entry, last entry < off[hi]
};
__device__ __forceinline__ int row_search(const int* off, long long i, int lo, int hi) {
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= i) lo = mid;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ TileRows tile_rows(const int* off, int n, long long base, long long count) {
  const int lane = threadIdx.x & 31;
  int r = 0;
  if (lane < 2) r = row_search(off, lane ? min(base + kTile - 1, count - 1) : base, 0, n);
  TileRows t;
  t.lo = __shfl_sync(0xffffffffu, r, 0);
  t.hi = __shfl_sync(0xffffffffu, r, 1) + 1;
  return t;
}
// The same two rows from a table of every tile's first row (db_tile_rows):
// the last entry of tile t lies before the first of tile t + 1, so its row
// is at most trow[t + 1].
__device__ __forceinline__ TileRows tile_rows_tab(const int* trow, long long base) {
  const long long t = base / kTile;
  TileRows r;
  r.lo = __ldg(trow + t);
  r.hi = __ldg(trow + t + 1) + 1;
  return r;
}
// trow[t] = the row holding entry t * kTile for the tiles t < ntiles of
// count entries, trow[ntiles] = the row of the last entry: one independent
// search per tile, instead of a chain of dependent ones at the start of
// every tile a warp walks
__global__ void db_tile_rows(const int* off, int n, long long count, int* trow) {
  const long long ntiles = (count + kTile - 1) / kTile;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t <= ntiles;
       t += (long long)gridDim.x * blockDim.x)
    trow[t] = row_search(off, t < ntiles ? t * kTile : count - 1, 0, n);
}
#define FOR_TILES(count)                                                                        \
  for (long long base = (blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5)) * kTile; \
       base < (count); base += (long long)gridDim.x * (blockDim.x >> 5) * kTile)

// Sum of v over the run of equal keys ending at this lane (keys are
// non-decreasing across the warp); true on the run's last lane.
__device__ __forceinline__ bool run_sum(int key, bool valid, long long& v) {
  const int lane = threadIdx.x & 31;
  for (int d = 1; d < 32; d <<= 1) {
    const long long y = __shfl_up_sync(0xffffffffu, v, d);
    const int k = __shfl_up_sync(0xffffffffu, key, d);
    if (lane >= d && k == key) v += y;
  }
  const int kn = __shfl_down_sync(0xffffffffu, key, 1);
  const bool vn = __shfl_down_sync(0xffffffffu, valid, 1);
  return valid && (lane == 31 || !vn || kn != key);
}

__device__ __forceinline__ void verify_flush(VerifyAcc* out, int bad, int lv, long long cut) {
  for (int o = 16; o > 0; o >>= 1) {
    bad += __shfl_down_sync(0xffffffffu, bad, o);
    lv += __shfl_down_sync(0xffffffffu, lv, o);
    cut += __shfl_down_sync(0xffffffffu, cut, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (bad) atomicAdd(&out->cap_viol, bad);
    if (lv) atomicAdd(&out->label_viol, lv);
    if (cut) atomicAdd((unsigned long long*)&out->cut, (unsigned long long)cut);
  }
}

// Certificate, arc part (BCSR): capacity pair invariant, label validity, cut
// of the sink side, and each vertex's net residual change into net[].
__global__ void verify_arcs_bcsr(const int* row, const int2* arc, const int2* arx, const int* lab,
                                 const int* h, int n, int s, long long na, long long* net, VerifyAcc* out) {
  const int lane = threadIdx.x & 31;
  int bad = 0, lv = 0;
  long long cut = 0;
  FOR_TILES(na) {
    const TileRows tr = tile_rows(row, n, base, na);
#pragma unroll 1
    for (int k = 0; k < kTile / 32; ++k) {
      const long long a = base + k * 32 + lane;
      const bool ok = a < na;
      int u = -1;
      long long d = 0;
      if (ok) {
        u = row_search(row, a, tr.lo, tr.hi);
        const int2 r = arc[a], x = arx[a];
        const int2 rr = arc[x.x], xr = arx[x.x];
        if (r.y < 0 || (long long)r.y + rr.y != (long long)x.y + xr.y) ++bad;
        d = (long long)r.y - x.y;
        if (x.y > 0 && lab[u] >= n && lab[r.x] < n) cut += x.y;
        const int hu = h[u];
        if (r.y > 0 && u != s && hu < n && hu > h[r.x] + 1) ++lv;
      }
      if (run_sum(u, ok, d) && d) atomicAdd((unsigned long long*)(net + u), (unsigned long long)d);
    }
  }
  verify_flush(out, bad, lv, cut);
}
// RCSR: forward arcs (tails by frow) and reverse entries (tails by rrow)
__global__ void verify_arcs_rcsr(const int* frow, const int2* farc, const int* fcb, const int* fcap,
                                 const int* rrow, const int2* rarc, const int* lab, const int* h, int n, int s,
                                 long long m, long long* net, VerifyAcc* out) {
  const int lane = threadIdx.x & 31;
  int bad = 0, lv = 0;
  long long cut = 0;
  // forward arcs in tiles [0, M), reverse entries in tiles [M, 2M), M = m
  // rounded up to whole tiles, so no tile mixes the two
  const long long M = (m + kTile - 1) / kTile * kTile;
  FOR_TILES(2 * M) {
    const bool rev = base >= M;
    const long long b0 = rev ? base - M : base;
    const int* off = rev ? rrow : frow;
    const TileRows tr = tile_rows(off, n, b0, m);
#pragma unroll 1
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = b0 + k * 32 + lane;
      const bool ok = i < m;
      int u = -1;
      long long d = 0;
      if (ok) {
        u = row_search(off, i, tr.lo, tr.hi);
        const int hu = h[u];
        if (!rev) {
          const int2 r = farc[i];
          const int fb = fcb[i], c = fcap[i];
          if (r.y < 0 || fb < 0 || (long long)r.y + fb != c) ++bad;
          d = -(long long)fb;
          if (c > 0 && lab[u] >= n && lab[r.x] < n) cut += c;
          if (r.y > 0 && u != s && hu < n && hu > h[r.x] + 1) ++lv;
        } else {
          const int2 q = rarc[i];
          const int f = fcb[q.y];
          d = f;
          if (f > 0 && u != s && hu < n && hu > h[q.x] + 1) ++lv;
        }
      }
      if (run_sum(u, ok, d) && d) atomicAdd((unsigned long long*)(net + u), (unsigned long long)d);
    }
  }
  verify_flush(out, bad, lv, cut);
}
// Certificate, vertex part: conservation and excess that still reaches t.
__global__ void verify_vertices(const int* e, const int* lab, const long long* net, int n, int s, int t,
                                VerifyAcc* out) {
  int cv = 0, er = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (v == s) continue;
    const int ev = e[v];
    if (net[v] != (long long)ev) ++cv;
    if (v != t && ev > 0 && lab[v] < n) ++er;
  }
  for (int o = 16; o > 0; o >>= 1) {
    cv += __shfl_down_sync(0xffffffffu, cv, o);
    er += __shfl_down_sync(0xffffffffu, er, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (cv) atomicAdd(&out->cons_viol, cv);
    if (er) atomicAdd(&out->excess_reach, er);
  }
}

// per input arc (tail u, head v): side 0 -> [u cannot reach t, v can];
// side 1 -> [u reachable from s, v not]  (labels < n mark the BFS's set)
__global__ void indicator_kernel(const int* ioff, const int* row, const int2* arc, const int2* farc,
                                 const int* lab, int n, long long m, int side, int8_t* ind) {
  const int lane = threadIdx.x & 31;
  FOR_TILES(m) {
    const TileRows tr = tile_rows(ioff, n, base, m);
#pragma unroll 2
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int u = row_search(ioff, i, tr.lo, tr.hi);
      const int v = row ? arc[row[u] + (int)(i - ioff[u])].x : farc[i].x;
      const bool uin = lab[u] < n, vin = lab[v] < n;
      ind[i] = side == 0 ? (int8_t)(!uin && vin) : (int8_t)(uin && !vin);
    }
  }
}

// the excess of each sink of a multi-pair solve
__global__ void sink_flows(const int* e, const int* sinks, int k, long long* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < k; i += gridDim.x * blockDim.x) out[i] = e[sinks[i]];
}
__global__ void set_terms(signed char* term, const int* pairs, int k) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 2 * k; i += gridDim.x * blockDim.x)
    term[pairs[i]] = i < k ? 1 : 2;
}

// per input arc: flow = capacity - residual
__global__ void flow_kernel(const int* ioff, const int* row, const int2* arc, const int2* arx,
                            const int* fcb, int n, long long m, int* flow) {
  const int lane = threadIdx.x & 31;
  FOR_TILES(m) {
    if (!row) {
      for (int k = 0; k < kTile / 32; ++k) {
        const long long i = base + k * 32 + lane;
        if (i < m) flow[i] = fcb[i];
      }
      continue;
    }
    const TileRows tr = tile_rows(ioff, n, base, m);
#pragma unroll 2
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int u = row_search(ioff, i, tr.lo, tr.hi);
      const int a = row[u] + (int)(i - ioff[u]);
      flow[i] = arx[a].y - arc[a].y;
    }
  }
}

// New capacities, in input order, for a built graph: pass 0 checks them
// (non-negative; incoming sums per head within int32, summed into incap),
// pass 1 writes them (BCSR forward slots' arx.y, RCSR fcap).
__global__ void caps_kernel(const int* ioff, const int* row, const int2* arc, int2* arx, const int2* farc,
                            int* fcap, const int* cap, int n, long long m, int pass, unsigned long long* incap,
                            unsigned long long* bad) {
  const int lane = threadIdx.x & 31;
  bool b = false;
  FOR_TILES(m) {
    const TileRows tr = row ? tile_rows(ioff, n, base, m) : TileRows{0, 0};
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int c = cap[i];
      int a = -1, v;
      if (row) {
        const int u = row_search(ioff, i, tr.lo, tr.hi);
        a = row[u] + (int)(i - ioff[u]);
        v = arc[a].x;
      } else {
        v = farc[i].x;
      }
      if (pass == 0) {
        if (c < 0) b = true;
        else if (c > 0) atomicAdd(incap + v, (unsigned long long)c);
      } else if (row) {
        arx[a].y = c;
      } else {
        fcap[i] = c;
      }
    }
  }
  if (__any_sync(0xffffffffu, b) && lane == 0) atomicOr(bad, 1ull);
}

// ---------------------------------------------------------------------------
// On-device BCSR16 builder.  Produces exactly the layout of the host builder:
// row u holds its forward arcs in input order, then one twin per arc entering
// u in increasing input-arc order.  With inoff = exclusive scan of in-degrees,
// row[u] = off[u] + inoff[u], the forward slot of input arc i (tail u) is
// i + inoff[u], and the twin of the arc at position p of the arcs stably
// sorted by head v is off[v + 1] + p.  The stable sort is an LSD radix sort
// by head over block tiles; the in-degree pass records each arc's position p.
// The input is validated on the way (what the host
// checks only for its own builders): non-decreasing offsets here, heads in
// [0, n) by the sort's first histogram, capacities >= 0 by the forward fill.
// Unit-capacity bipartite shape of (s, t), pass 1: every forward arc of s
// (capacity 1, head neither s nor t) counts its head into cl, every arc into t
// (capacity 1, tail neither s nor t; t's reverse slots) counts its tail into cr.
// (BCSR16: row/arc/arx; RCSR: frow = ioff, farc, fcap and the reverse entries
// rrow/rarc {tail, forward arc id}, with row null)
__global__ void mt_count(const int* row, const int* ioff, const int2* arc, const int2* arx, const int2* farc,
                         const int* fcap, const int* rrow, const int2* rarc, int s, int t, int* cl, int* cr,
                         MCtl* mc) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  bool bad = false;
  const int fs = ioff[s + 1] - ioff[s];
  for (int i = gt; i < fs; i += gs) {
    int x, c;
    if (row) {
      x = arc[row[s] + i].x;
      c = arx[row[s] + i].y;
    } else {
      x = farc[ioff[s] + i].x;
      c = fcap[ioff[s] + i];
    }
    if (c != 1 || x == s || x == t) bad = true;
    else atomicAdd(cl + x, 1);
  }
  // the arcs into t: BCSR16 the twins after t's own arcs, RCSR t's reverse entries
  const int tb = row ? row[t] + (ioff[t + 1] - ioff[t]) : rrow[t], te = row ? row[t + 1] : rrow[t + 1];
  for (int a = tb + gt; a < te; a += gs) {
    int y, c;
    if (row) {
      y = arc[a].x;
      c = arx[arx[a].x].y;
    } else {
      y = rarc[a].x;
      c = fcap[rarc[a].y];
    }
    if (c != 1 || y == s || y == t) bad = true;
    else atomicAdd(cr + y, 1);
  }
  if (bad) atomicOr(&mc->bad, 1);
}
// Pass 2, every input arc u -> v: s -> x with x counted once in cl and never
// in cr; y -> t with y counted once in cr and never in cl; any other arc of
// capacity 1 from a left vertex (cl 1, cr 0) to a right one (cr 1, cl 0).
__global__ void mt_check(const int* ioff, const int* row, const int2* arc, const int2* arx, const int2* farc,
                         const int* fcap, int n, long long m, int s, int t, const int* cl, const int* cr,
                         MCtl* mc) {
  const int lane = threadIdx.x & 31;
  bool bad = false;
  FOR_TILES(m) {
    const TileRows tr = tile_rows(ioff, n, base, m);
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int u = row_search(ioff, i, tr.lo, tr.hi);
      int v, c;
      if (row) {
        const int a = row[u] + (int)(i - ioff[u]);
        v = arc[a].x;
        c = arx[a].y;
      } else {
        v = farc[i].x;
        c = fcap[i];
      }
      if (u == s) bad |= cl[v] != 1 || cr[v] != 0;  // capacity and head checked by pass 1
      else if (v == t) bad |= c != 1 || cr[u] != 1 || cl[u] != 0;
      else bad |= c != 1 || cl[u] != 1 || cr[u] != 0 || cr[v] != 1 || cl[v] != 0;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&mc->bad, 1);
}
// Pass 3: the left vertices (rows of at most `heavy` forward arcs into lv,
// longer ones into hv) and the right vertices into rv.
// A left vertex's arcs are its input arcs (its one incoming arc is s -> x).
__global__ void mt_list(const int* ioff, int n, int heavy, const int* cl, const int* cr, int* lv, int* hv, int* rv,
                        MCtl* mc) {
  long long arcs = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    if (cl[v] == 1) {
      const int d = ioff[v + 1] - ioff[v];
      arcs += d;
      if (d > heavy) append(hv, &mc->nlist[1], v);
      else append(lv, &mc->nlist[0], v);
    } else if (cr[v] == 1) {
      append(rv, &mc->nlist[2], v);
    }
  }
  for (int o = 16; o > 0; o >>= 1) arcs += __shfl_down_sync(0xffffffffu, arcs, o);
  if ((threadIdx.x & 31) == 0 && arcs) atomicAdd((unsigned long long*)&mc->larcs, (unsigned long long)arcs);
}

__global__ void db_check_off(const int* off, int n, unsigned long long* bad) {
  bool b = false;
  for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < n; u += (long long)gridDim.x * blockDim.x)
    if (off[u + 1] < off[u]) b = true;
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1ull);
}
// In-degrees from the heads sorted ascending (all checked to lie in [0, n)):
// the first position p0 of a head's run adds -p0, its last position p1 adds
// p1 + 1, so indeg[v] ends as the run length.  Two atomics per head, on
// distinct words, instead of one per arc on a few hot ones.
// Four positions per thread from one 16-byte load (and the two neighbours).
__global__ void db_indeg_sorted(const int* skey, long long m, int* indeg) {
  const long long gs = (long long)gridDim.x * blockDim.x, m4 = m >> 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < m4; q += gs) {
    const int4 k = __ldcs(reinterpret_cast<const int4*>(skey) + q);
    const long long p = 4 * q;
    // heads lie in [0, n): -1 marks the ends of the array
    const int ks[6] = {p > 0 ? __ldg(skey + p - 1) : -1, k.x, k.y, k.z, k.w, p + 4 < m ? __ldg(skey + p + 4) : -1};
#pragma unroll
    for (int j = 1; j <= 4; ++j) {
      if (ks[j - 1] != ks[j]) atomicAdd(indeg + ks[j], -(int)(p + j - 1));
      if (ks[j + 1] != ks[j]) atomicAdd(indeg + ks[j], (int)(p + j));
    }
  }
  for (long long p = 4 * m4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m; p += gs) {
    const int v = skey[p];
    if (p == 0 || skey[p - 1] != v) atomicAdd(indeg + v, -(int)p);
    if (p == m - 1 || skey[p + 1] != v) atomicAdd(indeg + v, (int)p + 1);
  }
}
__global__ void db_max(const unsigned long long* incap, int n, unsigned long long* out) {
  unsigned long long mx = 0;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) mx = max(mx, incap[u]);
  for (int d = 16; d; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
  if ((threadIdx.x & 31) == 0 && mx) atomicMax(out, mx);
}
__global__ void db_row(const int* off, const int* inoff, int n, int* row) {
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u <= n; u += gridDim.x * blockDim.x) row[u] = off[u] + inoff[u];
}

constexpr int kScanTile = 4096;  // 1024 threads x 4 items
__global__ void __launch_bounds__(1024) db_scan_tiles(int* data, long long count, int* sums) {
  __shared__ int s_w[32];
  const long long base = (long long)blockIdx.x * kScanTile + 4LL * threadIdx.x;
  int v[4], t = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = base + k < count ? data[base + k] : 0;
    t += v[k];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int inc = t;
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) s_w[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int w = s_w[lane];
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += y;
    }
    s_w[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  int run = (wid ? s_w[wid - 1] : 0) + inc - t;  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (base + k < count) data[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == blockDim.x - 1 && sums) sums[blockIdx.x] = run;
}
__global__ void db_scan_add(int* data, long long count, const int* sums) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    data[i] += sums[i / kScanTile];
}

// Radix sort by head, 8-bit digits, stable.  A tile is one block of 8 warps
// x kSortRounds rounds x 32 arcs; warp w holds arcs [w * 32 * kSortRounds,
// (w + 1) * 32 * kSortRounds) of the tile, round-major, so (warp, round,
// lane) order is input order.  Lanes holding the same digit are found with
// eight ballots (one per digit bit).  The scatter pass first sorts its tile
// in shared memory (digit, then input order), then writes each digit's run
// to its global place, so consecutive threads write consecutive slots.
constexpr int kSortRounds = 16;
constexpr int kHeadChunks = 4;  // pieces the heads are copied in
constexpr int kSortTile = 8 * kSortRounds * 32;  // 4096 arcs
__device__ __forceinline__ unsigned digit_peers(int d, bool ok) {
  unsigned peers = __ballot_sync(0xffffffffu, ok);
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    const bool bit = (d >> b) & 1;
    const unsigned x = __ballot_sync(0xffffffffu, bit);
    peers &= bit ? x : ~x;
  }
  return peers;
}
// n_check > 0 (the first pass): also flag keys outside [0, n_check).  Each
// warp counts into its own shared histogram (lanes of one warp with equal
// digits are the only conflicts), summed at the end.  Block b counts tile
// tile0 + b.
__global__ void __launch_bounds__(256) db_sort_hist(const int* key, long long m, int shift, int ntiles, int tile0,
                                                    int* hist, int n_check, unsigned long long* bad) {
  __shared__ int cnt[8][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x + tile0;
#pragma unroll
  for (int j = 0; j < 8; ++j) cnt[j][threadIdx.x] = 0;
  __syncthreads();
  const long long base = (long long)tile * kSortTile + (long long)w * kSortRounds * 32;
  bool b = false;
  // all of the lane's keys in flight first, then the counts
  int k[kSortRounds];
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    const long long i = base + r * 32 + lane;
    k[r] = i < m ? __ldcs(key + i) : 0;
  }
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    if (base + r * 32 + lane < m) {
      if (n_check > 0 && (k[r] < 0 || k[r] >= n_check)) b = true;
      atomicAdd(&cnt[w][(k[r] >> shift) & 255], 1);
    }
  }
  if (__any_sync(0xffffffffu, b) && lane == 0) atomicOr(bad, 1ull);
  __syncthreads();
  int t = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) t += cnt[j][threadIdx.x];
  hist[(long long)threadIdx.x * ntiles + tile] = t;
}
// four blocks per SM (64 registers): with 3 (79 registers) the create took 5.30 ms at scale 22,
// with 4 5.28-5.29
__global__ void __launch_bounds__(256, 4) db_sort_scatter(const int* kin, const int* vin, long long m, int shift,
                                                       int ntiles, const int* hist, int* kout, int* vout) {
  __shared__ int wc[8][256];     // per-warp digit counts, then each warp's start within its digit
  __shared__ int dstart[256];    // tile-local start of each digit
  __shared__ int gofs[256];      // global start of this tile's run of each digit
  __shared__ int sk[kSortTile], sv[kSortTile];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, t = threadIdx.x;
  const int tile = blockIdx.x;
  const unsigned lt = (1u << lane) - 1;
  for (int j = 0; j < 8; ++j) wc[j][t] = 0;
  gofs[t] = hist[(long long)t * ntiles + tile];
  __syncthreads();
  const long long base = (long long)tile * kSortTile + (long long)w * kSortRounds * 32;
  int key[kSortRounds], val[kSortRounds], rk[kSortRounds];
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    const long long i = base + r * 32 + lane;
    const bool ok = i < m;
    key[r] = ok ? kin[i] : -1;
    val[r] = ok ? (vin ? vin[i] : (int)i) : 0;
  }
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    const bool ok = key[r] >= 0;
    const int d = ok ? (key[r] >> shift) & 255 : 0;
    const unsigned peers = digit_peers(d, ok);
    rk[r] = ok ? wc[w][d] + __popc(peers & lt) : 0;
    __syncwarp();
    if (ok && lane == __ffs(peers) - 1) wc[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // per digit t: each warp's start among the tile's arcs of that digit, and
  // the digit's total; then the tile-local digit starts by a block scan
  int tot = 0;
  for (int j = 0; j < 8; ++j) {
    const int c = wc[j][t];
    wc[j][t] = tot;
    tot += c;
  }
  int inc = tot;
  for (int d = 1; d < 32; d <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  __shared__ int ws[8];
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  int wpre = 0;
  for (int j = 0; j < w; ++j) wpre += ws[j];
  dstart[t] = wpre + inc - tot;
  __syncthreads();
#pragma unroll
  for (int r = 0; r < kSortRounds; ++r) {
    if (key[r] < 0) continue;
    const int d = (key[r] >> shift) & 255;
    const int lp = dstart[d] + wc[w][d] + rk[r];
    sk[lp] = key[r];
    sv[lp] = val[r];
  }
  __syncthreads();
  const int cnt = (int)min((long long)kSortTile, m - (long long)tile * kSortTile);
  for (int i = t; i < cnt; i += 256) {
    const int k = sk[i];
    const int d = (k >> shift) & 255;
    const int pos = gofs[d] + (i - dstart[d]);
    kout[pos] = k;
    vout[pos] = sv[i];
  }
}

// The largest capacity (warp maxima, one atomic a warp).
__device__ __forceinline__ void warp_cap_max(int c, unsigned long long* out) {
  const int w = __reduce_max_sync(0xffffffffu, max(c, 0));
  if ((threadIdx.x & 31) == 0 && w > 0) atomicMax(out, (unsigned long long)w);
}
// The largest in-degree, from the scanned in-offsets.
__global__ void db_indeg_max(const int* inoff, int n, unsigned long long* out) {
  int mx = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
    mx = max(mx, inoff[v + 1] - inoff[v]);
  mx = __reduce_max_sync(0xffffffffu, mx);
  if ((threadIdx.x & 31) == 0 && mx > 0) atomicMax(out, (unsigned long long)mx);
}
// Whether some head's incoming capacities could pass int32: only then are
// they summed (largest capacity x largest in-degree bounds every sum).
__device__ __forceinline__ bool incap_needed(const unsigned long long* bound) {
  return bound[0] * bound[1] > 0x7fffffffull;
}

// forward slots, arc-parallel (tails as in the tile walk above); the tail of
// every arc for the twin pass; the largest capacity into bound[0]; flags
// negative capacities
__global__ void db_fill_fwd(const int* off, const int* trow, const int* inoff, const int* dst, const int* cap,
                            const int* pos_of, long long m, int2* arc, int2* arx, int* tail,
                            unsigned long long* bad, unsigned long long* bound) {
  const int lane = threadIdx.x & 31;
  bool b = false;
  int cm = 0;
  FOR_TILES(m) {
    const TileRows tr = tile_rows_tab(trow, base);
#pragma unroll 4
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int u = row_search(off, i, tr.lo, tr.hi);
      const int v = dst[i], c = cap ? cap[i] : 1;
      if (c < 0) b = true;
      cm = max(cm, c);
      const int f = (int)i + __ldg(inoff + u);
      const int r = __ldg(off + v + 1) + pos_of[i];
      arc[f] = make_int2(v, c);
      arx[f] = make_int2(r, c);
      tail[i] = u;
    }
  }
  if (__any_sync(0xffffffffu, b) && lane == 0) atomicOr(bad, 1ull);
  warp_cap_max(cm, bound);
}
// Sum of x over the lanes from this one to the end of its run of equal keys
// (keys ascending across the warp, so a run is a block of adjacent lanes);
// the first lane of a run gets the run's sum.
__device__ __forceinline__ unsigned long long run_suffix_sum(int key, unsigned long long x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_down_sync(0xffffffffu, x, d);
    const int ky = __shfl_down_sync(0xffffffffu, key, d);
    if (lane + d < 32 && ky == key) x += y;
  }
  return x;
}
// twin slots in sorted order: the twin of sorted position p is off[v + 1] + p,
// so consecutive p write consecutive slots, and the forward slot of arc i
// from tail u is i + inoff[u]; when the bound asks for it, every head also
// gets the sum of its incoming capacities (one atomic per run of the head
// within a warp)
__global__ void db_fill_twin(const int* off, const int* inoff, const int* skey, const int* sval, const int* tail,
                             const int* cap, const unsigned long long* bound, long long m, int2* arc, int2* arx,
                             unsigned long long* incap) {
  const int lane = threadIdx.x & 31;
  const long long gs = (long long)gridDim.x * blockDim.x;
  const bool sum = incap_needed(bound);
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < m; base += gs) {
    const long long p = base + lane;
    int v = -1;
    unsigned long long c = 0;
    if (p < m) {
      v = skey[p];
      const int i = sval[p];
      const int u = tail[i];
      const int r = __ldg(off + v + 1) + (int)p;
      arc[r] = make_int2(u, 0);
      arx[r] = make_int2(i + __ldg(inoff + u), 0);
      if (sum) c = cap ? (unsigned long long)max(cap[i], 0) : 1ull;
    }
    if (sum) {
      const unsigned long long t = run_suffix_sum(v, c);
      const int vp = __shfl_up_sync(0xffffffffu, v, 1);
      if (v >= 0 && (lane == 0 || vp != v) && t) atomicAdd(incap + v, t);
    }
  }
}

// pos_of[sval[p]] = p for the arcs with id in [lo, hi).  A pass over all of
// sval scatters 4-byte writes over the whole array, and the L2 writes most of
// its sectors back to DRAM only partly filled; with the ids in a window of
// half the L2, each sector is complete before it leaves.  The sorted ids are
// read with an evict-first hint so that they do not push the window out.
__global__ void db_pos_window(const int* sval, long long m, int lo, int hi, int* pos_of) {
  const long long gs = (long long)gridDim.x * blockDim.x;
  const long long m4 = m >> 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < m4; q += gs) {
    const int4 i = __ldcs(reinterpret_cast<const int4*>(sval) + q);
    const int p = (int)(4 * q);
    if (i.x >= lo && i.x < hi) pos_of[i.x] = p;
    if (i.y >= lo && i.y < hi) pos_of[i.y] = p + 1;
    if (i.z >= lo && i.z < hi) pos_of[i.z] = p + 2;
    if (i.w >= lo && i.w < hi) pos_of[i.w] = p + 3;
  }
  for (long long p = 4 * m4 + blockIdx.x * (long long)blockDim.x + threadIdx.x; p < m; p += gs) {
    const int i = sval[p];
    if (i >= lo && i < hi) pos_of[i] = (int)p;
  }
}

// A row is one or two segments of offset arrays: BCSR [o1[u], o1[u+1]);
// RCSR forward arcs [o1[u], o1[u+1]) then reverse entries [o2[u], o2[u+1]).
__device__ __forceinline__ int seg_len(const int* o, int u) { return o ? __ldg(o + u + 1) - __ldg(o + u) : 0; }

// length classes (flags for three stable compactions) and the chunk counts
// cnt: [0] rows > kTdHeavy [1] their top-down chunk items [2] bound on the deep
// parts of a push phase (every vertex is filed at most once a round)
__global__ void db_classify(const int* o1, const int* o2, int n, int* f0, int* f1, int* f2,
                            unsigned long long* cnt) {
  unsigned long long a = 0, b = 0, c = 0;
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u <= n; u += gridDim.x * blockDim.x) {
    const int d = u < n ? seg_len(o1, u) + seg_len(o2, u) : 0;
    f0[u] = d > 0 && d <= kLightDeg;
    f1[u] = d > kLightDeg && d <= kHeavyDeg;
    f2[u] = d > kHeavyDeg;
    if (d > kFirst) c += (d - kFirst + kPart - 1) / kPart;  // deep parts of the row
    if (d > kTdHeavy) {
      a += 1;
      b += (d + kTdChunk - 1) / kTdChunk;
    }
  }
  for (int s = 16; s; s >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, s);
    b += __shfl_xor_sync(0xffffffffu, b, s);
    c += __shfl_xor_sync(0xffffffffu, c, s);
  }
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd(cnt + 0, a);
    if (b) atomicAdd(cnt + 1, b);
    if (c) atomicAdd(cnt + 2, c);
  }
}
__global__ void db_cls_scatter(const int* o1, const int* o2, int n, const int* s0, const int* s1, const int* s2,
                               int* cls) {
  const int n0 = s0[n], n01 = n0 + s1[n];
  for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
    const int d = seg_len(o1, u) + seg_len(o2, u);
    if (d == 0) continue;
    if (d <= kLightDeg) cls[s0[u]] = u;
    else if (d <= kHeavyDeg) cls[n0 + s1[u]] = u;
    else cls[n01 + s2[u]] = u;
  }
}
// chunk items of heavy row j: kChunk pieces of each segment
__global__ void db_heavy_chunks(const int* o1, const int* o2, const int* hcls, int nh, int* nch) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j <= nh; j += gridDim.x * blockDim.x) {
    if (j == nh) {
      nch[j] = 0;
    } else {
      const int u = hcls[j];
      nch[j] = (seg_len(o1, u) + kChunk - 1) / kChunk + (seg_len(o2, u) + kChunk - 1) / kChunk;
    }
  }
}
__global__ void db_bch_fill(const int* o1, const int* o2, const int* hcls, int nh, const int* cbase,
                            int4* bch) {
  for (int j = blockIdx.x; j < nh; j += gridDim.x) {
    const int u = hcls[j];
    int at = cbase[j];
    for (int k = 0; k < 2; ++k) {
      const int* o = k ? o2 : o1;
      if (!o) break;
      const int b = o[u], e = o[u + 1];
      const int nc = (e - b + kChunk - 1) / kChunk;
      for (int q = threadIdx.x; q < nc; q += blockDim.x)
        bch[at + q] = make_int4(u, k, b + q * kChunk, min(e, b + (q + 1) * kChunk));
      at += nc;
    }
  }
}

// RCSR forward arcs in input order, and the tail of every input arc; flags
// negative capacities
__global__ void db_rcsr_fwd(const int* off, const int* trow, const int* dst, const int* cap, long long m,
                            int2* farc, int* fcap, int* fcb, int* tail, unsigned long long* bad,
                            unsigned long long* bound) {
  const int lane = threadIdx.x & 31;
  bool b = false;
  int cm = 0;
  FOR_TILES(m) {
    const TileRows tr = tile_rows_tab(trow, base);
#pragma unroll 4
    for (int k = 0; k < kTile / 32; ++k) {
      const long long i = base + k * 32 + lane;
      if (i >= m) break;
      const int c = cap ? cap[i] : 1;
      if (c < 0) b = true;
      cm = max(cm, c);
      farc[i] = make_int2(dst[i], c);
      fcap[i] = c;
      fcb[i] = 0;
      tail[i] = row_search(off, i, tr.lo, tr.hi);
    }
  }
  if (__any_sync(0xffffffffu, b) && lane == 0) atomicOr(bad, 1ull);
  warp_cap_max(cm, bound);
}
// RCSR reverse entries: position p of the arcs stably sorted by head holds
// {tail, forward arc id} (the reference's rdestinations / flow_index); heads
// get the sum of their incoming capacities as in db_fill_twin
__global__ void db_rcsr_rev(const int* skey, const int* sval, const int* tail, const int* fcap,
                            const unsigned long long* bound, long long m, int2* rarc, unsigned long long* incap) {
  const int lane = threadIdx.x & 31;
  const long long gs = (long long)gridDim.x * blockDim.x;
  const bool sum = incap_needed(bound);
  for (long long base = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < m; base += gs) {
    const long long p = base + lane;
    int v = -1;
    unsigned long long c = 0;
    if (p < m) {
      v = skey[p];
      const int i = sval[p];
      rarc[p] = make_int2(__ldg(tail + i), i);
      if (sum) c = (unsigned long long)max(__ldg(fcap + i), 0);
    }
    if (sum) {
      const unsigned long long t = run_suffix_sum(v, c);
      const int vp = __shfl_up_sync(0xffffffffu, v, 1);
      if (v >= 0 && (lane == 0 || vp != v) && t) atomicAdd(incap + v, t);
    }
  }
}

// exclusive scan of data[0, count) in place (int32 totals)
wbpr_status device_scan(int* data, long long count, cudaStream_t st) {
  const long long tiles = (count + kScanTile - 1) / kScanTile;
  if (tiles <= 1) {
    db_scan_tiles<<<1, 1024, 0, st>>>(data, count, nullptr);
    CK(cudaGetLastError());
    return WBPR_OK;
  }
  int* sums = nullptr;
  CK(wbpr::pool_alloc_on((void**)&sums, sizeof(int) * tiles, st));
  db_scan_tiles<<<(unsigned)tiles, 1024, 0, st>>>(data, count, sums);
  cudaError_t e = cudaGetLastError();
  wbpr_status r = e == cudaSuccess ? device_scan(sums, tiles, st) : WBPR_ERR_CUDA;
  if (r == WBPR_OK) {
    db_scan_add<<<1024, 256, 0, st>>>(data, count, sums);
    e = cudaGetLastError();
    if (e != cudaSuccess) r = WBPR_ERR_CUDA;
  }
  cudaFreeAsync(sums, st);
  if (e != cudaSuccess) g_last_error = std::string("device scan: ") + cudaGetErrorString(e);
  return r;
}

// Builds the residual graph of g->layout in HBM from the input CSR:
// BCSR row/arc/arx or RCSR frow/farc/fcb/fcap/rrow/rarc, plus ioff, the
// length classes cls, the heavy-row chunks bch, hrec/hsum/hmin and counts.
wbpr_status build_device(wbpr_graph* g, const wbpr_csr* in) {
  NvtxRange nvtx_("device build");
  const int n = g->n;
  const long long m = g->m;
  cudaStream_t st = g->stream;
  const int blocks = g->sms * 8;
  const bool bcsr = g->layout == WBPR_LAYOUT_BCSR;
  wbpr_status rs;
  if (bcsr) {
    if ((rs = dalloc(g, &g->row, (size_t)n + 1))) return rs;
    if ((rs = dalloc(g, &g->arc, (size_t)(2 * m)))) return rs;
    if ((rs = dalloc(g, &g->arx, (size_t)(2 * m)))) return rs;
  } else {
    if ((rs = dalloc(g, &g->frow, (size_t)n + 1))) return rs;
    if ((rs = dalloc(g, &g->farc, (size_t)m))) return rs;
    if ((rs = dalloc(g, &g->fcb, (size_t)m))) return rs;
    if ((rs = dalloc(g, &g->fcap, (size_t)m))) return rs;
    if ((rs = dalloc(g, &g->rrow, (size_t)n + 1))) return rs;
    if ((rs = dalloc(g, &g->rarc, (size_t)m))) return rs;
  }
  if ((rs = dalloc(g, &g->ioff, (size_t)n + 1))) return rs;
  // every temporary is carved from one pool allocation, freed when the
  // build ends
  char* slab = nullptr;
  size_t slab_at = 0, slab_size = 0;
  cudaStream_t side = nullptr;
  cudaEvent_t side_done = nullptr;
  cudaEvent_t head_done[kHeadChunks] = {};
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    if (side) cudaStreamSynchronize(side);
    if (slab) cudaFreeAsync(slab, st);
    if (side_done) cudaEventDestroy(side_done);
    for (cudaEvent_t& e : head_done)
      if (e) {
        cudaEventDestroy(e);
        e = nullptr;
      }
    if (side) cudaStreamDestroy(side);
    slab = nullptr;
    side = nullptr;
    side_done = nullptr;
  };
  auto talloc = [&](size_t bytes) -> void* {
    bytes = (std::max<size_t>(bytes, 16) + 255) & ~(size_t)255;
    if (!slab || slab_at + bytes > slab_size) return nullptr;
    void* p = slab + slab_at;
    slab_at += bytes;
    return p;
  };
#define DB(x)                                                         \
  do {                                                                \
    cudaError_t e_ = (x);                                             \
    if (e_ != cudaSuccess) {                                          \
      g_last_error = std::string(#x) + ": " + cudaGetErrorString(e_); \
      cleanup();                                                      \
      return WBPR_ERR_CUDA;                                           \
    }                                                                 \
  } while (0)
#define DBS(x)          \
  do {                  \
    rs = (x);           \
    if (rs) {           \
      cleanup();        \
      return rs;        \
    }                   \
  } while (0)
  const int ntiles = (int)((m + kSortTile - 1) / kSortTile);
  // sort buffers double as the three class-flag arrays, the histogram as the
  // heavy-row chunk bases: size them for both uses
  const size_t mv = std::max<size_t>((size_t)m, (size_t)n + 1);
  const size_t nh_max = std::max<size_t>((size_t)ntiles * 256 + 1, (size_t)n + 1);
  slab_size = 256 * 16 + 4 * (size_t)m * (in->capacities ? 2 : 1) + 4 * ((size_t)n + 1) +
              8 * ((size_t)n + 1) + 64 + 16 * mv + 4 * nh_max + 4 * (size_t)m + (bcsr ? 4 * (size_t)m : 0) +
              4 * ((size_t)m / kTile + 2);
  if (wbpr::pool_alloc((void**)&slab, slab_size, st) != cudaSuccess) {
    cudaGetLastError();
    slab = nullptr;
    g_last_error = "device build: out of device memory";
    return WBPR_ERR_CUDA;
  }
  bool ev_ok = true;
  for (cudaEvent_t& e : head_done) ev_ok = ev_ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
  if (!ev_ok || cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&side_done, cudaEventDisableTiming) != cudaSuccess) {
    g_last_error = std::string("device build: ") + cudaGetErrorString(cudaGetLastError());
    cleanup();
    return WBPR_ERR_CUDA;
  }
  int* d_dst = (int*)talloc(4 * (size_t)m);
  int* d_cap = in->capacities ? (int*)talloc(4 * (size_t)m) : nullptr;
  int* inoff = (int*)talloc(4 * ((size_t)n + 1));
  auto* incap = (unsigned long long*)talloc(8 * ((size_t)n + 1));
  auto* cnt = (unsigned long long*)talloc(8 * 8);
  int* kb[2] = {(int*)talloc(4 * mv), (int*)talloc(4 * mv)};
  int* vb[2] = {(int*)talloc(4 * mv), (int*)talloc(4 * mv)};
  int* hist = (int*)talloc(4 * nh_max);
  int* tail = (int*)talloc(4 * (size_t)m);  // BCSR: sorted position of each arc; RCSR: its tail
  int* utail = bcsr ? (int*)talloc(4 * (size_t)m) : tail;  // BCSR: the tail of each arc (RCSR keeps it in tail)
  int* trow = (int*)talloc(4 * ((size_t)m / kTile + 2));
  if (!d_dst || (in->capacities && !d_cap) || !inoff || !incap || !cnt || !kb[0] || !kb[1] || !vb[0] || !vb[1] ||
      !hist || !tail || !utail || !trow) {
    cudaGetLastError();
    g_last_error = "device build: out of device memory";
    cleanup();
    return WBPR_ERR_CUDA;
  }
  // Heads first: the sort needs only them, so it runs while the capacities
  // are copied on a second stream.  The heads come in kHeadChunks pieces on
  // that stream, and the first pass's histogram of each piece runs while the
  // next one is copied.  The in-degrees come from the sorted heads.
  DB(cudaMemcpyAsync(g->ioff, in->offsets, 4 * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
  // the side stream uses the pool's slab only after its allocation on st
  DB(cudaEventRecord(side_done, st));
  DB(cudaStreamWaitEvent(side, side_done, 0));
  const int nchunks = (int)std::min<long long>(kHeadChunks, ntiles);
  const long long tpc = nchunks ? (ntiles + nchunks - 1) / nchunks : 0;  // tiles per piece
  for (int k = 0; k < nchunks; ++k) {
    const long long a0 = k * tpc * kSortTile, a1 = std::min<long long>(m, (k + 1) * tpc * kSortTile);
    if (a1 <= a0) break;
    DB(cudaMemcpyAsync(d_dst + a0, in->destinations + a0, 4 * (size_t)(a1 - a0), cudaMemcpyHostToDevice, side));
    DB(cudaEventRecord(head_done[k], side));
  }
  DB(cudaMemsetAsync(inoff, 0, 4 * ((size_t)n + 1), st));
  DB(cudaMemsetAsync(incap, 0, 8 * ((size_t)n + 1), st));
  DB(cudaMemsetAsync(cnt, 0, 8 * 8, st));
  db_check_off<<<blocks, 256, 0, st>>>(g->ioff, n, cnt + 6);
  DB(cudaGetLastError());
  if (m) {
    db_tile_rows<<<blocks, 256, 0, st>>>(g->ioff, n, m, trow);
    DB(cudaGetLastError());
  }
  const int bits = n > 1 ? 32 - __builtin_clz((unsigned)(n - 1)) : 1;
  const int passes = (bits + 7) / 8;
  const int* skey = kb[(passes - 1) & 1];
  const int* sval = vb[(passes - 1) & 1];
  if (m) {
    const unsigned sblocks = (unsigned)ntiles;
    for (int p = 0; p < passes; ++p) {
      const int* kin = p ? kb[(p - 1) & 1] : d_dst;
      const int* vin = p ? vb[(p - 1) & 1] : nullptr;
      if (p == 0) {
        for (int k = 0; k < nchunks; ++k) {
          const long long t0 = k * tpc, t1 = std::min<long long>(ntiles, t0 + tpc);
          if (t1 <= t0) break;
          DB(cudaStreamWaitEvent(st, head_done[k], 0));
          db_sort_hist<<<(unsigned)(t1 - t0), 256, 0, st>>>(kin, m, 0, ntiles, (int)t0, hist, n, cnt + 6);
          DB(cudaGetLastError());
        }
      } else {
        db_sort_hist<<<sblocks, 256, 0, st>>>(kin, m, 8 * p, ntiles, 0, hist, 0, cnt + 6);
        DB(cudaGetLastError());
      }
      DBS(device_scan(hist, (long long)ntiles * 256, st));
      db_sort_scatter<<<sblocks, 256, 0, st>>>(kin, vin, m, 8 * p, ntiles, hist, kb[p & 1], vb[p & 1]);
      DB(cudaGetLastError());
    }
  }
  // capacities: copied on the side stream (its host call may block while
  // the sort above runs)
  if (m && d_cap) {
    DB(cudaMemcpyAsync(d_cap, in->capacities, 4 * (size_t)m, cudaMemcpyHostToDevice, side));
    DB(cudaEventRecord(side_done, side));
  }
  // heads and offsets must be valid before anything indexes with them
  unsigned long long chk[2] = {0, 0};
  DB(cudaMemcpyAsync(chk, cnt + 6, 8, cudaMemcpyDeviceToHost, st));
  DB(cudaStreamSynchronize(st));
  if (chk[0]) {
    cleanup();
    return WBPR_ERR_INVALID_ARG;
  }
  if (m) {
    db_indeg_sorted<<<blocks, 256, 0, st>>>(skey, m, inoff);
    DB(cudaGetLastError());
    if (bcsr) {
      // the sorted position of every arc, one window of arc ids at a time
      const long long win = std::max<long long>(1 << 20, (long long)g->l2_bytes / 8);
      for (long long lo = 0; lo < m; lo += win) {
        db_pos_window<<<blocks, 256, 0, st>>>(sval, m, (int)lo, (int)std::min(m, lo + win), tail);
        DB(cudaGetLastError());
      }
    }
  }
  DBS(device_scan(inoff, (long long)n + 1, st));
  db_indeg_max<<<blocks, 256, 0, st>>>(inoff, n, cnt + 4);
  DB(cudaGetLastError());
  if (bcsr) {
    db_row<<<blocks, 256, 0, st>>>(g->ioff, inoff, n, g->row);
    DB(cudaGetLastError());
  } else {
    DB(cudaMemcpyAsync(g->frow, g->ioff, 4 * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
    DB(cudaMemcpyAsync(g->rrow, inoff, 4 * ((size_t)n + 1), cudaMemcpyDeviceToDevice, st));
  }
  if (m && d_cap) DB(cudaStreamWaitEvent(st, side_done, 0));
  if (m) {
    if (bcsr) {
      db_fill_fwd<<<blocks, 256, 0, st>>>(g->ioff, trow, inoff, d_dst, d_cap, tail, m, g->arc, g->arx, utail,
                                          cnt + 6, cnt + 3);
      db_fill_twin<<<blocks, 256, 0, st>>>(g->ioff, inoff, skey, sval, utail, d_cap, cnt + 3, m, g->arc, g->arx,
                                           incap);
    } else {
      db_rcsr_fwd<<<blocks, 256, 0, st>>>(g->ioff, trow, d_dst, d_cap, m, g->farc, g->fcap, g->fcb, tail, cnt + 6,
                                          cnt + 3);
      db_rcsr_rev<<<blocks, 256, 0, st>>>(skey, sval, tail, g->fcap, cnt + 3, m, g->rarc, incap);
    }
    DB(cudaGetLastError());
  }
  db_max<<<blocks, 256, 0, st>>>(incap, n, cnt + 7);
  DB(cudaGetLastError());
  const int* o1 = bcsr ? g->row : g->frow;
  const int* o2 = bcsr ? nullptr : g->rrow;
  // length classes in vertex order, by three stable compactions
  int* fl[3] = {vb[0], vb[1], kb[0]};  // free once the fill kernels have run (stream order)
  db_classify<<<blocks, 256, 0, st>>>(o1, o2, n, fl[0], fl[1], fl[2], cnt);
  DB(cudaGetLastError());
  for (int k = 0; k < 3; ++k) DBS(device_scan(fl[k], (long long)n + 1, st));
  int tot[3];
  unsigned long long hc[3];
  for (int k = 0; k < 3; ++k) DB(cudaMemcpyAsync(tot + k, fl[k] + n, 4, cudaMemcpyDeviceToHost, st));
  DB(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
  DB(cudaMemcpyAsync(chk, cnt + 6, 16, cudaMemcpyDeviceToHost, st));
  DB(cudaStreamSynchronize(st));
  if (chk[0]) {  // a negative capacity
    cleanup();
    return WBPR_ERR_INVALID_ARG;
  }
  if (chk[1] > 0x7fffffffull) {  // some vertex's incoming capacities pass int32
    cleanup();
    return WBPR_ERR_OVERFLOW;
  }
  g->n_light = tot[0];
  g->n_medium = tot[1];
  g->n_heavy = tot[2];
  g->n_td_heavy = (int)hc[0];
  g->n_td_items = (int64_t)hc[1];
  g->total_deg = 2 * m;
  g->avg_deg = (double)g->total_deg / std::max<int64_t>(1, g->n_light + g->n_medium + g->n_heavy);
  DBS(dalloc(g, &g->cls, (size_t)(tot[0] + tot[1] + tot[2])));
  db_cls_scatter<<<blocks, 256, 0, st>>>(o1, o2, n, fl[0], fl[1], fl[2], g->cls);
  DB(cudaGetLastError());
  // static kChunk pieces of the heavy rows, in vertex order
  const int nh = tot[2];
  int* cbase = hist;  // holds at least n + 1 entries
  const int* hcls = g->cls + tot[0] + tot[1];
  db_heavy_chunks<<<blocks, 256, 0, st>>>(o1, o2, hcls, nh, cbase);
  DB(cudaGetLastError());
  DBS(device_scan(cbase, (long long)nh + 1, st));
  int nbch = 0;
  DB(cudaMemcpyAsync(&nbch, cbase + nh, 4, cudaMemcpyDeviceToHost, st));
  DB(cudaStreamSynchronize(st));
  g->n_bch = nbch;
  DBS(dalloc(g, &g->bch, (size_t)nbch));
  if (nh) db_bch_fill<<<std::min(nh, blocks), 128, 0, st>>>(o1, o2, hcls, nh, cbase, g->bch);
  DB(cudaGetLastError());
  const size_t max_chunks = (size_t)hc[2] + 1;
  DBS(dalloc(g, &g->hrec, 3 * max_chunks));
  DBS(dalloc(g, &g->hsum, max_chunks));
  DBS(dalloc(g, &g->hmin, max_chunks));
  DB(cudaStreamSynchronize(st));
#undef DB
#undef DBS
  cleanup();
  return WBPR_OK;
}

// ---------------------------------------------------------------------------
wbpr_status create_impl(const wbpr_csr* in, wbpr_layout layout, wbpr_graph** out) {
  if (!out) return WBPR_ERR_INVALID_ARG;
  *out = nullptr;
  // the O(n + m) validation runs on the device while it builds
  wbpr_status st = wbpr::check_csr_shape(in);
  if (st) return st;
  if (in->num_nodes < 2) return WBPR_ERR_INVALID_ARG;
  if (layout != WBPR_LAYOUT_RCSR && layout != WBPR_LAYOUT_BCSR && layout != WBPR_LAYOUT_BCSR2)
    return WBPR_ERR_INVALID_ARG;
  if (2 * in->num_edges > std::numeric_limits<int32_t>::max()) return WBPR_ERR_OVERFLOW;
  // incoming-capacity overflow is checked on the device while it builds
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return WBPR_ERR_NO_DEVICE;
  }
  wbpr_graph* g = new wbpr_graph();
  g->layout = layout == WBPR_LAYOUT_RCSR ? WBPR_LAYOUT_RCSR : WBPR_LAYOUT_BCSR;
  g->n = in->num_nodes;
  g->m = in->num_edges;
  g->s = in->source;
  g->t = in->sink;
  auto fail = [&](wbpr_status s) {
    release(g);
    return s;
  };
#define TRY(x)                          \
  do {                                  \
    wbpr_status s_ = (x);               \
    if (s_) return fail(s_);            \
  } while (0)
#define TRYC(x)                                                           \
  do {                                                                    \
    cudaError_t e_ = (x);                                                 \
    if (e_ != cudaSuccess) {                                              \
      g_last_error = std::string(#x) + ": " + cudaGetErrorString(e_);     \
      return fail(WBPR_ERR_CUDA);                                         \
    }                                                                     \
  } while (0)
  TRYC(cudaGetDevice(&g->device));
  TRYC(cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device));
  TRYC(cudaDeviceGetAttribute(&g->l2_bytes, cudaDevAttrL2CacheSize, g->device));
  TRYC(cudaStreamCreateWithFlags(&g->own_stream, cudaStreamNonBlocking));
  g->stream = g->own_stream;
  TRYC(cudaEventCreate(&g->ev0));
  TRYC(cudaEventCreate(&g->ev1));
  TRYC(cudaEventCreate(&g->ev2));
  TRYC(cudaEventCreate(&g->ev3));
  const int n = g->n;
  TRY(build_device(g, in));
  int** vec[] = {&g->h, &g->e, &g->rl_min, &g->rl_left, &g->lq[0], &g->lq[1], &g->hq[0], &g->hq[1],
                 &g->esnap, &g->dmin0,
                 &g->qraw, &g->fr[0], &g->fr[1], &g->fr[2], &g->vlab};
  {
    // one allocation for the per-vertex scratch, one for the BFS chunk lists
    const size_t nvec = sizeof(vec) / sizeof(vec[0]);
    const size_t stride = ((size_t)n + 63) & ~(size_t)63;
    int* base = nullptr;
    TRY(dalloc(g, &base, stride * nvec));
    for (size_t k = 0; k < nvec; ++k) *vec[k] = base + k * stride;
    const size_t fstride = ((size_t)g->n_td_items + 1 + 31) & ~(size_t)31;
    int2* fb = nullptr;
    TRY(dalloc(g, &fb, 3 * fstride));
    for (int k = 0; k < 3; ++k) g->frh[k] = fb + k * fstride;
  }
  TRY(dalloc(g, &g->ctl, 1));
  TRY(dalloc(g, &g->st, 1));
  if (g->layout == WBPR_LAYOUT_BCSR && g->m > 0) {
    // undo log: a quarter of the residual arcs (at least 2^20 entries), over
    // kLogSlots slots; the built residuals are the capacities, so it starts empty
    const int64_t want = std::max<int64_t>((2 * g->m) / 4, (int64_t)1 << 20);
    g->ulog_cap = (int)((want + kLogSlots - 1) / kLogSlots);
    TRY(dalloc(g, &g->ulog, (size_t)g->ulog_cap * kLogSlots));
    TRY(dalloc(g, &g->ulog_n, (size_t)kLogSlots * kLogStride));
    TRYC(cudaMemsetAsync(g->ulog_n, 0, sizeof(int) * (size_t)kLogSlots * kLogStride, g->stream));
  }
  // in the stream the pool allocations were made on (stream-ordered memory)
  TRYC(cudaMemsetAsync(g->h, 0, 4 * (size_t)n, g->stream));
  TRYC(cudaMemsetAsync(g->e, 0, 4 * (size_t)n, g->stream));
  TRYC(cudaStreamSynchronize(g->stream));
#undef TRY
#undef TRYC
  *out = g;
  return WBPR_OK;
}

// a grid-barrier wait gives up after this long unless the tuning says otherwise
constexpr unsigned long long kBarrierTimeoutNs = 10ull * 1000 * 1000 * 1000;

template <class Topo>
void fill_common(wbpr_graph* g, Params<Topo>& p) {
  p.n = g->n;
  p.lab = g->h;
  p.e = g->e;
  p.rl_min = g->rl_min;
  p.rl_left = g->rl_left;
  for (int k = 0; k < 2; ++k) {
    p.lq[k] = g->lq[k];
    p.hq[k] = g->hq[k];
  }
  p.esnap = g->esnap;
  p.dmin0 = g->dmin0;
  p.hrec = g->hrec;
  p.hsum = g->hsum;
  p.hmin = g->hmin;
  p.bch = g->bch;
  p.n_bch = g->n_bch;
  p.qraw = g->qraw;
  for (int k = 0; k < 3; ++k) {
    p.fr[k] = g->fr[k];
    p.frh[k] = g->frh[k];
  }
  p.cls = g->cls;
  p.n_light = g->n_light;
  p.n_medium = g->n_medium;
  p.n_heavy = g->n_heavy;
  p.ctl = g->ctl;
  p.st = g->st;
  p.total_deg = g->total_deg;
  p.bar_timeout_ns = kBarrierTimeoutNs;
  p.bfs_dir = 0;
  p.bfs_root = 0;
  p.bfs_excl = -1;
}

void topo_of(wbpr_graph* g, TopoB& b) {
  b.row = g->row;
  b.arc = g->arc;
  b.arx = g->arx;
  b.bd.viol = &g->ctl->viol;
  b.bd.na = 2 * g->m;
  b.bd.n = g->n;
  b.ulog = g->ulog;
  b.ulog_n = g->ulog_n;
  b.ulog_cap = g->ulog_cap;
}
void topo_of(wbpr_graph* g, TopoR& r) {
  r.frow = g->frow;
  r.farc = g->farc;
  r.fcb = g->fcb;
  r.rrow = g->rrow;
  r.rarc = g->rarc;
  r.bd.viol = &g->ctl->viol;
  r.bd.na = g->m;
  r.bd.n = g->n;
}


struct RunCfg {
  int mode;
  int s, t;
  int tile;
  int threads;
  int blocks_per_sm;
  int grid_blocks;
  int heavy_deg;
  unsigned long long gr_threshold;
  int gr_rounds;
  int gr_stall;
  int greedy;
  int bfs_alpha;
  int gr_plateau;
  bool matching;  // the matching kernel may take unit-capacity bipartite networks
  long long max_rounds;
  unsigned long long budget_ns;
  unsigned long long bar_timeout_ns;
  int bfs_dir, bfs_root, bfs_excl;
  int* lab;
  bool trace;
  // terminal sets (multi-pair solve); term == nullptr for one pair
  const signed char* term;
  const int* sources;
  int n_sources;
  const int* sinks;
  int n_sinks;
};

// The event-trace buffers (wbpr_tuning.trace), allocated at first use.
wbpr_status ensure_trace(wbpr_graph* g) {
  if (g->trace) return WBPR_OK;
  g->trace_cap = 1 << 14;
  wbpr_status st = dalloc(g, &g->trace, 6 * (size_t)g->trace_cap);
  if (st) return st;
  st = dalloc(g, &g->bt, 4096);
  if (st) return st;
  st = dalloc(g, &g->bt2, 8192);
  if (st) return st;
  CK(cudaMemset(g->bt, 0, 8 * 4096));
  CK(cudaMemset(g->bt2, 0, 8 * 8192));
  return WBPR_OK;
}

template <class Topo>
wbpr_status run_kernel(wbpr_graph* g, const RunCfg& rc, Stats* hs, float* launch_ms) {
  Params<Topo> p{};  // every field zero unless it has its own initializer
  topo_of(g, p.g);
  fill_common(g, p);
  p.s = rc.s;
  p.t = rc.t;
  p.mode = rc.mode;
  p.heavy_deg = rc.heavy_deg;
  p.gr_threshold = rc.gr_threshold;
  p.gr_rounds = rc.gr_rounds;
  p.gr_stall = rc.gr_stall;
  p.greedy = rc.greedy;
  if (rc.bfs_alpha > 0) p.bfs_alpha = rc.bfs_alpha;
  p.gr_plateau = rc.gr_plateau;
  if (rc.bar_timeout_ns) p.bar_timeout_ns = rc.bar_timeout_ns;
  p.max_rounds = rc.max_rounds;
  p.budget_ns = rc.budget_ns;
  p.bfs_dir = rc.bfs_dir;
  p.bfs_root = rc.bfs_root;
  p.bfs_excl = rc.bfs_excl;
  if (rc.lab) p.lab = rc.lab;
  if (rc.term) {
    p.term = rc.term;
    p.sources = rc.sources;
    p.n_sources = rc.n_sources;
    p.sinks = rc.sinks;
    p.n_sinks = rc.n_sinks;
    p.s = -1;
    p.t = -1;
    p.bfs_excl = -1;
  }
  if (rc.trace) {
    wbpr_status st = ensure_trace(g);
    if (st) return st;
    p.trace = g->trace;
    p.bt = g->bt;
    p.bt2 = g->bt2;
    p.trace_cap = g->trace_cap;
  }
  const int occ = occupancy_pr(&p, rc.tile, rc.threads);
  if (occ <= 0) {
    g_last_error = "persistent kernel does not fit on an SM";
    return WBPR_ERR_CUDA;
  }
  const int bps = rc.blocks_per_sm > 0 ? std::min(occ, rc.blocks_per_sm) : occ;
  int blocks = g->sms * bps;
  if (rc.grid_blocks > 0) blocks = std::min(blocks, rc.grid_blocks);
  else blocks = grid_blocks_for((long long)g->n + g->total_deg, g->sms, blocks);
  CK(cudaMemsetAsync(g->ctl, 0, sizeof(Ctl), g->stream));
  CK(cudaMemsetAsync(g->st, 0, sizeof(Stats), g->stream));
  CK(cudaEventRecord(g->ev2, g->stream));
  CK(launch_pr(p, rc.tile, blocks, rc.threads, g->stream));
  CK(cudaEventRecord(g->ev3, g->stream));
  if (rc.mode != kModeBfsOnly) CK(launch_stranded(p, g->sms * 4, 256, g->stream));
  Ctl hc;
  CK(cudaMemcpyAsync(&hc, g->ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaMemcpyAsync(hs, g->st, sizeof(Stats), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (launch_ms) CK(cudaEventElapsedTime(launch_ms, g->ev2, g->ev3));
  g->trace_n = rc.trace ? hs->trace_n : 0;
  if (hc.err) return (wbpr_status)hc.err;
  if (hc.viol) {
    g_last_error = "bounds check: " + std::to_string(hc.viol) + " out-of-range arc or vertex indices";
    return WBPR_ERR_VERIFY;
  }
  return WBPR_OK;
}

wbpr_status run(wbpr_graph* g, const RunCfg& rc, Stats* hs, float* launch_ms = nullptr) {
  return g->layout == WBPR_LAYOUT_RCSR ? run_kernel<TopoR>(g, rc, hs, launch_ms)
                                       : run_kernel<TopoB>(g, rc, hs, launch_ms);
}

// Rows longer than this are discharged by a whole warp in the matching kernel
// (the left-vertex lists are split by it once, at the shape check).
constexpr int kMatchHeavy = 32;
// The matching kernel's global relabel runs when the active set shrank by
// less than 10% over this many rounds (wbpr_tuning.gr_plateau overrides it):
// after the first few rounds most active vertices cannot reach t.
constexpr int kMatchPlateau = 2;
// The matching relabel's BFS turns bottom-up when the frontier's arcs x this
// exceed the unlabelled left arcs (wbpr_tuning.bfs_alpha overrides it).  On
// the 2M x 2M matching, 4 against the general solver's 14: half the arcs
// inspected, 1.88-1.90 against 1.93-1.95 ms; 8, 24 and 48 no better.
constexpr int kMatchBfsAlpha = 4;

// Is (s, t) of this BCSR16 graph a unit-capacity bipartite matching network
// (s -> left, left -> right, right -> t, every capacity 1, no other arc)?
// Checked on the device in three O(n + m) passes and cached per terminal pair
// (wbpr_graph_set_capacities drops the cache); on success the left and right
// vertex lists stay on the device for the matching kernel.
wbpr_status match_detect(wbpr_graph* g, int s, int t, bool* ok) {
  *ok = false;
  if (g->m == 0 || s == t) return WBPR_OK;
  if (g->mt_s == s && g->mt_t == t) {
    *ok = g->mt_ok;
    return WBPR_OK;
  }
  wbpr_status st;
  const size_t n = (size_t)g->n;
  if (!g->mt_ctl && (st = dalloc(g, &g->mt_ctl, 1))) return st;
  // the counts live in the relabel records, free between solves
  int* cl = g->rl_min;
  int* cr = g->rl_left;
  CK(cudaMemsetAsync(cl, 0, 4 * n, g->stream));
  CK(cudaMemsetAsync(cr, 0, 4 * n, g->stream));
  CK(cudaMemsetAsync(g->mt_ctl, 0, sizeof(MCtl), g->stream));
  g->mt_s = s;
  g->mt_t = t;
  g->mt_ok = false;
  mt_count<<<g->sms * 4, 256, 0, g->stream>>>(g->row, g->ioff, g->arc, g->arx, g->farc, g->fcap, g->rrow, g->rarc,
                                              s, t, cl, cr, g->mt_ctl);
  CK(cudaGetLastError());
  // most graphs fail on s's or t's arcs already (a capacity other than 1):
  // then the pass over every arc (0.35 ms at 65M arcs) is skipped
  int bad = 0;
  CK(cudaMemcpyAsync(&bad, &g->mt_ctl->bad, 4, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (bad) return WBPR_OK;
  mt_check<<<g->sms * 8, 256, 0, g->stream>>>(g->ioff, g->row, g->arc, g->arx, g->farc, g->fcap, g->n, g->m, s, t,
                                              cl, cr, g->mt_ctl);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&bad, &g->mt_ctl->bad, 4, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (bad) return WBPR_OK;
  // a matching network: the kernel's arrays, then the vertex lists
  if (!g->mt_mate &&
      ((st = dalloc(g, &g->mt_mate, n)) || (st = dalloc(g, &g->mt_claim, n)) || (st = dalloc(g, &g->mt_cy, n)) ||
       (st = dalloc(g, &g->mt_lmin, n)) || (st = dalloc(g, &g->mt_lv, n)) || (st = dalloc(g, &g->mt_rv, n))))
    return st;
  mt_list<<<g->sms * 4, 256, 0, g->stream>>>(g->ioff, g->n, kMatchHeavy, cl, cr, g->mt_lv, g->lq[0], g->mt_rv,
                                            g->mt_ctl);
  CK(cudaGetLastError());
  MCtl hc;
  CK(cudaMemcpyAsync(&hc, g->mt_ctl, sizeof(MCtl), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  g->mt_ok = hc.nlist[0] + hc.nlist[1] > 0 && hc.nlist[2] > 0;
  if (g->mt_ok) {
    g->mt_nl_light = hc.nlist[0];
    g->mt_nl = hc.nlist[0] + hc.nlist[1];
    g->mt_nr = hc.nlist[2];
    g->mt_larcs = hc.larcs;
    if (hc.nlist[1])  // the long rows after the short ones
      CK(cudaMemcpyAsync(g->mt_lv + hc.nlist[0], g->lq[0], 4 * (size_t)hc.nlist[1], cudaMemcpyDeviceToDevice,
                         g->stream));
    CK(cudaStreamSynchronize(g->stream));
  }
  *ok = g->mt_ok;
  return WBPR_OK;
}

// One launch of the matching kernel (match.cu) for the pair (s, t) that
// match_detect accepted; the residuals were restored before it.
wbpr_status run_match(wbpr_graph* g, const RunCfg& rc, Stats* hs, float* launch_ms) {
  MatchParams p{};
  if (g->layout == WBPR_LAYOUT_BCSR) {
    p.lrow = p.rrow = g->row;
    p.lhd = g->arc;
    p.rhd = g->arc;
    p.ltrim = p.rskip = 1;
    p.arx = g->arx;
    p.ulog_n = g->ulog ? g->ulog_n : nullptr;
  } else {
    p.lrow = g->frow;
    p.lhd = g->farc;
    p.rrow = g->rrow;
    p.rhd = g->rarc;
    p.fcb = g->fcb;
  }
  p.n = g->n;
  p.s = rc.s;
  p.t = rc.t;
  p.nl = g->mt_nl;
  p.nl_light = g->mt_nl_light;
  p.nr = g->mt_nr;
  p.lv = g->mt_lv;
  p.rv = g->mt_rv;
  p.left_arcs = g->mt_larcs;
  p.mate = g->mt_mate;
  p.claim = g->mt_claim;
  p.cy = g->mt_cy;
  p.lmin = g->mt_lmin;
  p.lab = g->h;
  p.e = g->e;
  for (int k = 0; k < 2; ++k) {
    p.q[k] = g->lq[k];
    p.hq[k] = g->hq[k];
    p.fr[k] = g->fr[k];
  }
  p.ctl = g->mt_ctl;
  p.st = g->st;
  p.heavy_deg = kMatchHeavy;
  p.bfs_alpha = rc.bfs_alpha > 0 ? rc.bfs_alpha : kMatchBfsAlpha;
  p.gr_threshold = rc.gr_threshold;
  p.gr_rounds = rc.gr_rounds;
  p.gr_plateau = rc.gr_plateau > 0 ? rc.gr_plateau : kMatchPlateau;
  p.max_rounds = rc.max_rounds;
  p.budget_ns = rc.budget_ns;
  p.bar_timeout_ns = rc.bar_timeout_ns ? rc.bar_timeout_ns : kBarrierTimeoutNs;
  if (rc.trace) {
    wbpr_status st = ensure_trace(g);
    if (st) return st;
    p.trace = g->trace;
    p.bt = g->bt;
    p.trace_cap = g->trace_cap;
  }
  const int occ = occupancy_match(rc.threads);
  if (occ <= 0) {
    g_last_error = "matching kernel does not fit on an SM";
    return WBPR_ERR_CUDA;
  }
  int blocks = g->sms * (rc.blocks_per_sm > 0 ? std::min(occ, rc.blocks_per_sm) : occ);
  if (rc.grid_blocks > 0) blocks = std::min(blocks, rc.grid_blocks);
  else blocks = grid_blocks_for((long long)g->n + g->total_deg, g->sms, blocks);
  CK(cudaMemsetAsync(g->mt_ctl, 0, sizeof(MCtl), g->stream));
  CK(cudaMemsetAsync(g->st, 0, sizeof(Stats), g->stream));
  CK(cudaEventRecord(g->ev2, g->stream));
  CK(launch_match(p, blocks, rc.threads, g->stream));
  CK(cudaEventRecord(g->ev3, g->stream));
  g->full_reset = true;  // the matching's residuals are not in the undo log
  MCtl hc;
  CK(cudaMemcpyAsync(&hc, g->mt_ctl, sizeof(MCtl), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaMemcpyAsync(hs, g->st, sizeof(Stats), cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (launch_ms) CK(cudaEventElapsedTime(launch_ms, g->ev2, g->ev3));
  g->trace_n = rc.trace ? hs->trace_n : 0;
  if (hc.err) return (wbpr_status)hc.err;
  return WBPR_OK;
}

void tuning_defaults(wbpr_tuning* t) {
  std::memset(t, 0, sizeof(*t));
  t->gr_alpha = kDefaultGrAlpha;
  t->max_ms = 120000.0;
}

wbpr_status make_cfg(wbpr_graph* g, int s, int t, wbpr_algo algo, const wbpr_tuning* tu, RunCfg* rc) {
  wbpr_tuning d;
  tuning_defaults(&d);
  if (!tu) tu = &d;
  if (algo != WBPR_ALGO_TC && algo != WBPR_ALGO_VC) return WBPR_ERR_INVALID_ARG;
  if (s < 0 || t < 0 || s >= g->n || t >= g->n || s == t) return WBPR_ERR_INVALID_ARG;
  std::memset(rc, 0, sizeof(*rc));
  rc->s = s;
  rc->t = t;
  int tile = tu->tile;
  if (tile != 0 && tile != 8 && tile != 16 && tile != 32) return WBPR_ERR_INVALID_ARG;
  if (tile == 0) tile = g->avg_deg < 10 ? 8 : (g->avg_deg < 20 ? 16 : 32);
  rc->tile = algo == WBPR_ALGO_TC ? 1 : tile;
  int threads = tu->block ? tu->block : 256;
  if (threads < 64 || threads > 256 || threads % 32) return WBPR_ERR_INVALID_ARG;
  rc->threads = threads;
  rc->blocks_per_sm = tu->blocks_per_sm > 0 ? tu->blocks_per_sm : 0;
  if (tu->grid_blocks < 0) return WBPR_ERR_INVALID_ARG;
  rc->grid_blocks = tu->grid_blocks;
  rc->heavy_deg = tu->heavy_degree > 0 ? tu->heavy_degree : 32;
  const double alpha = tu->gr_alpha > 0 ? tu->gr_alpha : kDefaultGrAlpha;
  rc->gr_threshold = (unsigned long long)(alpha * ((double)g->n + (double)g->total_deg)) + 1;
  rc->gr_rounds = tu->gr_rounds > 0 ? tu->gr_rounds : 48;
  if (tu->gr_stall < -1 || tu->barrier_timeout_ns < 0 || tu->greedy < -1 || tu->greedy > 0)
    return WBPR_ERR_INVALID_ARG;
  rc->greedy = tu->greedy == 0 ? 1 : 0;
  if (tu->bfs_alpha < 0) return WBPR_ERR_INVALID_ARG;
  rc->bfs_alpha = tu->bfs_alpha;
  if (tu->gr_plateau < -1 || tu->gr_plateau > kMaxPlateau) return WBPR_ERR_INVALID_ARG;
  if (tu->matching < -1 || tu->matching > 0) return WBPR_ERR_INVALID_ARG;
  rc->matching = tu->matching == 0;
  rc->gr_plateau = tu->gr_plateau == 0 ? kDefaultPlateau : (tu->gr_plateau < 0 ? 0 : tu->gr_plateau);
  rc->gr_stall = tu->gr_stall == 0 ? default_gr_stall((long long)g->n + g->total_deg)
                                   : (tu->gr_stall < 0 ? 0 : tu->gr_stall);
  rc->bar_timeout_ns = tu->barrier_timeout_ns > 0 ? (unsigned long long)tu->barrier_timeout_ns : kBarrierTimeoutNs;
  rc->max_rounds = tu->max_rounds;
  rc->trace = tu->trace != 0;
  const double ms = tu->max_ms > 0 ? tu->max_ms : 120000.0;
  rc->budget_ns = (unsigned long long)(ms * 1e6);
  rc->bfs_excl = -1;
  return WBPR_OK;
}

// Residuals back to the capacities before a fresh BCSR16 solve: only the arcs
// the undo log holds, or all of them after a change of capacities.
void restore_bcsr(wbpr_graph* g) {
  if (!g->m) return;
  if (g->ulog) {
    reset_logged<<<g->sms * 8, 256, 0, g->stream>>>(g->arc, g->arx, 2 * g->m, g->ulog, g->ulog_n, g->ulog_cap,
                                                    g->full_reset ? 1 : 0);
  } else {
    reset_bcsr<<<g->sms * 8, 256, 0, g->stream>>>(g->arc, g->arx, 2 * g->m);
  }
  g->full_reset = false;
}

// Algorithmic bytes of one persistent-kernel launch, by phase, from its
// counters (the residual restore before the launch is not included).
struct PhaseBytes {
  uint64_t push, deep, relabel, gr, init;
  uint64_t total() const { return push + relabel + gr + init; }  // deep is part of push
};
PhaseBytes phase_bytes(const wbpr_graph* g, const Stats& s) {
  const uint64_t arc_b = 12;   // {dst, cf} record + label of the head
  const uint64_t visit_b = 16; // row bounds, excess, label
  // twin index, residual store, twin residual read-modify-write, excess
  // atomic; plus the undo-log entry where the handle keeps one
  const uint64_t push_b = 24 + (g->ulog ? 4 : 0);
  const uint64_t rel_b = 12;   // relabel record + label store
  const uint64_t bfs_arc_b = 12, bfs_v_b = 8;
  PhaseBytes b;
  b.push = s.arcs_scanned * arc_b + s.vertex_visits * visit_b + s.pushes * push_b;
  b.deep = s.deep_scanned * arc_b;
  b.relabel = s.relabels * rel_b;
  b.gr = s.bfs_arcs * bfs_arc_b + s.bfs_vertices * bfs_v_b + (uint64_t)s.grs * g->n * 4;
  b.init = (uint64_t)g->n * 12;  // labels, excess, relabel records
  return b;
}

// The same for a matching-kernel launch: 8 bytes per arc scanned (the head of
// the record + its label), 8 per visit (queue entry, row bounds), 20 per
// claim (mate exchange, label, the claimer's two words), 8 per BFS arc and
// vertex check, 12 per left and right vertex per global relabel (label, mate
// or claim), and 8 n + 16 per vertex of the lists to initialise; the push
// bytes also count the write-back, 48 per matched edge plus its 3 log entries.
PhaseBytes match_bytes(const wbpr_graph* g, const Stats& s, int64_t flow) {
  PhaseBytes b;
  b.push = s.arcs_scanned * 8 + s.vertex_visits * 8 + s.pushes * 20 + (uint64_t)flow * (48 + 12);
  b.deep = 0;
  b.relabel = 0;
  b.gr = s.bfs_arcs * 8 + s.bfs_vertices * 8 + (uint64_t)s.grs * (uint64_t)(g->mt_nl + g->mt_nr) * 12;
  b.init = (uint64_t)g->n * 8 + (uint64_t)(g->mt_nl + g->mt_nr) * 16;
  return b;
}

}  // namespace

// ===========================================================================
extern "C" {

const char* wbpr_last_error(void) { return g_last_error.c_str(); }

void wbpr_default_tuning(wbpr_tuning* t) {
  if (t) tuning_defaults(t);
}

int32_t wbpr_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

wbpr_status wbpr_graph_create(const wbpr_csr* g, wbpr_layout layout, wbpr_graph** out) {
  NvtxRange nvtx_("wbpr_graph_create");
  return create_impl(g, layout, out);
}

wbpr_status wbpr_graph_destroy(wbpr_graph* g) {
  if (!g) return WBPR_ERR_INVALID_ARG;
  release(g);
  return WBPR_OK;
}

int64_t wbpr_graph_device_bytes(const wbpr_graph* g) { return g ? g->bytes : 0; }

wbpr_status wbpr_memory_cache(int64_t max_bytes) {
  if (max_bytes < 0) return WBPR_ERR_INVALID_ARG;
  int ndev = 0, dev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return WBPR_ERR_NO_DEVICE;
  }
  {
    std::lock_guard<std::mutex> lk(wbpr::g_pool_mu);
    wbpr::g_cache_bytes = (unsigned long long)max_bytes;
  }
  cudaMemPool_t pool = wbpr::device_pool(dev);
  if (!pool) {
    g_last_error = "wbpr_memory_cache: no memory pool on this device";
    return WBPR_ERR_CUDA;
  }
  unsigned long long thr = (unsigned long long)max_bytes;
  CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  CK(cudaMemPoolTrimTo(pool, (size_t)max_bytes));
  return WBPR_OK;
}

wbpr_status wbpr_autotune(wbpr_graph* g, int32_t s, int32_t t, wbpr_algo algo, wbpr_tuning* best,
                          float* best_ms) {
  NvtxRange nvtx_("wbpr_autotune");
  if (!g || !best) return WBPR_ERR_INVALID_ARG;
  {
    // a unit-capacity bipartite network goes to the matching kernel, which
    // has none of the knobs below: the defaults, timed
    wbpr_tuning tu;
    wbpr_default_tuning(&tu);
    wbpr_result r0, r1;
    wbpr_status st = wbpr_solve(g, s, t, algo, &tu, &r0);
    if (st) return st;
    if (r0.matching) {
      if ((st = wbpr_solve(g, s, t, algo, &tu, &r1))) return st;
      if (r1.flow != r0.flow) return WBPR_ERR_VERIFY;
      *best = tu;
      if (best_ms) *best_ms = std::min(r0.solve_ms, r1.solve_ms);
      return WBPR_OK;
    }
  }
  const int tiles_vc[] = {8, 16, 32};
  const int tiles_tc[] = {0};
  const double alphas[] = {0.5, 1.0, 1.5, 3.0};
  const int heavies[] = {32, 64};
  const int* tiles = algo == WBPR_ALGO_TC ? tiles_tc : tiles_vc;
  const int ntiles = algo == WBPR_ALGO_TC ? 1 : 3;
  float bms = 0;
  bool have = false;
  int64_t flow = -1;
  for (int ti = 0; ti < ntiles; ++ti)
    for (double a : alphas)
      for (int hd : heavies) {
        wbpr_tuning tu;
        wbpr_default_tuning(&tu);
        tu.tile = tiles[ti];
        tu.gr_alpha = a;
        tu.heavy_degree = hd;
        float ms = 0;
        for (int rep = 0; rep < 2; ++rep) {  // the faster of two solves
          wbpr_result r;
          const wbpr_status st = wbpr_solve(g, s, t, algo, &tu, &r);
          if (st) return st;
          if (flow >= 0 && r.flow != flow) return WBPR_ERR_VERIFY;  // every tuning must agree
          flow = r.flow;
          ms = rep ? std::min(ms, r.solve_ms) : r.solve_ms;
        }
        if (!have || ms < bms) {
          have = true;
          bms = ms;
          *best = tu;
        }
      }
  // then, on the best of those, the global relabel's BFS turning bottom-up
  // earlier and the plateau trigger (both pay on unit-capacity matching
  // networks and lose on GENRMF, layered networks and large R-MAT graphs)
  const wbpr_tuning base = *best;
  for (int k = 0; k < 3; ++k) {
    wbpr_tuning tu = base;
    if (k != 1) tu.bfs_alpha = 4;
    if (k != 0) tu.gr_plateau = 4;
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {
      wbpr_result r;
      const wbpr_status st = wbpr_solve(g, s, t, algo, &tu, &r);
      if (st) return st;
      if (r.flow != flow) return WBPR_ERR_VERIFY;
      ms = rep ? std::min(ms, r.solve_ms) : r.solve_ms;
    }
    if (ms < bms) {
      bms = ms;
      *best = tu;
    }
  }
  if (best_ms) *best_ms = bms;
  return WBPR_OK;
}

wbpr_status wbpr_graph_set_capacities(wbpr_graph* g, const int32_t* capacities) {
  NvtxRange nvtx_("wbpr_graph_set_capacities");
  if (!g || (g->m > 0 && !capacities)) return WBPR_ERR_INVALID_ARG;
  if (g->m == 0) return WBPR_OK;
  CK(cudaSetDevice(g->device));
  const size_t m = (size_t)g->m, n = (size_t)g->n;
  if (!g->cap_tmp) {
    wbpr_status st = dalloc(g, &g->cap_tmp, m + 2 * (n + 1) + 8);
    if (st) return st;
  }
  int* dcap = g->cap_tmp;
  auto* incap = (unsigned long long*)(g->cap_tmp + ((m + 1) & ~(size_t)1));
  unsigned long long* chk = incap + n + 1;  // [0] bad, [1] max incoming sum
  cudaPointerAttributes pa;
  const bool on_device = cudaPointerGetAttributes(&pa, capacities) == cudaSuccess &&
                         (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  CK(cudaMemcpyAsync(dcap, capacities, 4 * m, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                     g->stream));
  CK(cudaMemsetAsync(incap, 0, 8 * (n + 1) + 16, g->stream));
  const bool bcsr = g->layout == WBPR_LAYOUT_BCSR;
  caps_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->ioff, bcsr ? g->row : nullptr, g->arc, g->arx, g->farc, g->fcap,
                                                dcap, g->n, g->m, 0, incap, chk);
  db_max<<<g->sms * 8, 256, 0, g->stream>>>(incap, g->n, chk + 1);
  CK(cudaGetLastError());
  unsigned long long h[2] = {0, 0};
  CK(cudaMemcpyAsync(h, chk, 16, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (h[0]) return WBPR_ERR_INVALID_ARG;
  if (h[1] > 0x7fffffffull) return WBPR_ERR_OVERFLOW;
  caps_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->ioff, bcsr ? g->row : nullptr, g->arc, g->arx, g->farc, g->fcap,
                                                dcap, g->n, g->m, 1, incap, chk);
  g->full_reset = true;  // every residual goes back to its new capacity at the next solve
  g->mt_s = g->mt_t = -1;  // capacities other than 1 may have come
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(g->stream));
  return WBPR_OK;
}

wbpr_status wbpr_graph_set_stream(wbpr_graph* g, void* stream) {
  if (!g) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  CK(cudaStreamSynchronize(g->stream));  // finish what was queued on the previous stream
  g->stream = stream ? (cudaStream_t)stream : g->own_stream;
  return WBPR_OK;
}

wbpr_status wbpr_graph_read_rcsr(const wbpr_graph* g, int32_t* roffsets, int32_t* rdestinations,
                                 int32_t* flow_index) {
  if (!g || g->layout != WBPR_LAYOUT_RCSR) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  CK(cudaStreamSynchronize(g->stream));
  if (roffsets) CK(cudaMemcpy(roffsets, g->rrow, 4 * ((size_t)g->n + 1), cudaMemcpyDeviceToHost));
  const size_t m = (size_t)g->m;
  if (m && (rdestinations || flow_index)) {
    std::vector<int2> r(m);
    CK(cudaMemcpy(r.data(), g->rarc, 8 * m, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < m; ++k) {
      if (rdestinations) rdestinations[k] = r[k].x;
      if (flow_index) flow_index[k] = r[k].y;
    }
  }
  return WBPR_OK;
}

wbpr_status wbpr_graph_read_bcsr(const wbpr_graph* g, int32_t* offsets, int32_t* destinations,
                                 int32_t* capacities, int32_t* backward_idx) {
  if (!g || g->layout != WBPR_LAYOUT_BCSR) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  CK(cudaStreamSynchronize(g->stream));
  if (offsets) CK(cudaMemcpy(offsets, g->row, 4 * ((size_t)g->n + 1), cudaMemcpyDeviceToHost));
  const size_t na = (size_t)(2 * g->m);
  if (na && (destinations || capacities || backward_idx)) {
    std::vector<int2> a(na), x(na);
    CK(cudaMemcpy(a.data(), g->arc, 8 * na, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(x.data(), g->arx, 8 * na, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < na; ++k) {
      if (destinations) destinations[k] = a[k].x;
      if (capacities) capacities[k] = x[k].y;
      if (backward_idx) backward_idx[k] = x[k].x;
    }
  }
  return WBPR_OK;
}

wbpr_status wbpr_solve(wbpr_graph* g, int32_t s, int32_t t, wbpr_algo algo, const wbpr_tuning* tu,
                       wbpr_result* out) {
  NvtxRange nvtx_("wbpr_solve");
  if (!g) return WBPR_ERR_INVALID_ARG;
  if (s < 0) s = g->s;
  if (t < 0) t = g->t;
  RunCfg rc;
  wbpr_status st = make_cfg(g, s, t, algo, tu, &rc);
  if (st) return st;
  rc.mode = kModeFresh;
  rc.bfs_excl = s;
  CK(cudaSetDevice(g->device));
  bool matched = false;
  if (rc.matching && (st = match_detect(g, s, t, &matched))) return st;
  CK(cudaEventRecord(g->ev0, g->stream));
  if (g->layout == WBPR_LAYOUT_RCSR) {
    if (g->m) reset_rcsr<<<g->sms * 8, 256, 0, g->stream>>>(g->farc, g->fcb, g->fcap, g->m);
  } else {
    restore_bcsr(g);
  }
  CK(cudaGetLastError());
  Stats hs;
  float launch_ms = 0;
  st = matched ? run_match(g, rc, &hs, &launch_ms) : run(g, rc, &hs, &launch_ms);
  CK(cudaEventRecord(g->ev1, g->stream));
  CK(cudaEventSynchronize(g->ev1));
  if (st) return st;
  int et = 0;
  CK(cudaMemcpy(&et, g->e + t, 4, cudaMemcpyDeviceToHost));
  if (out) {
    std::memset(out, 0, sizeof(*out));
    out->flow = et;
    CK(cudaEventElapsedTime(&out->solve_ms, g->ev0, g->ev1));
    out->kernel_ms = (float)(hs.round_ns * 1e-6);
    out->gr_ms = (float)(hs.gr_ns * 1e-6);
    out->arcs_scanned = hs.arcs_scanned;
    out->pushes = hs.pushes;
    out->relabels = hs.relabels;
    out->vertex_visits = hs.vertex_visits;
    out->bfs_arcs = hs.bfs_arcs;
    out->bfs_vertices = hs.bfs_vertices;
    out->rounds = hs.rounds;
    out->global_relabels = hs.grs;
    out->stranded = hs.stranded;
    const PhaseBytes pb = matched ? match_bytes(g, hs, et) : phase_bytes(g, hs);
    out->alg_bytes = pb.total();
    out->bytes_push = pb.push;
    out->bytes_deep = pb.deep;
    out->bytes_relabel = pb.relabel;
    out->bytes_gr = pb.gr;
    out->deep_ms = (float)(hs.deep_ns * 1e-6);
    out->deep_arcs_scanned = hs.deep_scanned;
    out->launch_ms = launch_ms;
    out->push_ms = (float)(hs.push_ns * 1e-6);
    out->bfs_levels = hs.bfs_levels;
    out->bfs_bottom_up_levels = hs.bu_levels;
    out->heavy_visits = hs.heavy_visits;
    out->matching = matched ? 1 : 0;
  }
  g->s = s;
  g->t = t;
  if (tu && tu->verify) {
    wbpr_verify_report rep;
    st = wbpr_verify(g, &rep);
    if (st) return st;
    if (!rep.ok) return WBPR_ERR_VERIFY;
  }
  return WBPR_OK;
}

wbpr_status wbpr_solve_pairs(wbpr_graph* g, int32_t k, const int32_t* sources, const int32_t* sinks,
                             wbpr_algo algo, const wbpr_tuning* tu, int64_t* flows, wbpr_result* out) {
  NvtxRange nvtx_("wbpr_solve_pairs");
  if (!g || k < 1 || !sources || !sinks || !flows) return WBPR_ERR_INVALID_ARG;
  {
    // every vertex at most one terminal role, all in range
    std::vector<signed char> seen((size_t)g->n, 0);
    for (int i = 0; i < 2 * k; ++i) {
      const int v = i < k ? sources[i] : sinks[i - k];
      if (v < 0 || v >= g->n || seen[(size_t)v]) return WBPR_ERR_INVALID_ARG;
      seen[(size_t)v] = 1;
    }
  }
  RunCfg rc;
  wbpr_status st = make_cfg(g, sources[0], sinks[0], algo, tu, &rc);
  if (st) return st;
  CK(cudaSetDevice(g->device));
  if (!g->term) {
    st = dalloc(g, &g->term, (size_t)g->n);
    if (st) return st;
  }
  if (g->pairs_cap < k) {
    // grow the pair arrays (the old ones stay with the handle until destroy)
    const int64_t cap = std::max<int64_t>(k, 2 * g->pairs_cap);
    if ((st = dalloc(g, &g->pairs, (size_t)(2 * cap))) || (st = dalloc(g, &g->pair_flow, (size_t)cap))) return st;
    g->pairs_cap = cap;
  }
  CK(cudaMemsetAsync(g->term, 0, (size_t)g->n, g->stream));
  CK(cudaMemcpyAsync(g->pairs, sources, 4 * (size_t)k, cudaMemcpyHostToDevice, g->stream));
  CK(cudaMemcpyAsync(g->pairs + k, sinks, 4 * (size_t)k, cudaMemcpyHostToDevice, g->stream));
  set_terms<<<std::max(1, std::min(g->sms * 4, (2 * k + 255) / 256)), 256, 0, g->stream>>>(g->term, g->pairs, k);
  CK(cudaGetLastError());
  rc.mode = kModeFresh;
  rc.term = g->term;
  rc.sources = g->pairs;
  rc.n_sources = k;
  rc.sinks = g->pairs + k;
  rc.n_sinks = k;
  CK(cudaEventRecord(g->ev0, g->stream));
  if (g->layout == WBPR_LAYOUT_RCSR) {
    if (g->m) reset_rcsr<<<g->sms * 8, 256, 0, g->stream>>>(g->farc, g->fcb, g->fcap, g->m);
  } else {
    restore_bcsr(g);
  }
  CK(cudaGetLastError());
  Stats hs;
  float launch_ms = 0;
  st = run(g, rc, &hs, &launch_ms);
  CK(cudaEventRecord(g->ev1, g->stream));
  CK(cudaEventSynchronize(g->ev1));
  if (st) return st;
  sink_flows<<<std::max(1, std::min(g->sms * 4, (k + 255) / 256)), 256, 0, g->stream>>>(g->e, g->pairs + k, k,
                                                                                        g->pair_flow);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(flows, g->pair_flow, 8 * (size_t)k, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (out) {
    std::memset(out, 0, sizeof(*out));
    int64_t total = 0;
    for (int i = 0; i < k; ++i) total += flows[i];
    out->flow = total;
    CK(cudaEventElapsedTime(&out->solve_ms, g->ev0, g->ev1));
    out->kernel_ms = (float)(hs.round_ns * 1e-6);
    out->gr_ms = (float)(hs.gr_ns * 1e-6);
    out->arcs_scanned = hs.arcs_scanned;
    out->pushes = hs.pushes;
    out->relabels = hs.relabels;
    out->vertex_visits = hs.vertex_visits;
    out->bfs_arcs = hs.bfs_arcs;
    out->bfs_vertices = hs.bfs_vertices;
    out->rounds = hs.rounds;
    out->global_relabels = hs.grs;
    out->stranded = hs.stranded;
    const PhaseBytes pb = phase_bytes(g, hs);
    out->alg_bytes = pb.total();
    out->bytes_push = pb.push;
    out->bytes_deep = pb.deep;
    out->bytes_relabel = pb.relabel;
    out->bytes_gr = pb.gr;
    out->deep_ms = (float)(hs.deep_ns * 1e-6);
    out->deep_arcs_scanned = hs.deep_scanned;
    out->launch_ms = launch_ms;
    out->push_ms = (float)(hs.push_ns * 1e-6);
    out->bfs_levels = hs.bfs_levels;
    out->bfs_bottom_up_levels = hs.bu_levels;
  }
  return WBPR_OK;
}

int32_t wbpr_read_trace(wbpr_graph* g, int64_t* out, int32_t cap) {
  if (!g || !out || cap <= 0 || !g->trace) return 0;
  // the device keeps the last trace_cap records in a ring
  const int total = g->trace_n, kept = std::min(total, g->trace_cap);
  std::vector<long long> ring(6 * (size_t)g->trace_cap);
  if (kept > 0 && cudaMemcpy(ring.data(), g->trace, 48 * (size_t)g->trace_cap, cudaMemcpyDeviceToHost) !=
                      cudaSuccess)
    return 0;
  const int n = std::min(cap, kept);
  for (int i = 0; i < n; ++i) {
    const int src = (total - n + i) % g->trace_cap;
    std::memcpy(out + 6 * (size_t)i, ring.data() + 6 * (size_t)src, 48);
  }
  return n;
}

wbpr_status wbpr_read_state(wbpr_graph* g, int32_t* height, int32_t* excess, int32_t* arc_flow) {
  NvtxRange nvtx_("wbpr_read_state");
  if (!g) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  CK(cudaStreamSynchronize(g->stream));
  if (height) CK(cudaMemcpy(height, g->h, 4 * (size_t)g->n, cudaMemcpyDeviceToHost));
  if (excess) CK(cudaMemcpy(excess, g->e, 4 * (size_t)g->n, cudaMemcpyDeviceToHost));
  if (arc_flow && g->m) {
    if (!g->flow_tmp) {
      wbpr_status st = dalloc(g, &g->flow_tmp, (size_t)g->m);
      if (st) return st;
    }
    flow_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->ioff, g->row, g->arc, g->arx, g->fcb, g->n, g->m,
                                                   g->flow_tmp);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(arc_flow, g->flow_tmp, 4 * (size_t)g->m, cudaMemcpyDeviceToHost, g->stream));
    CK(cudaStreamSynchronize(g->stream));
  }
  return WBPR_OK;
}

static wbpr_status bfs_labels(wbpr_graph* g, int root, int dir, int excl) {
  RunCfg rc;
  wbpr_status st = make_cfg(g, g->s, g->t, WBPR_ALGO_VC, nullptr, &rc);
  if (st) return st;
  rc.mode = kModeBfsOnly;
  rc.bfs_root = root;
  rc.bfs_dir = dir;
  rc.bfs_excl = excl;
  rc.lab = g->vlab;
  Stats hs;
  return run(g, rc, &hs);
}

wbpr_status wbpr_verify(wbpr_graph* g, wbpr_verify_report* rep) {
  NvtxRange nvtx_("wbpr_verify");
  if (!g || !rep) return WBPR_ERR_INVALID_ARG;
  std::memset(rep, 0, sizeof(*rep));
  if (g->s < 0 || g->t < 0) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  wbpr_status st = bfs_labels(g, g->t, 0, -1);
  if (st) return st;
  VerifyAcc* dacc = nullptr;
  CK(wbpr::pool_alloc_on((void**)&dacc, sizeof(VerifyAcc), g->stream));
  cudaMemsetAsync(dacc, 0, sizeof(VerifyAcc), g->stream);
  long long* net = nullptr;
  CK(wbpr::pool_alloc_on((void**)&net, 8 * (size_t)g->n, g->stream));
  cudaMemsetAsync(net, 0, 8 * (size_t)g->n, g->stream);
  if (g->layout == WBPR_LAYOUT_RCSR)
    verify_arcs_rcsr<<<g->sms * 8, 256, 0, g->stream>>>(g->frow, g->farc, g->fcb, g->fcap, g->rrow, g->rarc,
                                                        g->vlab, g->h, g->n, g->s, g->m, net, dacc);
  else
    verify_arcs_bcsr<<<g->sms * 8, 256, 0, g->stream>>>(g->row, g->arc, g->arx, g->vlab, g->h, g->n, g->s,
                                                        2 * g->m, net, dacc);
  verify_vertices<<<g->sms * 4, 256, 0, g->stream>>>(g->e, g->vlab, net, g->n, g->s, g->t, dacc);
  cudaFreeAsync(net, g->stream);
  VerifyAcc h;
  int ls = 0, et = 0;
  cudaError_t ce = cudaGetLastError();
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&h, dacc, sizeof(h), cudaMemcpyDeviceToHost, g->stream);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&ls, g->vlab + g->s, 4, cudaMemcpyDeviceToHost, g->stream);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(&et, g->e + g->t, 4, cudaMemcpyDeviceToHost, g->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(g->stream);
  cudaFreeAsync(dacc, g->stream);
  if (ce != cudaSuccess) {
    g_last_error = std::string("verify: ") + cudaGetErrorString(ce);
    return WBPR_ERR_CUDA;
  }
  rep->capacity_violations = h.cap_viol;
  rep->conservation_violations = h.cons_viol;
  rep->excess_reaches_sink = h.excess_reach;
  rep->label_violations = h.label_viol;
  rep->source_reaches_sink = ls < g->n ? 1 : 0;
  rep->cut_value = h.cut;
  rep->flow_value = et;
  rep->ok = (h.cap_viol == 0 && h.cons_viol == 0 && h.excess_reach == 0 && ls >= g->n &&
             h.cut == (long long)et)
                ? 1
                : 0;
  return WBPR_OK;
}

}  // extern "C"

// Phase 2: return the excess stranded at vertices that cannot reach t to s
// (s absorbs, t is excluded), so the residual graph is that of a maximum flow.
static wbpr_status return_stranded(wbpr_graph* g) {
  RunCfg rc;
  wbpr_status st = make_cfg(g, g->t, g->s, WBPR_ALGO_VC, nullptr, &rc);
  if (st) return st;
  rc.mode = kModeState;
  rc.bfs_excl = g->t;
  Stats hs;
  return run(g, rc, &hs);
}

extern "C" {

wbpr_status wbpr_complete_flow(wbpr_graph* g, float* ms) {
  NvtxRange nvtx_("wbpr_complete_flow");
  if (!g || g->s < 0 || g->t < 0) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  CK(cudaEventRecord(g->ev0, g->stream));
  wbpr_status st = return_stranded(g);
  if (st) return st;
  CK(cudaEventRecord(g->ev1, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (ms) CK(cudaEventElapsedTime(ms, g->ev0, g->ev1));
  return WBPR_OK;
}

wbpr_status wbpr_cut_sides(wbpr_graph* g, int32_t side, int8_t* in_set) {
  NvtxRange nvtx_("wbpr_cut_sides");
  if (!g || !in_set || (side != 0 && side != 1) || g->s < 0 || g->t < 0) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  wbpr_status st;
  if (side == 0) {
    st = bfs_labels(g, g->t, 0, -1);
  } else {
    st = return_stranded(g);
    if (st) return st;
    st = bfs_labels(g, g->s, 1, -1);
  }
  if (st) return st;
  std::vector<int32_t> lab((size_t)g->n);
  CK(cudaMemcpyAsync(lab.data(), g->vlab, 4 * (size_t)g->n, cudaMemcpyDeviceToHost, g->stream));
  CK(cudaStreamSynchronize(g->stream));
  for (int32_t v = 0; v < g->n; ++v) in_set[v] = lab[(size_t)v] < g->n ? 1 : 0;
  return WBPR_OK;
}

wbpr_status wbpr_mincut_adjoint(wbpr_graph* g, int32_t side, int8_t* indicator, float* adjoint_ms) {
  NvtxRange nvtx_("wbpr_mincut_adjoint");
  if (!g || !indicator || (side != 0 && side != 1)) return WBPR_ERR_INVALID_ARG;
  if (g->s < 0 || g->t < 0) return WBPR_ERR_INVALID_ARG;
  CK(cudaSetDevice(g->device));
  if (!g->ind) {
    wbpr_status st = dalloc(g, &g->ind, (size_t)g->m);
    if (st) return st;
  }
  CK(cudaEventRecord(g->ev0, g->stream));
  wbpr_status st;
  if (side == 0) {
    st = bfs_labels(g, g->t, 0, -1);
  } else {
    st = return_stranded(g);
    if (st) return st;
    st = bfs_labels(g, g->s, 1, -1);
  }
  if (st) return st;
  indicator_kernel<<<g->sms * 8, 256, 0, g->stream>>>(g->ioff, g->row, g->arc, g->farc, g->vlab, g->n, g->m,
                                                      side, g->ind);
  CK(cudaGetLastError());
  CK(cudaEventRecord(g->ev1, g->stream));
  // the caller's buffer may be host or device memory
  cudaPointerAttributes pa;
  const bool on_device = cudaPointerGetAttributes(&pa, indicator) == cudaSuccess &&
                         (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged);
  cudaGetLastError();
  CK(cudaMemcpyAsync(indicator, g->ind, (size_t)g->m, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                     g->stream));
  CK(cudaStreamSynchronize(g->stream));
  if (adjoint_ms) CK(cudaEventElapsedTime(adjoint_ms, g->ev0, g->ev1));
  return WBPR_OK;
}

int32_t wbpr_rcsr_preflow(int32_t V, int32_t source, int32_t sink, int32_t* cpu_height,
                          int32_t* cpu_excess_flow, const int32_t* offsets,
                          const int32_t* destinations, const int32_t* capacities,
                          int32_t* forward_flows, int32_t* backward_flows, const int32_t*,
                          const int32_t*, const int32_t*, int32_t* Excess_total) {
  if (V < 2 || source < 0 || source >= V || sink < 0 || sink >= V || source == sink || !cpu_height ||
      !cpu_excess_flow || !offsets || !destinations || !capacities || !forward_flows ||
      !backward_flows || !Excess_total)
    return WBPR_ERR_INVALID_ARG;
  for (int i = 0; i < V; ++i) {
    cpu_height[i] = 0;
    cpu_excess_flow[i] = 0;
  }
  cpu_height[source] = V;
  int64_t total = 0;
  for (int i = offsets[source]; i < offsets[source + 1]; ++i) {
    const int v = destinations[i];
    if (v < 0 || v >= V) return WBPR_ERR_INVALID_ARG;
    if (capacities[i] > 0) {
      forward_flows[i] = 0;
      backward_flows[i] = capacities[i];
      const int64_t ev = (int64_t)cpu_excess_flow[v] + capacities[i];
      total += capacities[i];
      if (ev > std::numeric_limits<int32_t>::max() || total > std::numeric_limits<int32_t>::max())
        return WBPR_ERR_OVERFLOW;
      cpu_excess_flow[v] = (int32_t)ev;
    }
  }
  *Excess_total = (int32_t)total;
  return WBPR_OK;
}

int32_t wbpr_rcsr_push_relabel(int32_t algo_type, int32_t V, int32_t E, int32_t source, int32_t sink,
                               int32_t* cpu_height, int32_t* cpu_excess_flow,
                               const int32_t* cpu_offsets, const int32_t* cpu_destinations,
                               const int32_t* cpu_capacities, int32_t* cpu_fflows,
                               int32_t* cpu_bflows, const int32_t*, const int32_t*, const int32_t*,
                               int32_t* Excess_total, float* kernel_ms) {
  if (!cpu_height || !cpu_excess_flow || !cpu_fflows || !cpu_bflows || !Excess_total)
    return WBPR_ERR_INVALID_ARG;
  if (algo_type != 0 && algo_type != 1) return WBPR_ERR_INVALID_ARG;
  wbpr_csr c{V, E, cpu_offsets, cpu_destinations, cpu_capacities, source, sink};
  wbpr_graph* g = nullptr;
  // the reverse pairing is rebuilt exactly from the forward CSR; the caller's
  // roffsets / rdestinations / flow_idx are not needed on the device
  wbpr_status st = create_impl(&c, WBPR_LAYOUT_RCSR, &g);
  if (st) return st;
  struct Guard {
    wbpr_graph* g;
    ~Guard() { release(g); }
  } guard{g};
  if (source < 0 || sink < 0 || source >= V || sink >= V || source == sink) return WBPR_ERR_INVALID_ARG;
  // upload the caller's preflow state
  std::vector<int32_t> farc(2 * (size_t)E);
  for (int64_t i = 0; i < E; ++i) {
    if (cpu_fflows[i] < 0 || cpu_bflows[i] < 0 ||
        (int64_t)cpu_fflows[i] + cpu_bflows[i] != (int64_t)(cpu_capacities ? cpu_capacities[i] : 1))
      return WBPR_ERR_INVALID_ARG;
    farc[2 * i] = cpu_destinations[i];
    farc[2 * i + 1] = cpu_fflows[i];
  }
  CK(cudaSetDevice(g->device));
  if (E) {
    CK(cudaMemcpy(g->farc, farc.data(), 8 * (size_t)E, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(g->fcb, cpu_bflows, 4 * (size_t)E, cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(g->e, cpu_excess_flow, 4 * (size_t)V, cudaMemcpyHostToDevice));
  RunCfg rc;
  st = make_cfg(g, source, sink, (wbpr_algo)algo_type, nullptr, &rc);
  if (st) return st;
  rc.mode = kModeState;
  rc.bfs_excl = source;
  Stats hs;
  st = run(g, rc, &hs);
  if (st) return st;
  if (E) {
    CK(cudaMemcpy(farc.data(), g->farc, 8 * (size_t)E, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cpu_bflows, g->fcb, 4 * (size_t)E, cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < E; ++i) cpu_fflows[i] = farc[2 * i + 1];
  }
  CK(cudaMemcpy(cpu_excess_flow, g->e, 4 * (size_t)V, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(cpu_height, g->h, 4 * (size_t)V, cudaMemcpyDeviceToHost));
  cpu_height[source] = V;
  *Excess_total = cpu_excess_flow[source] + cpu_excess_flow[sink];
  if (kernel_ms) *kernel_ms = (float)(hs.round_ns * 1e-6);
  return WBPR_OK;
}

}  // extern "C"
