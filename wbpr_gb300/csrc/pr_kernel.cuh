// Persistent push-relabel solver for sm_103a.
//
// One cooperative launch runs a whole solve: reset + preflow, then a loop of
//   global relabel (direction-optimising BFS from the sink, in-kernel)
//   -> push/relabel rounds until the active set is empty or the work since the
//      last global relabel exceeds a threshold.
// Each round has two phases separated by a bounded grid barrier:
//   push phase   labels are frozen; every active vertex u pushes along its
//                admissible arcs (label(u) == label(v) + 1) in arc order,
//                allotting its excess with a saturating prefix sum over the
//                tile (or block, for heavy rows).  For any residual pair only
//                one endpoint can be admissible in a round, so the two
//                residual words of the pair are updated with plain stores;
//                only excess(v) needs an atomic.  A vertex that keeps excess
//                records min label over its remaining residual arcs.
//   relabel phase every vertex that kept excess sets label = 1 + min(...),
//                also counting arcs opened by pushes it received in the same
//                round (those heads sit exactly one label higher), so the
//                labelling stays valid and labels only grow.
// With valid labels, an empty active set (no vertex with excess and label < n
// other than s, t) means the preflow is maximum and excess(t) is the value
// (Goldberg-Tarjan phase 1).  This replaces the reference's thread-centric
// and vertex-centric kernels (maxflow-cuda/src/push_relabel_kernel.cu:14-158,
// 400-537), its active-vertex scan (:160-192), the warp min-height search
// (:253-397) and both global relabels (maxflow-cuda/src/global_relabel.cu:4-178,
// maxflow-bcsr/src/global_relabel_gpu.cu:122-189).
//
// Every grid-wide wait is bounded (globaltimer); on timeout the kernel records
// WBPR_ERR_TIMEOUT and all blocks leave.  No trap, no unbounded spin.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "wbpr.h"

namespace wbpr_dev {

namespace cg = cooperative_groups;

constexpr int kNone = -1;
constexpr int kBig = 0x7fffffff;
constexpr int kBfsAlpha = 14;  // top-down -> bottom-up when frontier arcs * alpha > unvisited arcs
constexpr int kBfsBeta = 24;   // bottom-up -> top-down when frontier * beta < n
constexpr int kLightDeg = 32;  // BFS: rows up to this length scanned by one thread
constexpr int kHeavyDeg = 2048;  // BFS: rows longer than this scanned by a whole block

enum Mode : int {
  kModeFresh = 0,   // reset residuals, preflow, solve
  kModeState = 1,   // solve from the current residuals / excess (no reset)
  kModeBfsOnly = 2  // only the BFS into `lab` (verification / adjoint)
};

// Device control block (scratch owned by the graph handle).
struct Ctl {
  unsigned bar_count;
  unsigned bar_gen;
  int err;
  int stop;
  int lcount[2];
  int hcount[2];
  int qraw_count[2];
  int light_next;
  int heavy_next;
  int fcount[3];
  int fhcount[3];
  long long fdeg[3];
  unsigned long long work[2];  // work done in rounds of even / odd parity
  int bfs_heavy_next[3];
  int pad[5];
};

struct Stats {
  unsigned long long arcs_scanned;
  unsigned long long pushes;
  unsigned long long relabels;
  unsigned long long vertex_visits;
  unsigned long long bfs_arcs;
  unsigned long long bfs_vertices;
  unsigned long long gr_ns;
  unsigned long long round_ns;
  int rounds;
  int grs;
  int stranded;
  int status;
};

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ldv(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ long long ldv64(const long long* p) { return *(const volatile long long*)p; }

// ---------------------------------------------------------------------------
// Residual topologies.  load() returns (head, residual of u->head); push()
// moves p units along the arc and its twin; twin_cf() is the residual of the
// opposite arc head->u.
struct TopoB {  // BCSR16: row[n+1], arc {dst, cf}, arx {rev, cap}
  const int* row;
  int2* arc;
  const int2* arx;
  static constexpr int kSeg = 1;
  __device__ __forceinline__ void seg(int u, int, int& b, int& e) const {
    b = __ldg(row + u);
    e = __ldg(row + u + 1);
  }
  __device__ __forceinline__ int deg(int u) const { return __ldg(row + u + 1) - __ldg(row + u); }
  __device__ __forceinline__ void load(int, int a, int& dst, int& cf) const {
    int2 r = __ldcg(arc + a);
    dst = r.x;
    cf = r.y;
  }
  __device__ __forceinline__ int head(int, int a) const { return __ldcg(&arc[a].x); }
  __device__ __forceinline__ void push(int, int a, int cf, int p) const {
    arc[a].y = cf - p;
    int r = __ldg(&arx[a].x);
    int* tc = &arc[r].y;
    *tc = __ldcg(tc) + p;
  }
  __device__ __forceinline__ int twin_cf(int, int a) const {
    int r = __ldg(&arx[a].x);
    return __ldcg(&arc[r].y);
  }
};

struct TopoR {  // RCSR: forward {dst, cf_f} + cf_b, reverse {tail, forward id}
  const int* frow;
  int2* farc;
  int* fcb;
  const int* rrow;
  const int2* rarc;
  static constexpr int kSeg = 2;
  __device__ __forceinline__ void seg(int u, int k, int& b, int& e) const {
    const int* r = k == 0 ? frow : rrow;
    b = __ldg(r + u);
    e = __ldg(r + u + 1);
  }
  __device__ __forceinline__ int deg(int u) const {
    return __ldg(frow + u + 1) - __ldg(frow + u) + __ldg(rrow + u + 1) - __ldg(rrow + u);
  }
  __device__ __forceinline__ void load(int k, int a, int& dst, int& cf) const {
    if (k == 0) {
      int2 r = __ldcg(farc + a);
      dst = r.x;
      cf = r.y;
    } else {
      int2 r = __ldg(rarc + a);
      dst = r.x;
      cf = __ldcg(fcb + r.y);
    }
  }
  __device__ __forceinline__ int head(int k, int a) const {
    return k == 0 ? __ldcg(&farc[a].x) : __ldg(&rarc[a].x);
  }
  __device__ __forceinline__ void push(int k, int a, int cf, int p) const {
    if (k == 0) {
      farc[a].y = cf - p;
      fcb[a] = __ldcg(fcb + a) + p;
    } else {
      int fi = __ldg(&rarc[a].y);
      fcb[fi] = cf - p;
      farc[fi].y = __ldcg(&farc[fi].y) + p;
    }
  }
  __device__ __forceinline__ int twin_cf(int k, int a) const {
    if (k == 0) return __ldcg(fcb + a);
    int fi = __ldg(&rarc[a].y);
    return __ldcg(&farc[fi].y);
  }
};

template <class Topo>
struct Params {
  Topo g;
  int n;
  int s;  // excluded vertex (the source; t in phase-2 solves)
  int t;  // absorbing vertex (the sink; s in phase-2 solves)
  int* lab;
  int* e;
  int* rl_min;
  int* rl_left;
  int* lq[2];
  int* hq[2];
  int* qraw;
  int* fr[3];
  int* frh[3];
  const int* cls;  // vertex ids: [0, n_light) light, then medium, then heavy
  int n_light;
  int n_medium;
  int n_heavy;
  Ctl* ctl;
  Stats* st;
  long long total_deg;
  unsigned long long gr_threshold;
  long long max_rounds;
  unsigned long long budget_ns;
  unsigned long long bar_timeout_ns;
  int heavy_deg;
  int mode;
  int bfs_dir;   // 0: vertices that reach the root (to sink); 1: reached from the root
  int bfs_root;
  int bfs_excl;  // vertex the BFS never labels (the source during a solve), or -1
};

// Per-block counters, flushed to Stats once per phase.
struct BlockAcc {
  unsigned long long scanned;
  unsigned long long pushes;
  unsigned long long relabels;
  unsigned long long visits;
  unsigned long long bfs_arcs;
  unsigned long long bfs_vertices;
  long long fdeg;
  int sink;
  int pad;
};

// ---------------------------------------------------------------------------
// Bounded grid barrier.  Thread 0 of each block arrives on a counter; the last
// arrival resets it and bumps the generation.  Waiting gives up after
// timeout_ns of globaltimer time and records WBPR_ERR_TIMEOUT.
__device__ __forceinline__ bool grid_sync(Ctl* c, unsigned long long timeout_ns) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* genp = &c->bar_gen;
    unsigned g = *genp;
    __threadfence();
    unsigned arrived = atomicAdd(&c->bar_count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&c->bar_count, 0u);
      __threadfence();
      atomicAdd(&c->bar_gen, 1u);
    } else {
      unsigned long long t0 = gtime();
      unsigned ns = 32;
      while (*genp == g) {
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
        if (gtime() - t0 > timeout_ns) {
          atomicCAS(&c->err, 0, (int)WBPR_ERR_TIMEOUT);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ldv(&c->err) == 0;
}

// Warp-aggregated append of v to q[*cnt] (one atomic per converged group).
__device__ __forceinline__ void append(int* q, int* cnt, int v) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(cnt, (int)g.size());
  base = g.shfl(base, 0);
  q[base + g.thread_rank()] = v;
}

__device__ __forceinline__ void flush_acc(BlockAcc& a, Stats* st,
                                          unsigned long long* work = nullptr) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long w = a.scanned + a.visits + a.relabels;
    if (work && w) atomicAdd(work, w);
    if (a.scanned) atomicAdd(&st->arcs_scanned, a.scanned);
    if (a.pushes) atomicAdd(&st->pushes, a.pushes);
    if (a.relabels) atomicAdd(&st->relabels, a.relabels);
    if (a.visits) atomicAdd(&st->vertex_visits, a.visits);
    if (a.bfs_arcs) atomicAdd(&st->bfs_arcs, a.bfs_arcs);
    if (a.bfs_vertices) atomicAdd(&st->bfs_vertices, a.bfs_vertices);
    a.scanned = a.pushes = a.relabels = a.visits = a.bfs_arcs = a.bfs_vertices = 0;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Push phase: one tile of W lanes (W = 1 is the thread-centric form).
template <class Topo, int W>
__device__ __forceinline__ void discharge_tile(const Params<Topo>& p, int u, int* rawcnt,
                                               BlockAcc& acc) {
  const unsigned lw = threadIdx.x & 31u;
  const int lane = (W == 1) ? 0 : (int)(lw & (W - 1));
  const unsigned mask =
      (W == 32) ? 0xffffffffu : (W == 1 ? (1u << lw) : (((1u << W) - 1u) << (lw & ~(unsigned)(W - 1))));
  const int hu = __ldcg(p.lab + u);
  int eu = 0;
  if (lane == 0) eu = ldv(p.e + u);
  if (W > 1) eu = __shfl_sync(mask, eu, 0, W);
  if (eu <= 0 || hu >= p.n) return;
  unsigned erem = (unsigned)eu;
  const int th = hu - 1;
  int minh = kBig;
  int npush = 0;
  unsigned long long scanned = 0;
#pragma unroll 1
  for (int k = 0; k < Topo::kSeg; ++k) {
    int b, e;
    p.g.seg(u, k, b, e);
#pragma unroll 1
    for (int base = b; base < e; base += W) {
      const int a = base + lane;
      int dst = 0, cf = 0, hv = kBig;
      if (a < e) {
        p.g.load(k, a, dst, cf);
        if (cf > 0) hv = __ldcg(p.lab + dst);
      }
      const bool adm = (cf > 0) && (hv == th);
      const unsigned am = (W == 1) ? (unsigned)adm : __ballot_sync(mask, adm);
      int pushed = 0;
      if (am) {
        unsigned incl = adm ? (unsigned)cf : 0u;
        if (incl > erem) incl = erem;
        unsigned prev = 0, total = incl;
        if (W > 1) {
#pragma unroll
          for (int d = 1; d < W; d <<= 1) {
            unsigned y = __shfl_up_sync(mask, incl, d, W);
            if (lane >= d) {
              incl += y;
              if (incl > erem) incl = erem;
            }
          }
          prev = __shfl_up_sync(mask, incl, 1, W);
          if (lane == 0) prev = 0;
          total = __shfl_sync(mask, incl, W - 1, W);
        }
        pushed = (int)(incl - prev);
        erem -= total;
        if (pushed > 0) {
          p.g.push(k, a, cf, pushed);
          ++npush;
          if (dst == p.t) {
            atomicAdd(&acc.sink, pushed);
          } else {
            int old = atomicAdd(p.e + dst, pushed);
            if (old == 0) append(p.qraw, rawcnt, dst);
          }
        }
      }
      if (cf - pushed > 0 && hv < minh) minh = hv;
      if (lane == 0) scanned += (unsigned long long)min(W, e - base);
      if (erem == 0) break;
    }
    if (erem == 0) break;
  }
  if (W > 1) minh = __reduce_min_sync(mask, minh);
  if (npush) atomicAdd(&acc.pushes, (unsigned long long)npush);
  if (lane == 0) {
    const int D = eu - (int)erem;
    bool self = true;
    if (D > 0) self = (atomicSub(p.e + u, D) - D) > 0;
    if (erem > 0) {
      p.rl_min[u] = minh;
      p.rl_left[u] = (int)erem;
    }
    if (self) append(p.qraw, rawcnt, u);
    atomicAdd(&acc.scanned, scanned);
    atomicAdd(&acc.visits, 1ull);
  }
}

// Push phase for one heavy row: the whole block walks the row in slabs of
// blockDim * kItems arcs (loads issued together), block-wide saturating scan.
constexpr int kItems = 4;

template <class Topo>
__device__ void discharge_block(const Params<Topo>& p, int u, int* rawcnt, BlockAcc& acc) {
  __shared__ unsigned s_wsum[32];
  __shared__ unsigned s_tot;
  __shared__ int s_eu;
  __shared__ int s_min[32];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  const int hu = __ldcg(p.lab + u);
  if (tid == 0) s_eu = ldv(p.e + u);
  __syncthreads();
  const int eu = s_eu;
  __syncthreads();
  if (eu <= 0 || hu >= p.n) return;
  unsigned erem = (unsigned)eu;
  const int th = hu - 1;
  int minh = kBig;
  int npush = 0;
  unsigned long long scanned = 0;
  for (int k = 0; k < Topo::kSeg && erem > 0; ++k) {
    int b, e;
    p.g.seg(u, k, b, e);
    for (int base = b; base < e && erem > 0; base += blockDim.x * kItems) {
      int dst[kItems], cf[kItems], hv[kItems];
#pragma unroll
      for (int j = 0; j < kItems; ++j) {
        const int a = base + j * blockDim.x + tid;
        dst[j] = 0;
        cf[j] = 0;
        if (a < e) p.g.load(k, a, dst[j], cf[j]);
      }
#pragma unroll
      for (int j = 0; j < kItems; ++j) hv[j] = cf[j] > 0 ? __ldcg(p.lab + dst[j]) : kBig;
      if (tid == 0) scanned += (unsigned long long)min(blockDim.x * kItems, e - base);
#pragma unroll 1
      for (int j = 0; j < kItems; ++j) {
        const int a = base + j * blockDim.x + tid;
        const bool adm = cf[j] > 0 && hv[j] == th;
        int pushed = 0;
        if (__syncthreads_or(adm)) {
          unsigned incl = adm ? (unsigned)cf[j] : 0u;
          if (incl > erem) incl = erem;
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= d) {
              incl += y;
              if (incl > erem) incl = erem;
            }
          }
          unsigned prevw = __shfl_up_sync(0xffffffffu, incl, 1);
          if (lane == 0) prevw = 0;
          if (lane == 31) s_wsum[wid] = incl;
          __syncthreads();
          if (wid == 0) {
            unsigned v = lane < nw ? s_wsum[lane] : 0u;
            unsigned inc2 = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
              unsigned y = __shfl_up_sync(0xffffffffu, inc2, d);
              if (lane >= d) {
                inc2 += y;
                if (inc2 > erem) inc2 = erem;
              }
            }
            unsigned exc2 = __shfl_up_sync(0xffffffffu, inc2, 1);
            if (lane == 0) exc2 = 0;
            if (lane < nw) s_wsum[lane] = exc2;
            if (lane == nw - 1) s_tot = inc2;
          }
          __syncthreads();
          const unsigned wpre = s_wsum[wid];
          unsigned ib = wpre + incl, pb = wpre + prevw;
          if (ib > erem) ib = erem;
          if (pb > erem) pb = erem;
          pushed = (int)(ib - pb);
          const unsigned total = s_tot;
          __syncthreads();
          erem -= total;
          if (pushed > 0) {
            p.g.push(k, a, cf[j], pushed);
            ++npush;
            if (dst[j] == p.t) {
              atomicAdd(&acc.sink, pushed);
            } else {
              int old = atomicAdd(p.e + dst[j], pushed);
              if (old == 0) append(p.qraw, rawcnt, dst[j]);
            }
          }
        }
        if (cf[j] - pushed > 0 && hv[j] < minh) minh = hv[j];
        if (erem == 0) break;
      }
    }
  }
  // block min over remaining residual arcs
  minh = __reduce_min_sync(0xffffffffu, minh);
  if (lane == 0) s_min[wid] = minh;
  __syncthreads();
  if (tid == 0) {
    int mh = kBig;
    for (int w = 0; w < nw; ++w) mh = min(mh, s_min[w]);
    const int D = eu - (int)erem;
    bool self = true;
    if (D > 0) self = (atomicSub(p.e + u, D) - D) > 0;
    if (erem > 0) {
      p.rl_min[u] = mh;
      p.rl_left[u] = (int)erem;
    }
    if (self) append(p.qraw, rawcnt, u);
    atomicAdd(&acc.scanned, scanned);
    atomicAdd(&acc.visits, 1ull);
  }
  if (npush) atomicAdd(&acc.pushes, (unsigned long long)npush);
  __syncthreads();
}

template <class Topo, int W>
__device__ void push_phase(const Params<Topo>& p, int cur, int raw, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int nH = ldv(&c->hcount[cur]);
  const int nL = ldv(&c->lcount[cur]);
  int* rawcnt = &c->qraw_count[raw];
  __shared__ int s_item;
  // heavy rows first (whole block each), dynamically claimed
  for (;;) {
    if (threadIdx.x == 0) s_item = nH > 0 ? atomicAdd(&c->heavy_next, 1) : nH;
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nH) break;
    discharge_block<Topo>(p, __ldcg(p.hq[cur] + it), rawcnt, acc);
  }
  // light rows: each warp claims 2 entries per tile at a time
  constexpr int kTpw = 32 / W;
  constexpr int kGrab = 2 * kTpw;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int base = 0;
    if (lane == 0) base = atomicAdd(&c->light_next, kGrab);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= nL) break;
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const int idx = base + r * kTpw + lane / W;
      if (idx < nL) discharge_tile<Topo, W>(p, __ldcg(p.lq[cur] + idx), rawcnt, acc);
    }
    __syncwarp();
  }
  __syncthreads();
  if (threadIdx.x == 0 && acc.sink) {
    atomicAdd(p.e + p.t, acc.sink);
    acc.sink = 0;
  }
}

// Relabel phase over the raw next queue; also files the survivors into the
// light / heavy lists of the next round.
template <class Topo>
__device__ void relabel_phase(const Params<Topo>& p, int cur, int nxt, int raw, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int nq = ldv(&c->qraw_count[raw]);
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  unsigned long long rl = 0;
  for (int i = gt; i < nq; i += gs) {
    const int u = __ldcg(p.qraw + i);
    int m = __ldcg(p.rl_min + u);
    int hu = __ldcg(p.lab + u);
    const int eu = ldv(p.e + u);
    if (m != kNone) {
      p.rl_min[u] = kNone;
      if (eu > __ldcg(p.rl_left + u) && hu + 1 < m) m = hu + 1;
      int nh = (m >= p.n - 1) ? p.n : m + 1;
      if (nh <= hu) nh = hu + 1;
      if (nh > p.n) nh = p.n;
      p.lab[u] = nh;
      hu = nh;
      ++rl;
    }
    if (eu > 0 && hu < p.n) {
      if (p.g.deg(u) > p.heavy_deg) append(p.hq[nxt], &c->hcount[nxt], u);
      else append(p.lq[nxt], &c->lcount[nxt], u);
    }
  }
  if (rl) atomicAdd(&acc.relabels, rl);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c->lcount[cur] = 0;
    c->hcount[cur] = 0;
    c->qraw_count[raw ^ 1] = 0;
    c->work[raw ^ 1] = 0;
    c->light_next = 0;
    c->heavy_next = 0;
  }
}

// ---------------------------------------------------------------------------
// Global relabel: level-synchronous BFS over residual arcs from `root`.
// DIR 0 labels every vertex with its residual distance TO the root (the
// reference's backward BFS from the sink); DIR 1 with its distance FROM the
// root.  Unreached vertices keep label n.  Top-down expands the frontier
// (warp per light row, all warps of the grid per heavy row); bottom-up lets
// every unvisited vertex look for a frontier neighbour (thread / warp / block
// per row by length class).
template <class Topo, int DIR>
__device__ __forceinline__ bool bfs_edge(const Params<Topo>& p, int k, int a, int& dst) {
  // true when the arc a (in the row of x, head dst) links dst to the row
  // owner in the BFS direction: DIR 0 needs residual dst -> x, DIR 1 x -> dst.
  int cf;
  if (DIR == 0) {
    dst = p.g.head(k, a);
    (void)cf;
    return true;
  } else {
    p.g.load(k, a, dst, cf);
    return cf > 0;
  }
}

template <class Topo>
__device__ __forceinline__ void bfs_discover(const Params<Topo>& p, int v, int level, int fn,
                                             BlockAcc& acc) {
  const int d = p.g.deg(v);
  if (d > kHeavyDeg) append(p.frh[fn], &p.ctl->fhcount[fn], v);
  else append(p.fr[fn], &p.ctl->fcount[fn], v);
  atomicAdd((unsigned long long*)&acc.fdeg, (unsigned long long)d);
}

template <class Topo, int DIR>
__device__ __forceinline__ void td_arc(const Params<Topo>& p, int k, int a, int level, int fn,
                                       BlockAcc& acc, unsigned long long& arcs) {
  int dst, cf;
  bool ok;
  if (DIR == 0) {
    dst = p.g.head(k, a);
    ok = true;
  } else {
    p.g.load(k, a, dst, cf);
    ok = cf > 0;
  }
  ++arcs;
  if (!ok || dst == p.bfs_excl || __ldcg(p.lab + dst) != p.n) return;
  if (DIR == 0 && p.g.twin_cf(k, a) <= 0) return;
  if (atomicCAS(p.lab + dst, p.n, level + 1) == p.n) bfs_discover(p, dst, level, fn, acc);
}

// does the arc a of row x make x adjacent to a vertex labelled `level`?
template <class Topo, int DIR>
__device__ __forceinline__ bool bu_arc(const Params<Topo>& p, int k, int a, int level) {
  int dst, cf;
  p.g.load(k, a, dst, cf);
  if (DIR == 0) {
    if (cf <= 0) return false;
    return __ldcg(p.lab + dst) == level;
  } else {
    if (__ldcg(p.lab + dst) != level) return false;
    return p.g.twin_cf(k, a) > 0;
  }
}

template <class Topo, int DIR>
__device__ void bfs_top_down(const Params<Topo>& p, int level, int fc, int fn, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int nf = ldv(&c->fcount[fc]);
  const int nfh = ldv(&c->fhcount[fc]);
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long arcs = 0;
  // heavy frontier rows: every warp of the grid takes 32-arc chunks
  for (int i = 0; i < nfh; ++i) {
    const int x = __ldcg(p.frh[fc] + i);
    for (int k = 0; k < Topo::kSeg; ++k) {
      int b, e;
      p.g.seg(x, k, b, e);
      for (int a = b + gw * 32 + lane; a < e; a += nwarps * 32) td_arc<Topo, DIR>(p, k, a, level, fn, acc, arcs);
    }
  }
  // light frontier rows: warp per row
  for (int i = gw; i < nf; i += nwarps) {
    const int x = __ldcg(p.fr[fc] + i);
    for (int k = 0; k < Topo::kSeg; ++k) {
      int b, e;
      p.g.seg(x, k, b, e);
      for (int a = b + lane; a < e; a += 32) td_arc<Topo, DIR>(p, k, a, level, fn, acc, arcs);
    }
  }
  if (arcs) atomicAdd(&acc.bfs_arcs, arcs);
}

template <class Topo, int DIR>
__device__ void bfs_bottom_up(const Params<Topo>& p, int level, int fn, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int gw = gt >> 5, nwarps = gs >> 5;
  unsigned long long arcs = 0, verts = 0;
  // light rows: one thread each
  for (int i = gt; i < p.n_light; i += gs) {
    const int x = __ldg(p.cls + i);
    ++verts;
    if (x == p.bfs_excl || __ldcg(p.lab + x) != p.n) continue;
    bool hit = false;
    for (int k = 0; k < Topo::kSeg && !hit; ++k) {
      int b, e;
      p.g.seg(x, k, b, e);
      for (int a = b; a < e; ++a) {
        ++arcs;
        if (bu_arc<Topo, DIR>(p, k, a, level)) { hit = true; break; }
      }
    }
    if (hit) {
      p.lab[x] = level + 1;
      bfs_discover(p, x, level, fn, acc);
    }
  }
  // medium rows: one warp each
  for (int i = gw; i < p.n_medium; i += nwarps) {
    const int x = __ldg(p.cls + p.n_light + i);
    if (lane == 0) ++verts;
    if (x == p.bfs_excl || __ldcg(p.lab + x) != p.n) continue;
    bool hit = false;
    for (int k = 0; k < Topo::kSeg && !hit; ++k) {
      int b, e;
      p.g.seg(x, k, b, e);
      for (int base = b; base < e; base += 32) {
        const int a = base + lane;
        bool h = false;
        if (a < e) { ++arcs; h = bu_arc<Topo, DIR>(p, k, a, level); }
        if (__any_sync(0xffffffffu, h)) { hit = true; break; }
      }
    }
    if (hit && lane == 0) {
      p.lab[x] = level + 1;
      bfs_discover(p, x, level, fn, acc);
    }
  }
  if (arcs) atomicAdd(&acc.bfs_arcs, arcs);
  if (verts) atomicAdd(&acc.bfs_vertices, verts);
  // heavy rows: one block each, claimed dynamically
  __shared__ int s_item;
  const int cur3 = (level) % 3;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(&c->bfs_heavy_next[cur3], 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= p.n_heavy) break;
    const int x = __ldg(p.cls + p.n_light + p.n_medium + it);
    if (x == p.bfs_excl || __ldcg(p.lab + x) != p.n) continue;  // uniform per block
    bool hit = false;
    unsigned long long ha = 0;
    for (int k = 0; k < Topo::kSeg && !hit; ++k) {
      int b, e;
      p.g.seg(x, k, b, e);
      for (int base = b; base < e; base += blockDim.x) {
        const int a = base + threadIdx.x;
        bool h = false;
        if (a < e) { ++ha; h = bu_arc<Topo, DIR>(p, k, a, level); }
        if (__syncthreads_or(h)) { hit = true; break; }
      }
    }
    if (ha) atomicAdd(&acc.bfs_arcs, ha);
    if (hit && threadIdx.x == 0) {
      p.lab[x] = level + 1;
      bfs_discover(p, x, level, fn, acc);
    }
  }
}

// Full BFS; on return every block has passed the closing barrier.  When
// `queues` is set, the light/heavy active lists `cur` are rebuilt from the new
// labels (vertices with excess and label < n, other than s and t).
template <class Topo, int DIR>
__device__ bool bfs(const Params<Topo>& p, int root, bool queues, int cur, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  for (int v = gt; v < p.n; v += gs) p.lab[v] = (v == root) ? 0 : p.n;
  if (gt == 0) {
    const int d = p.g.deg(root);
    if (d > kHeavyDeg) {
      p.frh[0][0] = root;
      c->fhcount[0] = 1;
      c->fcount[0] = 0;
    } else {
      p.fr[0][0] = root;
      c->fcount[0] = 1;
      c->fhcount[0] = 0;
    }
    c->fcount[1] = c->fcount[2] = 0;
    c->fhcount[1] = c->fhcount[2] = 0;
    c->fdeg[0] = d;
    c->fdeg[1] = c->fdeg[2] = 0;
    c->bfs_heavy_next[0] = c->bfs_heavy_next[1] = c->bfs_heavy_next[2] = 0;
    if (queues) {
      c->lcount[cur] = 0;
      c->hcount[cur] = 0;
      c->light_next = 0;
      c->heavy_next = 0;
    }
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return false;
  // Every block derives the direction from values that are final at the
  // barrier (frontier size and degree of this level), so all blocks agree.
  bool bu = false;
  long long visited = 0;
  for (int level = 0;; ++level) {
    const int fc = level % 3, fn = (level + 1) % 3, fr = (level + 2) % 3;
    const int nf = ldv(&c->fcount[fc]) + ldv(&c->fhcount[fc]);
    if (nf == 0) break;
    const long long fdeg = ldv64(&c->fdeg[fc]);
    visited += fdeg;
    const long long rem = p.total_deg - visited;
    if (!bu && fdeg * kBfsAlpha > rem) bu = true;
    else if (bu && (long long)nf * kBfsBeta < (long long)p.n) bu = false;
    if (gt == 0) {
      c->fcount[fr] = 0;
      c->fhcount[fr] = 0;
      c->fdeg[fr] = 0;
      c->bfs_heavy_next[fn] = 0;
    }
    if (threadIdx.x == 0) acc.fdeg = 0;
    __syncthreads();
    if (bu) bfs_bottom_up<Topo, DIR>(p, level, fn, acc);
    else bfs_top_down<Topo, DIR>(p, level, fc, fn, acc);
    __syncthreads();
    if (threadIdx.x == 0 && acc.fdeg)
      atomicAdd((unsigned long long*)&c->fdeg[fn], (unsigned long long)acc.fdeg);
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
  }
  if (queues) {
    const int nall = p.n_light + p.n_medium + p.n_heavy;
    for (int i = gt; i < nall; i += gs) {
      const int v = __ldg(p.cls + i);
      if (v == p.s || v == p.t) continue;
      if (ldv(p.e + v) > 0 && __ldcg(p.lab + v) < p.n) {
        if (p.g.deg(v) > p.heavy_deg) append(p.hq[cur], &c->hcount[cur], v);
        else append(p.lq[cur], &c->lcount[cur], v);
      }
    }
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
template <class Topo, int W>
__global__ void __launch_bounds__(256, 2) pr_persistent(Params<Topo> p) {
  __shared__ BlockAcc acc;
  Ctl* c = p.ctl;
  if (threadIdx.x == 0) {
    acc.scanned = acc.pushes = acc.relabels = acc.visits = acc.bfs_arcs = acc.bfs_vertices = 0;
    acc.fdeg = 0;
    acc.sink = 0;
  }
  __syncthreads();
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const unsigned long long t_start = gtime();

  if (p.mode == kModeBfsOnly) {
    if (p.bfs_dir == 0) bfs<Topo, 0>(p, p.bfs_root, false, 0, acc);
    else bfs<Topo, 1>(p, p.bfs_root, false, 0, acc);
    flush_acc(acc, p.st);
    return;
  }

  if (p.mode == kModeFresh) {
    // heights 0, excess 0, no pending relabel; residuals are reset by the
    // host-side reset kernel before this launch
    for (int v = gt; v < p.n; v += gs) {
      p.lab[v] = 0;
      p.e[v] = 0;
      p.rl_min[v] = kNone;
    }
    if (!grid_sync(c, p.bar_timeout_ns)) return;
    // preflow: saturate every residual arc out of s (reference preflow.cu:3-31,
    // with excess accumulated so parallel source arcs are kept)
    for (int k = 0; k < Topo::kSeg; ++k) {
      int b, e;
      p.g.seg(p.s, k, b, e);
      for (int a = b + gt; a < e; a += gs) {
        int dst, cf;
        p.g.load(k, a, dst, cf);
        if (cf > 0 && dst != p.s) {
          p.g.push(k, a, cf, cf);
          atomicAdd(p.e + dst, cf);
        }
      }
    }
  } else {
    for (int v = gt; v < p.n; v += gs) p.rl_min[v] = kNone;
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return;

  int cur = 0, raw = 0, rounds = 0;
  bool need_gr = true;
  // work since the last global relabel: every block adds the per-round
  // counter of the finished round (final at the barrier), so all agree
  unsigned long long work = 0;
  unsigned long long gr_ns = 0, round_ns = 0;
  for (;;) {
    if (need_gr) {
      const unsigned long long t0 = gtime();
      if (!bfs<Topo, 0>(p, p.t, true, cur, acc)) break;
      if (threadIdx.x == 0 && blockIdx.x == 0) {
        gr_ns += gtime() - t0;
        atomicAdd(&p.st->grs, 1);
      }
      need_gr = false;
      work = 0;
    }
    const int nact = ldv(&c->lcount[cur]) + ldv(&c->hcount[cur]);
    if (nact == 0) break;
    if (ldv(&c->stop)) {
      if (gt == 0) atomicCAS(&c->err, 0, (int)WBPR_ERR_NO_CONVERGENCE);
      break;
    }
    const unsigned long long t0 = gtime();
    push_phase<Topo, W>(p, cur, raw, acc);
    flush_acc(acc, p.st, &c->work[raw]);
    if (!grid_sync(c, p.bar_timeout_ns)) break;
    relabel_phase<Topo>(p, cur, cur ^ 1, raw, acc);
    flush_acc(acc, p.st, &c->work[raw]);
    if (gt == 0) {
      round_ns += gtime() - t0;
      if ((p.max_rounds > 0 && rounds + 1 >= p.max_rounds) || gtime() - t_start > p.budget_ns)
        c->stop = 1;
    }
    if (!grid_sync(c, p.bar_timeout_ns)) break;
    work += *(volatile unsigned long long*)&c->work[raw];
    ++rounds;
    cur ^= 1;
    raw ^= 1;
    if (work > p.gr_threshold) need_gr = true;
  }
  flush_acc(acc, p.st);
  if (gt == 0) {
    p.st->rounds = rounds;
    p.st->gr_ns = gr_ns;
    p.st->round_ns = round_ns;
  }
}

// Count vertices left with excess that cannot reach t (label n).
template <class Topo>
__global__ void count_stranded(Params<Topo> p) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  int cnt = 0;
  for (int v = gt; v < p.n; v += gs)
    if (v != p.s && v != p.t && p.e[v] > 0 && p.lab[v] >= p.n) ++cnt;
  if (cnt) atomicAdd(&p.st->stranded, cnt);
}

}  // namespace wbpr_dev
