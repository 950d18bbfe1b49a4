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
constexpr int kMaxPlateau = 8;
constexpr int kBfsAlpha = 14;  // default: top-down -> bottom-up when frontier arcs * alpha > unvisited arcs
#ifndef WBPR_BFS_BETA
#define WBPR_BFS_BETA 24
#endif
constexpr int kBfsBeta = WBPR_BFS_BETA;  // bottom-up -> top-down when frontier * beta < n
constexpr int kLightDeg = 32;  // BFS: rows up to this length scanned by one thread
constexpr int kHeavyDeg = 2048;  // BFS: rows longer than this scanned by a whole block
constexpr int kChunk = 2048;     // BFS: heavy rows are cut into static chunks of this many arcs

enum Mode : int {
  kModeFresh = 0,   // reset residuals, preflow, solve
  kModeState = 1,   // solve from the current residuals / excess (no reset)
  kModeBfsOnly = 2  // only the BFS into `lab` (verification / adjoint)
};

// Device control block (scratch owned by the graph handle).  Words that every
// block hits in the same phase sit on their own 128-byte lines, so the barrier
// word, the work-claim counters and the list counters do not share an L2 line.
constexpr int kWorkSlots = 32;  // the per-round work sum is spread over 32 lines
struct Ctl {
  alignas(128) unsigned bar;  // grid barrier word (zero at launch)
  alignas(128) int err;
  int stop;
  alignas(128) int lcount[2];
  int hcount[2];
  alignas(128) int qraw_count[2];
  alignas(128) int light_next;
  alignas(128) int heavy_next;
  alignas(128) int fcount[3];
  int fhcount[3];
  long long fdeg[3];
  alignas(128) unsigned long long dpack;  // deep list of the round: (entries << 32) | chunk items
  alignas(128) int bu_found[3];  // vertices labelled by a bottom-up level, by level % 3
  alignas(128) int bu_med[3];    // medium-row batches a bottom-up level has handed out, by level % 3
  int mcount;       // materialised frontier: short rows
  int glong;        // greedy routing: walkers left for the warp stage
  alignas(128) int glong_next;  //   and the claim counter of that stage
  int mhcount;      //   long-row chunk items
  alignas(128) int gr_ok;  // the rounds since the last global relabel took at least half as long as it
  int stalled;             // excess(t) has not changed for gr_stall rounds
  int viol;                // out-of-range indices seen by the checked build
  long long dead_deg;      // arcs of the vertices global relabels marked unable to reach the sink
  // work done in rounds of even / odd parity; block b adds to slot b % 32
  alignas(128) unsigned long long work[2][kWorkSlots * 16];
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
  unsigned long long push_ns;
  unsigned long long heavy_visits;
  unsigned long long deep_ns;       // deep passes A and B of the push phases
  unsigned long long deep_scanned;  // arcs those passes read (part of arcs_scanned)
  int rounds;
  int grs;
  int stranded;
  int status;
  int bfs_levels;
  int bu_levels;
  int trace_n;
  int pad2;
  unsigned long long t0;
};

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Whether more than limit ns have passed since t0.  The global timer follows
// the host clock, which can be stepped: the difference is taken signed, so a
// step back reads as no time passed instead of as a wrapped-around eternity.
__device__ __forceinline__ bool time_past(unsigned long long t0, unsigned long long limit) {
  return (long long)(gtime() - t0) > (long long)limit;
}
__device__ __forceinline__ int ldv(const int* p) { return *(const volatile int*)p; }

__device__ __forceinline__ void trace_rec(long long* tr, int cap, int* n, unsigned long long t0, int kind,
                                          int aux, long long v0, long long v1, long long v2, long long v3) {
  if (!tr) return;
  const int i = *n;
  *n = i + 1;
  long long* r = tr + 6 * (long long)(i % cap);
  r[0] = (long long)kind | ((long long)aux << 32);
  r[1] = (long long)(gtime() - t0);
  r[2] = v0;
  r[3] = v1;
  r[4] = v2;
  r[5] = v3;
}
// Record an event; v2 / v3 = longest / shortest work time of any block in
// the phase that just ended (each block stores it in bt[] before the barrier).
#define TRACE(p, kind, aux, v0, v1)                                                           \
  do {                                                                                        \
    if ((p).trace) {                                                                          \
      unsigned long long mx_ = 0, mn_ = ~0ull;                                                \
      for (int b_ = 0; b_ < (int)gridDim.x; ++b_) {                                           \
        const unsigned long long d_ = *(volatile unsigned long long*)((p).bt + b_);           \
        mx_ = d_ > mx_ ? d_ : mx_;                                                            \
        mn_ = d_ < mn_ ? d_ : mn_;                                                            \
      }                                                                                       \
      trace_rec((p).trace, (p).trace_cap, &(p).st->trace_n, (p).st->t0, (kind), (aux), (v0), \
                (v1), (long long)mx_, (long long)mn_);                                        \
    }                                                                                         \
  } while (0)
// each block stores how long its share of the current phase took
#define TRACE_BLOCK(p, tb)                                            \
  do {                                                                \
    if ((p).trace) {                                                  \
      __syncthreads();                                                \
      if (threadIdx.x == 0) (p).bt[blockIdx.x] = gtime() - (tb);      \
    }                                                                 \
  } while (0)
__device__ __forceinline__ long long ldv64(const long long* p) { return *(const volatile long long*)p; }
__device__ __forceinline__ unsigned long long ldv64u(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}

// ---------------------------------------------------------------------------
// Residual topologies.  load() returns (head, residual of u->head); push()
// moves p units along the arc and its twin; twin_cf() is the residual of the
// opposite arc head->u.
// Bounds of a topology for the checked build (compiled with -DWBPR_CHECKED):
// an arc index >= na or a vertex >= n is counted in *viol and replaced by 0,
// so the kernel still finishes and the host reports WBPR_ERR_VERIFY.  With
// viol == nullptr, or in the normal build, nothing is checked.
struct Bounds {
  int* viol = nullptr;
  long long na = 0;
  int n = 0;
};
__device__ __forceinline__ long long chk(const Bounds& b, long long i, long long lim) {
#ifdef WBPR_CHECKED
  if (b.viol && (unsigned long long)i >= (unsigned long long)lim) {
    atomicAdd(b.viol, 1);
    return 0;
  }
#endif
  return i;
}

// Undo log of a BCSR16 graph: every push records its arc, so the next fresh
// solve restores only the arcs (and their twins) that changed instead of
// rewriting all 2m residuals.  kLogSlots counters, one per 128-byte line,
// picked by warp (a burst of pushes, as in the greedy routing after the
// preflow, would otherwise queue on a few counters), each owning `ulog_cap`
// entries; a slot that fills up sets its overflow word and the next restore
// rewrites every arc.
constexpr int kLogSlots = 256;
constexpr int kLogStride = 32;  // ints between two slot counters: [0] count, [1] overflow

struct TopoB {  // BCSR16: row[n+1], arc {dst, cf}, arx {rev, cap}
  const int* row;
  int2* arc;
  const int2* arx;
  Bounds bd;
  int* ulog = nullptr;    // undo log (nullptr: not recorded)
  int* ulog_n = nullptr;  // kLogSlots x kLogStride counter words
  int ulog_cap = 0;       // entries per slot
  static constexpr int kSeg = 1;
  __device__ __forceinline__ void seg(int u, int, int& b, int& e) const {
    u = (int)chk(bd, u, bd.n);
    b = __ldg(row + u);
    e = __ldg(row + u + 1);
  }
  __device__ __forceinline__ int deg(int u) const {
    u = (int)chk(bd, u, bd.n);
    return __ldg(row + u + 1) - __ldg(row + u);
  }
  __device__ __forceinline__ void load(int, int a, int& dst, int& cf) const {
    a = (int)chk(bd, a, bd.na);
    int2 r = __ldcg(arc + a);
    dst = (int)chk(bd, r.x, bd.n);
    cf = r.y;
  }
  __device__ __forceinline__ int head(int, int a) const {
    a = (int)chk(bd, a, bd.na);
    return (int)chk(bd, __ldcg(&arc[a].x), bd.n);
  }
  __device__ __forceinline__ void push(int, int a, int cf, int p) const {
    a = (int)chk(bd, a, bd.na);
    arc[a].y = cf - p;
    int r = (int)chk(bd, __ldg(&arx[a].x), bd.na);
    int* tc = &arc[r].y;
    *tc = __ldcg(tc) + p;
    log_push(a);
  }
  // record arc a (and so its twin) in the undo log
  __device__ __forceinline__ void log_push(int a) const {
    if (!ulog) return;
    const int slot = ((blockIdx.x << 3) + (threadIdx.x >> 5)) & (kLogSlots - 1);  // by warp
    int* c = ulog_n + slot * kLogStride;
    const int i = atomicAdd(c, 1);
    if (i < ulog_cap) ulog[(long long)slot * ulog_cap + i] = a;
    else c[1] = 1;
  }
  __device__ __forceinline__ int twin_cf(int, int a) const {
    a = (int)chk(bd, a, bd.na);
    int r = (int)chk(bd, __ldg(&arx[a].x), bd.na);
    return __ldcg(&arc[r].y);
  }
  // address of the twin's residual (one load here, none for RCSR forward)
  __device__ __forceinline__ const int* twin_ptr(int, int a) const {
    a = (int)chk(bd, a, bd.na);
    return &arc[chk(bd, __ldg(&arx[a].x), bd.na)].y;
  }
  // forward arc a of a row (segment 0): its residual word, its twin's, and
  // its capacity (greedy routing)
  __device__ __forceinline__ int* resid(int a) const { return &arc[chk(bd, a, bd.na)].y; }
  __device__ __forceinline__ int* twin_resid(int a) const {
    return &arc[chk(bd, __ldg(&arx[chk(bd, a, bd.na)].x), bd.na)].y;
  }
  __device__ __forceinline__ int cap_of(int a) const { return __ldg(&arx[chk(bd, a, bd.na)].y); }
};

struct TopoR {  // RCSR: forward {dst, cf_f} + cf_b, reverse {tail, forward id}
  const int* frow;
  int2* farc;
  int* fcb;
  const int* rrow;
  const int2* rarc;
  Bounds bd;  // na = m (forward arcs and reverse entries alike)
  static constexpr int kSeg = 2;
  __device__ __forceinline__ void seg(int u, int k, int& b, int& e) const {
    u = (int)chk(bd, u, bd.n);
    const int* r = k == 0 ? frow : rrow;
    b = __ldg(r + u);
    e = __ldg(r + u + 1);
  }
  __device__ __forceinline__ int deg(int u) const {
    u = (int)chk(bd, u, bd.n);
    return __ldg(frow + u + 1) - __ldg(frow + u) + __ldg(rrow + u + 1) - __ldg(rrow + u);
  }
  __device__ __forceinline__ void load(int k, int a, int& dst, int& cf) const {
    a = (int)chk(bd, a, bd.na);
    if (k == 0) {
      int2 r = __ldcg(farc + a);
      dst = (int)chk(bd, r.x, bd.n);
      cf = r.y;
    } else {
      int2 r = __ldg(rarc + a);
      dst = (int)chk(bd, r.x, bd.n);
      cf = __ldcg(fcb + chk(bd, r.y, bd.na));
    }
  }
  __device__ __forceinline__ int head(int k, int a) const {
    a = (int)chk(bd, a, bd.na);
    return (int)chk(bd, k == 0 ? __ldcg(&farc[a].x) : __ldg(&rarc[a].x), bd.n);
  }
  __device__ __forceinline__ void push(int k, int a, int cf, int p) const {
    a = (int)chk(bd, a, bd.na);
    if (k == 0) {
      farc[a].y = cf - p;
      fcb[a] = __ldcg(fcb + a) + p;
    } else {
      int fi = (int)chk(bd, __ldg(&rarc[a].y), bd.na);
      fcb[fi] = cf - p;
      farc[fi].y = __ldcg(&farc[fi].y) + p;
    }
  }
  __device__ __forceinline__ int twin_cf(int k, int a) const {
    a = (int)chk(bd, a, bd.na);
    if (k == 0) return __ldcg(fcb + a);
    int fi = (int)chk(bd, __ldg(&rarc[a].y), bd.na);
    return __ldcg(&farc[fi].y);
  }
  __device__ __forceinline__ const int* twin_ptr(int k, int a) const {
    a = (int)chk(bd, a, bd.na);
    return k == 0 ? fcb + a : &farc[chk(bd, __ldg(&rarc[a].y), bd.na)].y;
  }
  __device__ __forceinline__ void log_push(int) const {}
  __device__ __forceinline__ int* resid(int a) const { return &farc[chk(bd, a, bd.na)].y; }
  __device__ __forceinline__ int* twin_resid(int a) const { return fcb + chk(bd, a, bd.na); }
  // residual + flow: the capacity (no capacity array on the device side)
  __device__ __forceinline__ int cap_of(int a) const {
    a = (int)chk(bd, a, bd.na);
    return __ldcg(&farc[a].y) + __ldcg(fcb + a);
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
  int* hq[2];      // heavy active vertices (rows longer than heavy_deg)
  int* esnap;      // excess of each active vertex when it was filed for the round
  int* dmin0;      // deep entry -> min label over the first part's remaining residual arcs
  int4* hrec;      // chunk item -> 3 x int4: {u, first item, E, E left}, {label, items, entry, 0},
                   //   the vertex's row {b0, d0, b1, deg}: all a block needs, in one load
  int* hsum;       // chunk item -> admissible residual (saturated)
  int* hmin;       // chunk item -> min label over other residual arcs
  int* qraw;
  int* fr[3];
  int2* frh[3];    // long frontier rows as chunk items {vertex, chunk index}
  const int* cls;  // vertex ids: [0, n_light) light, then medium, then heavy
  int n_light;
  int n_medium;
  int n_heavy;
  const int4* bch; // static 2048-arc chunks {v, segment, begin, end} of heavy rows
  int n_bch;
  Ctl* ctl;
  Stats* st;
  long long total_deg;
  unsigned long long gr_threshold;
  int gr_rounds;  // global relabel at the latest after this many rounds
  int gr_stall;   // also after this many rounds in a row that moved no flow into t (0: off)
  int greedy;     // fresh one-sink BCSR solves: route along x->t and x->y->t before the first round
  int bfs_alpha = kBfsAlpha;  // the BFS goes bottom-up when frontier arcs * this > unvisited arcs
  int gr_plateau = 0;         // also relabel globally when the active set shrank by less than 10% over
                              // this many rounds (1..kMaxPlateau; 0: off)
  long long max_rounds;
  unsigned long long budget_ns;
  unsigned long long bar_timeout_ns;
  int heavy_deg;
  int mode;
  int bfs_dir;   // 0: vertices that reach the root (to sink); 1: reached from the root
  int bfs_root;
  int bfs_excl;  // vertex the BFS never labels (the source during a solve), or -1
  // Terminal sets (nullptr: the single pair s, t above).  term[v] is 1 for a
  // source, 2 for a sink; the preflow saturates every source's arcs, every
  // sink absorbs excess and roots the global relabel.
  const signed char* term = nullptr;
  const int* sources = nullptr;
  int n_sources = 0;
  const int* sinks = nullptr;
  int n_sinks = 0;
  long long* trace;  // optional event records {kind | aux << 32, t_ns, v0, v1, max, min}
  unsigned long long* bt;  // per-block work time of the current phase (trace only)
  unsigned long long* bt2; // per-block time of the heavy part of the push phase (trace only)
  int trace_cap;
};

template <class Topo>
__device__ __forceinline__ bool is_sink(const Params<Topo>& p, int v) {
  return p.term ? p.term[v] == 2 : v == p.t;
}
template <class Topo>
__device__ __forceinline__ bool is_terminal(const Params<Topo>& p, int v) {
  return p.term ? p.term[v] != 0 : (v == p.s || v == p.t);
}
// vertices the BFS never labels: the excluded vertex, and every source
template <class Topo>
__device__ __forceinline__ bool bfs_skip(const Params<Topo>& p, int v) {
  return v == p.bfs_excl || (p.term && p.term[v] == 1);
}

// Optional event trace (written by global thread 0 only; count in Stats).
enum TraceKind : int {
  kTrLevel = 1, kTrRound = 2, kTrPassA = 3, kTrPassB = 4, kTrRelabel = 5, kTrGrEnd = 6, kTrSplit = 7,
  kTrBuSplit = 8, kTrGreedy = 9
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
  unsigned long long wmark;  // scanned + visits + relabels at the last work flush
  unsigned long long deep;   // arcs scanned by the deep passes (also in `scanned`)
  int sink;
  int pad;
};

// ---------------------------------------------------------------------------
// Bounded grid barrier on one word.  Block 0 adds 2^31 - (blocks - 1), every other
// block adds 1: the arrivals of one episode sum to exactly 2^31, so bit 31
// flips when -- and only when -- the last block arrives, and the low 31 bits
// stay zero between episodes (the word is zero at launch).  A block waits for
// bit 31 to differ from the value its own arrival returned; a block that
// races ahead into the next episode cannot flip it back before the slowest
// block has left this one.  The wait gives up after timeout_ns.
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned atom_add_release(unsigned* p, unsigned x) {
  unsigned old;
  asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(x) : "memory");
  return old;
}
// The block's writes are ordered before thread 0's arrival by the block
// barrier and the release of the arrival; the acquire load that sees bit 31
// flip (or, for the last arrival, the count complete) orders the block's
// later reads after every other block's arrival.  Measured on GB300: 2.1 us
// per barrier at 456 blocks, against 2.4 us with full fences around a
// relaxed atomic.
// C is any control block with an `unsigned bar` word and an `int err` word.
template <class C>
__device__ __forceinline__ bool grid_sync(C* c, unsigned long long timeout_ns) {
  // Thread 0 reads the error word once and the block takes its answer: a
  // word another block may set at any moment (a timed-out wait) must not send
  // the threads of one block different ways.
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    if (gridDim.x > 1) {  // a one-block grid: the block barriers are enough
      const unsigned add = blockIdx.x == 0 ? 0x80000000u - (gridDim.x - 1u) : 1u;
      const unsigned old = atom_add_release(&c->bar, add);
      if (((old + add) ^ old) & 0x80000000u) {
        ld_acquire(&c->bar);  // last arrival
      } else {
        // A wait gives up after timeout_ns and at least timeout_ns / 1024
        // polls (each takes well over a nanosecond): a forward step of the
        // timer alone cannot end a wait early.
        const unsigned long long t0 = gtime(), min_polls = timeout_ns >> 10;
        unsigned long long polls = 0;
        while (!((ld_acquire(&c->bar) ^ old) & 0x80000000u)) {
          if (++polls > min_polls && time_past(t0, timeout_ns)) {
            atomicCAS(&c->err, 0, (int)WBPR_ERR_TIMEOUT);
            break;
          }
        }
      }
    }
    s_ok = ldv(&c->err) == 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Warp-aggregated append of v to q[*cnt] (one atomic per converged group).
__device__ __forceinline__ void append(int* q, int* cnt, int v) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(cnt, (int)g.size());
  base = g.shfl(base, 0);
  q[base + g.thread_rank()] = v;
}

// Per-round work (arcs scanned + vertex visits + relabels) of this block since
// its last flush, added to one of the 32 slots of the round's parity.
__device__ __forceinline__ void flush_work(BlockAcc& a, Ctl* c, int parity) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long tot = a.scanned + a.visits + a.relabels;
    const unsigned long long w = tot - a.wmark;
    a.wmark = tot;
    if (w) atomicAdd(&c->work[parity][(blockIdx.x % kWorkSlots) * 16], w);
  }
  __syncthreads();
}
// Sum of the 32 work slots of one parity (every warp computes it).
__device__ __forceinline__ unsigned long long work_total(Ctl* c, int parity) {
  unsigned long long w = *(volatile unsigned long long*)&c->work[parity][(threadIdx.x & 31) * 16];
  for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  return w;
}

// Counters into Stats, once per launch.
__device__ __forceinline__ void flush_acc(BlockAcc& a, Stats* st) {
  __syncthreads();
  if (threadIdx.x == 0) {
    if (a.scanned) atomicAdd(&st->arcs_scanned, a.scanned);
    if (a.pushes) atomicAdd(&st->pushes, a.pushes);
    if (a.relabels) atomicAdd(&st->relabels, a.relabels);
    if (a.visits) atomicAdd(&st->vertex_visits, a.visits);
    if (a.bfs_arcs) atomicAdd(&st->bfs_arcs, a.bfs_arcs);
    if (a.bfs_vertices) atomicAdd(&st->bfs_vertices, a.bfs_vertices);
    if (a.deep) atomicAdd(&st->deep_scanned, a.deep);
    a.scanned = a.pushes = a.relabels = a.visits = a.bfs_arcs = a.bfs_vertices = a.wmark = a.deep = 0;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
struct VRow {  // a row as one virtual range [0, deg): segment 0 then segment 1
  int b0, d0, b1, deg;
};

template <class Topo>
__device__ __forceinline__ VRow vrow(const Topo& g, int u) {
  VRow r;
  int e0, b1 = 0, e1 = 0;
  g.seg(u, 0, r.b0, e0);
  if (Topo::kSeg > 1) g.seg(u, 1, b1, e1);
  r.d0 = e0 - r.b0;
  r.b1 = b1;
  r.deg = r.d0 + (e1 - b1);
  return r;
}
__device__ __forceinline__ void vidx(const VRow& r, int vi, int& k, int& a) {
  if (vi < r.d0) {
    k = 0;
    a = r.b0 + vi;
  } else {
    k = 1;
    a = r.b1 + (vi - r.d0);
  }
}

// Long rows are walked by one warp over their first kFirst arcs; a vertex
// that still has excess after them becomes a deep entry, and the rest of its
// row is cut into kPart-arc parts that warps of the whole grid process in two
// passes (deep passes A and B below).
#ifndef WBPR_FIRST_ARCS
#define WBPR_FIRST_ARCS 2048
#endif
constexpr int kFirst = WBPR_FIRST_ARCS;  // arcs of a long row walked by one warp before it goes deep
constexpr int kPart = 256;               // arcs of a deep part: one warp, 8 arcs a lane in flight

template <class Topo>
__device__ __forceinline__ void make_deep(const Params<Topo>& p, int u, int E, int erem, int mn, int from, int hu,
                                          const VRow& r, int lane, int nl);

// The ordered walk of a tile of W lanes (W = 1: one thread) with Q arcs per
// lane in flight over the virtual arcs [lo, hi) of row r: pushes at most erem
// units along admissible arcs (label = th + 1 ... th = label(u) - 1) in arc
// order, apportioned by a saturating prefix sum across the tile, with early
// exit once erem is placed.  minh gets the minimum label over the arcs left
// residual; npush and scanned count for the caller.
template <class Topo, int W, int Q>
__device__ __forceinline__ void tile_walk(const Params<Topo>& p, const VRow& r, int lo, int hi, int th, unsigned mask,
                                          int lane, unsigned& erem, int& minh, int& npush,
                                          unsigned long long& scanned, int* rawcnt, BlockAcc& acc) {
#pragma unroll 1
  for (int base = lo; base < hi; base += W * Q) {
    int dst[Q], cf[Q], hv[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const int vi = base + q * W + lane;
      dst[q] = 0;
      cf[q] = 0;
      if (vi < hi) {
        int kk, aa;
        vidx(r, vi, kk, aa);
        p.g.load(kk, aa, dst[q], cf[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) hv[q] = cf[q] > 0 ? __ldcg(p.lab + dst[q]) : kBig;
    if (lane == 0) scanned += (unsigned long long)min(W * Q, hi - base);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const bool adm = (cf[q] > 0) && (hv[q] == th);
      const unsigned am = (W == 1) ? (unsigned)adm : __ballot_sync(mask, adm);
      int pushed = 0;
      if (am && erem > 0) {
        unsigned incl = adm ? (unsigned)cf[q] : 0u;
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
          int kk, aa;
          vidx(r, base + q * W + lane, kk, aa);
          p.g.push(kk, aa, cf[q], pushed);
          ++npush;
          if (dst[q] == p.t) {
            atomicAdd(&acc.sink, pushed);
          } else if (p.term && p.term[dst[q]] == 2) {
            atomicAdd(p.e + dst[q], pushed);  // one of several sinks: never filed
          } else {
            int old = atomicAdd(p.e + dst[q], pushed);
            if (old == 0) append(p.qraw, rawcnt, dst[q]);
          }
        }
      }
      if (cf[q] - pushed > 0 && hv[q] < minh) minh = hv[q];
    }
    if (erem == 0) break;
  }
}

// Push phase for one vertex: a tile walks its row from the start with early
// exit, over at most `limit` arcs; a longer row that keeps excess becomes a
// deep entry, anything else settles here.
template <class Topo, int W, int Q>
__device__ __forceinline__ void tile_discharge(const Params<Topo>& p, int u, int limit, int* rawcnt,
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
  const VRow r = vrow(p.g, u);
  const int hi = min(r.deg, limit);
  unsigned erem = (unsigned)eu;
  int minh = kBig;
  int npush = 0;
  unsigned long long scanned = 0;
  tile_walk<Topo, W, Q>(p, r, 0, hi, hu - 1, mask, lane, erem, minh, npush, scanned, rawcnt, acc);
  if (W > 1) minh = __reduce_min_sync(mask, minh);
  if (npush) atomicAdd(&acc.pushes, (unsigned long long)npush);
  if (lane == 0) atomicAdd(&acc.scanned, scanned);
  if (erem > 0 && r.deg > hi) {  // uniform over the tile
    make_deep(p, u, eu, (int)erem, minh, hi, hu, r, lane, W);
    return;
  }
  if (lane == 0) {
    const int D = eu - (int)erem;
    bool self = true;
    if (D > 0) self = (atomicSub(p.e + u, D) - D) > 0;
    if (erem > 0) {
      // Pushes into u during this phase open arcs u->w with label(w) =
      // label(u) + 1 that the scan may not have seen; the relabel phase
      // detects them by comparing excess with (filing snapshot - pushed).
      p.rl_min[u] = minh;
      p.rl_left[u] = __ldcg(p.esnap + u) - D;
    }
    if (self) append(p.qraw, rawcnt, u);
    atomicAdd(&acc.visits, 1ull);
  }
}

// ---------------------------------------------------------------------------
// Deep entries: the part of a long row beyond its first kFirst arcs, cut into
// kPart-arc parts, each processed by one warp in two passes of the push phase:
//   pass A  every part sums the residual capacity of its admissible arcs
//           (saturated at the vertex's excess left) and takes the minimum
//           label over its other residual arcs;
//   -- grid barrier --
//   pass B  part j of u receives allot = min(sum_j, E left - sum of earlier
//           parts) and pushes it along its admissible arcs in arc order; the
//           last part settles excess(u) and the relabel record.
// Total pushed = min(E left, sum of all parts), in arc order: the same pushes
// a single tile walking the whole row would make.  Labels are frozen across
// both passes, and admissible residuals of u change only by u's own pushes,
// so the two passes see the same admissible set.  Warps need no block
// barrier, and every part is the same size, so parts are dealt to warps
// statically (part k to warp k mod warps) without a claim counter.
//
// Part record (3 x int4, 48 bytes: all a warp needs, in one load):
//   {u, first part of the entry, E (excess at filing), E left after the first
//    kFirst arcs}, {label, parts, entry, first arc of part 0}, the row
//   {b0, d0, b1, deg}.

// Settle a vertex: subtract what it pushed, re-file it when it still has
// excess, record the relabel candidate when some of its own excess was left.
template <class Topo>
__device__ __forceinline__ void settle(const Params<Topo>& p, int u, int E, int erem, int mn, int* rawcnt,
                                       BlockAcc& acc) {
  const int D = E - erem;
  bool self = true;
  if (D > 0) self = (atomicSub(p.e + u, D) - D) > 0;
  if (erem > 0) {
    p.rl_min[u] = mn;
    p.rl_left[u] = __ldcg(p.esnap + u) - D;
  }
  if (self) append(p.qraw, rawcnt, u);
  atomicAdd(&acc.visits, 1ull);
  atomicAdd(&p.st->heavy_visits, 1ull);
}

// File the deep entry of u: the nl lanes of the tile that walked its first
// `from` arcs write the part records together.
template <class Topo>
__device__ __forceinline__ void make_deep(const Params<Topo>& p, int u, int E, int erem, int mn, int from, int hu,
                                          const VRow& r, int lane, int nl) {
  const int np = (r.deg - from + kPart - 1) / kPart;
  unsigned long long old = 0;
  if (lane == 0) old = atomicAdd(&p.ctl->dpack, (1ull << 32) | (unsigned long long)np);
  if (nl > 1) {
    const unsigned mask = nl == 32 ? 0xffffffffu : (((1u << nl) - 1u) << ((threadIdx.x & 31u) & ~(unsigned)(nl - 1)));
    old = __shfl_sync(mask, old, 0, nl);
  }
  const int di = (int)(old >> 32), base = (int)(old & 0xffffffffu);
  if (lane == 0) p.dmin0[di] = mn;
  const int4 a = make_int4(u, base, E, erem), b = make_int4(hu, np, di, from),
             rr = make_int4(r.b0, r.d0, r.b1, r.deg);
  for (int j = lane; j < np; j += nl) {
    int4* q = p.hrec + 3LL * (base + j);
    q[0] = a;
    q[1] = b;
    q[2] = rr;
  }
}

struct DeepPart {
  int u, first, E, Er, hu, np, di, lo, hi, j;
  VRow r;
};

__device__ __forceinline__ DeepPart deep_part(const int4* hrec, int k) {
  const int4* q = hrec + 3LL * k;
  const int4 a = __ldcg(q), b = __ldcg(q + 1), rr = __ldcg(q + 2);
  DeepPart d;
  d.u = a.x;
  d.first = a.y;
  d.E = a.z;
  d.Er = a.w;
  d.hu = b.x;
  d.np = b.y;
  d.di = b.z;
  d.j = k - a.y;
  d.r.b0 = rr.x;
  d.r.d0 = rr.y;
  d.r.b1 = rr.z;
  d.r.deg = rr.w;
  d.lo = b.w + d.j * kPart;
  d.hi = min(d.r.deg, d.lo + kPart);
  return d;
}

// Pass A of part k (all 32 lanes of a warp).
template <class Topo>
__device__ void deep_part_a(const Params<Topo>& p, int k, BlockAcc& acc) {
  const int lane = threadIdx.x & 31;
  const DeepPart d = deep_part(p.hrec, k);
  const int th = d.hu - 1;
  constexpr int kIt = kPart / 32;
  int dst[kIt], cf[kIt];
#pragma unroll
  for (int it = 0; it < kIt; ++it) {
    const int vi = d.lo + it * 32 + lane;
    dst[it] = 0;
    cf[it] = 0;
    if (vi < d.hi) {
      int kk, a;
      vidx(d.r, vi, kk, a);
      p.g.load(kk, a, dst[it], cf[it]);
    }
  }
  unsigned long long sum = 0;
  int mn = kBig;
#pragma unroll
  for (int it = 0; it < kIt; ++it) {
    if (cf[it] > 0) {
      const int hv = __ldcg(p.lab + dst[it]);
      if (hv == th) sum += (unsigned)cf[it];
      else if (hv < mn) mn = hv;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  mn = __reduce_min_sync(0xffffffffu, mn);
  if (lane == 0) {
    p.hsum[k] = (int)(sum > (unsigned long long)d.Er ? (unsigned long long)d.Er : sum);
    p.hmin[k] = mn;
    atomicAdd(&acc.scanned, (unsigned long long)(d.hi - d.lo));
    atomicAdd(&acc.deep, (unsigned long long)(d.hi - d.lo));
  }
}

// Pass B of part k (all 32 lanes of a warp): the sums of the earlier parts
// and, for the last part, the minima of all parts are read by the lanes in
// parallel.
template <class Topo>
__device__ void deep_part_b(const Params<Topo>& p, int k, int* rawcnt, BlockAcc& acc) {
  const int lane = threadIdx.x & 31;
  const DeepPart d = deep_part(p.hrec, k);
  long long prev = 0;
  for (int i = d.first + lane; i < k; i += 32) prev += __ldcg(p.hsum + i);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) prev += __shfl_xor_sync(0xffffffffu, prev, o);
  const int S = __ldcg(p.hsum + k);
  unsigned allot = prev >= d.Er ? 0u : (unsigned)min((long long)S, (long long)d.Er - prev);
  if (allot > 0) {
    int minh = kBig, npush = 0;
    unsigned long long scanned = 0;
    tile_walk<Topo, 32, 4>(p, d.r, d.lo, d.hi, d.hu - 1, 0xffffffffu, lane, allot, minh, npush, scanned, rawcnt,
                           acc);
    if (npush) atomicAdd(&acc.pushes, (unsigned long long)npush);
    if (lane == 0) {
      atomicAdd(&acc.scanned, scanned);
      atomicAdd(&acc.deep, scanned);
    }
  }
  if (d.j == d.np - 1) {
    int mn = kBig;
    for (int i = d.first + lane; i < d.first + d.np; i += 32) mn = min(mn, __ldcg(p.hmin + i));
    mn = __reduce_min_sync(0xffffffffu, mn);
    if (lane == 0) {
      const long long all = prev + S;
      const int erest = d.Er - (int)min((long long)d.Er, all);
      settle(p, d.u, d.E, erest, min(mn, __ldcg(p.dmin0 + d.di)), rawcnt, acc);
    }
  }
}

// Push phase, stage 1: rows longer than heavy_deg by a warp each (128 arcs in
// flight), shorter rows by W-lane tiles; both with early exit.
template <class Topo, int W>
__device__ void push_first(const Params<Topo>& p, int cur, int raw, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int nL = ldv(&c->lcount[cur]);
  const int nH = ldv(&c->hcount[cur]);
  int* rawcnt = &c->qraw_count[raw];
  const int lane = threadIdx.x & 31;
  // first item of every warp by its index, the rest claimed (an idle round
  // touches no counter)
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int idx = gw; idx < nH;) {
    tile_discharge<Topo, 32, 4>(p, __ldcg(p.hq[cur] + idx), kFirst, rawcnt, acc);
    int nx = 0;
    if (lane == 0) nx = nwarps + atomicAdd(&c->heavy_next, 1);
    idx = __shfl_sync(0xffffffffu, nx, 0);
  }
  if (p.trace && threadIdx.x == 0) p.bt2[blockIdx.x] = gtime();
  constexpr int kTpw = 32 / W;
  constexpr int kGrab = 2 * kTpw;
  for (int base = gw * kGrab; base < nL;) {
#pragma unroll 1
    for (int r = 0; r < 2; ++r) {
      const int idx = base + r * kTpw + lane / W;
      if (idx < nL) tile_discharge<Topo, W, 4>(p, __ldcg(p.lq[cur] + idx), kFirst, rawcnt, acc);
    }
    __syncwarp();
    int nx = 0;
    if (lane == 0) nx = nwarps * kGrab + atomicAdd(&c->light_next, kGrab);
    base = __shfl_sync(0xffffffffu, nx, 0);
  }
}

// Deep pass A or B over the round's nD parts: part k to warp k mod warps.
template <class Topo>
__device__ void push_deep(const Params<Topo>& p, int pass, int nD, int raw, BlockAcc& acc) {
  int* rawcnt = &p.ctl->qraw_count[raw];
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int k = gw; k < nD; k += nwarps) {
    if (pass == 0) deep_part_a<Topo>(p, k, acc);
    else deep_part_b<Topo>(p, k, rawcnt, acc);
  }
}

__device__ __forceinline__ void flush_sink(int* et, BlockAcc& acc) {
  __syncthreads();
  if (threadIdx.x == 0 && acc.sink) {
    atomicAdd(et, acc.sink);
    acc.sink = 0;
  }
}

// Warp-aggregated append: all 32 lanes call it; lanes with `pred` append v.
// One atomic per warp instead of one per element (a single frontier or queue
// counter otherwise serialises hundreds of thousands of atomics).
__device__ __forceinline__ void warp_append(int* q, int* cnt, int v, bool pred) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(cnt, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) q[base + __popc(m & ((1u << lane) - 1u))] = v;
}

// Warp-level filing of active vertices (all 32 lanes call it).
template <class Topo>
__device__ __forceinline__ void warp_file(const Params<Topo>& p, int nxt, int u, int eu, bool pred,
                                         int dpre = -1) {
  Ctl* c = p.ctl;
  bool light = false;
  if (pred) {
    p.esnap[u] = eu;
    light = (dpre >= 0 ? dpre : p.g.deg(u)) <= p.heavy_deg;
  }
  warp_append(p.lq[nxt], &c->lcount[nxt], u, pred && light);
  warp_append(p.hq[nxt], &c->hcount[nxt], u, pred && !light);
}

// Relabel phase over the raw next queue; also files the survivors into the
// light / heavy lists of the next round.
template <class Topo>
__device__ void relabel_phase(const Params<Topo>& p, int cur, int nxt, int raw, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int nq = ldv(&c->qraw_count[raw]);
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  unsigned long long rl = 0;
  for (int base = gt - lane; base < nq; base += gs) {
    const int i = base + lane;
    int u = -1, eu = 0, hu = p.n, du = 0;
    if (i < nq) {
      u = __ldcg(p.qraw + i);
      // every load that depends only on u in one step
      int m = __ldcg(p.rl_min + u);
      hu = __ldcg(p.lab + u);
      eu = ldv(p.e + u);
      const int left = __ldcg(p.rl_left + u);
      du = p.g.deg(u);
      if (m != kNone) {
        p.rl_min[u] = kNone;
        if (eu > left && hu + 1 < m) m = hu + 1;
        int nh = (m >= p.n - 1) ? p.n : m + 1;
        if (nh <= hu) nh = hu + 1;
        if (nh > p.n) nh = p.n;
        p.lab[u] = nh;
        hu = nh;
        ++rl;
      }
    }
    warp_file(p, nxt, u, eu, u >= 0 && eu > 0 && hu < p.n, du);
  }
  if (rl) atomicAdd(&acc.relabels, rl);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    c->lcount[cur] = 0;
    c->hcount[cur] = 0;
    c->dpack = 0;
    c->qraw_count[raw ^ 1] = 0;
    c->light_next = 0;
    c->heavy_next = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x < kWorkSlots) c->work[raw ^ 1][threadIdx.x * 16] = 0;
}

// ---------------------------------------------------------------------------
// Global relabel: level-synchronous BFS over residual arcs from `root`.
// DIR 0 labels every vertex with its residual distance TO the root (the
// reference's backward BFS from the sink); DIR 1 with its distance FROM the
// root.  Unreached vertices keep label n.  Top-down expands a frontier list
// (warp per short row; long rows as 1024-arc chunk items shared by all warps;
// warp-aggregated appends).  Bottom-up lets every unvisited vertex look for a
// neighbour labelled `level` (thread / warp / block per row by length class)
// and keeps no list: it only counts the vertices it labels and their arcs
// (one atomic per block); if the next level goes top-down, its frontier is
// materialised by a scan of the labels.
constexpr int kTdHeavy = 256;
constexpr int kTdChunk = 1024;

// Frontier entry of a vertex found top-down or by a label scan: short rows
// into fr, long rows as chunk items into frh.  All lanes call it.
template <class Topo>
__device__ __forceinline__ void warp_frontier(const Params<Topo>& p, int* fcnt, int* fhcnt, int fn, int v,
                                              bool pred, BlockAcc& acc, int dpre = -1) {
  int d = 0;
  if (pred) d = dpre >= 0 ? dpre : p.g.deg(v);
  const bool lng = pred && d > kTdHeavy;
  warp_append(p.fr[fn], fcnt, v, pred && !lng);
  if (lng) {
    const int nch = (d + kTdChunk - 1) / kTdChunk;
    const int base = atomicAdd(fhcnt, nch);
    for (int j = 0; j < nch; ++j) p.frh[fn][base + j] = make_int2(v, j);
  }
  unsigned long long sd = (unsigned long long)d;
  for (int o = 16; o > 0; o >>= 1) sd += __shfl_down_sync(0xffffffffu, sd, o);
  if ((threadIdx.x & 31) == 0 && sd) atomicAdd((unsigned long long*)&acc.fdeg, sd);
}

// warp_frontier for four candidates per lane (v[q] with pred[q], degree
// d[q]): one counter atomic per warp for all short rows, one degree sum.
template <class Topo>
__device__ __forceinline__ void warp_frontier4(const Params<Topo>& p, int* fcnt, int* fhcnt, int fn,
                                               const int* v, const bool* pred, const int* d, BlockAcc& acc) {
  const int lane = threadIdx.x & 31;
  int nshort = 0;
  unsigned long long sd = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (!pred[q]) continue;
    sd += (unsigned long long)d[q];
    if (d[q] <= kTdHeavy) {
      ++nshort;
    } else {
      const int nch = (d[q] + kTdChunk - 1) / kTdChunk;
      const int base = atomicAdd(fhcnt, nch);
      for (int j = 0; j < nch; ++j) p.frh[fn][base + j] = make_int2(v[q], j);
    }
  }
  int incl = nshort;  // inclusive scan of the short-row counts over the warp
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (total) {
    int base = 0;
    if (lane == 31) base = atomicAdd(fcnt, total);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - nshort;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (pred[q] && d[q] <= kTdHeavy) p.fr[fn][base++] = v[q];
  }
  for (int o = 16; o > 0; o >>= 1) sd += __shfl_down_sync(0xffffffffu, sd, o);
  if (lane == 0 && sd) atomicAdd((unsigned long long*)&acc.fdeg, sd);
}

// Top-down step over arcs [base, base + 128) of virtual row r (4 arcs per
// lane in flight); all 32 lanes call it.
template <class Topo, int DIR>
__device__ __forceinline__ void td_batch(const Params<Topo>& p, const VRow& r, int base, int vend, int level,
                                         int fn, BlockAcc& acc, unsigned long long& arcs) {
  const int lane = threadIdx.x & 31;
  int dst[4], cf[4], dg[4];
  const int* tp[4];
  bool ok[4];
  // step 1: heads (and residuals or twin addresses) of 4 arcs per lane
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int vi = base + q * 32 + lane;
    ok[q] = vi < vend;
    dst[q] = 0;
    cf[q] = 1;
    tp[q] = nullptr;
    if (ok[q]) {
      int kk, aa;
      vidx(r, vi, kk, aa);
      if (DIR == 0) {
        dst[q] = p.g.head(kk, aa);
        tp[q] = p.g.twin_ptr(kk, aa);
      } else {
        p.g.load(kk, aa, dst[q], cf[q]);
      }
      ++arcs;
    }
  }
  // step 2: label of the head, the residual towards this row, the head's
  // degree (for the next frontier), all independent of each other
  int lv[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    lv[q] = 0;
    dg[q] = 0;
    if (ok[q]) {
      lv[q] = __ldcg(p.lab + dst[q]);
      if (DIR == 0) cf[q] = __ldcg(tp[q]);
      dg[q] = p.g.deg(dst[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) ok[q] = ok[q] && cf[q] > 0 && lv[q] == p.n && !bfs_skip(p, dst[q]);
  // step 3: claim, the four CAS of a lane in flight together
  bool won[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) won[q] = ok[q] && atomicCAS(p.lab + dst[q], p.n, level + 1) == p.n;
  warp_frontier4(p, &p.ctl->fcount[fn], &p.ctl->fhcount[fn], fn, dst, won, dg, acc);
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
__device__ void bfs_top_down(const Params<Topo>& p, int level, int nf, int nfh, int fc, int fn,
                             BlockAcc& acc) {
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long arcs = 0;
  // chunk items of long rows: a warp per 1024-arc chunk, or per part of one
  // when the level has few of them (the sink's own row at level 0: a warp
  // walking 1024 arcs is 8 dependent steps; 8 parts of 128 arcs take one)
  int S = 1;
  while (S < 8 && 2LL * nfh * S <= nwarps) S <<= 1;
  const int part = kTdChunk / S;
  for (int i = gw; i < nfh * S; i += nwarps) {
    const int2 it = __ldcg(p.frh[fc] + i / S);
    const VRow r = vrow(p.g, it.x);
    const int lo = it.y * kTdChunk + (i % S) * part, hi = min(r.deg, lo + part);
    for (int b = lo; b < hi; b += 128) td_batch<Topo, DIR>(p, r, b, hi, level, fn, acc, arcs);
  }
  // short rows (<= kTdHeavy arcs): a warp per row
  for (int i = gw; i < nf; i += nwarps) {
    const int x = __ldcg(p.fr[fc] + i);
    const VRow r = vrow(p.g, x);
    for (int b = 0; b < r.deg; b += 128) td_batch<Topo, DIR>(p, r, b, r.deg, level, fn, acc, arcs);
  }
  if (arcs) atomicAdd(&acc.bfs_arcs, arcs);
}

// Materialise the frontier (vertices labelled `level`) after a bottom-up
// level, into fr[fc] / frh[fc] with the counters mcount / mhcount.
template <class Topo>
__device__ void bfs_materialise(const Params<Topo>& p, int level, int fc, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int nall = p.n_light + p.n_medium + p.n_heavy;
  // 4 entries per lane in flight: the scan is latency-bound, few entries hit
  for (long long base = 4LL * (gt - lane); base < nall; base += 4LL * gs) {
    int v[4];
    bool in[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long i = base + q * 32 + lane;
      v[q] = i < nall ? __ldg(p.cls + i) : -1;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) in[q] = v[q] >= 0 && __ldcg(p.lab + v[q]) == level;
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (__any_sync(0xffffffffu, in[q])) warp_frontier(p, &c->mcount, &c->mhcount, fc, v[q], in[q], acc);
  }
}

template <class Topo, int DIR>
__device__ void bfs_bottom_up(const Params<Topo>& p, int level, BlockAcc& acc) {
  Ctl* c = p.ctl;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int gw = gt >> 5, nwarps = gs >> 5;
  unsigned long long arcs = 0, verts = 0, found = 0, fdeg = 0;
  // short rows (<= kLightDeg): a thread each; kBuRows rows advance together,
  // kBuArcs arcs of each in flight per step
#ifndef WBPR_BU_ROWS
#define WBPR_BU_ROWS 4
#endif
  constexpr int kBuRows = WBPR_BU_ROWS, kBuArcs = 4;
  for (int i0 = gt; i0 < p.n_light; i0 += kBuRows * gs) {
    int xs[kBuRows];
    bool todo[kBuRows];
    VRow rr[kBuRows];
#pragma unroll
    for (int q = 0; q < kBuRows; ++q) {
      const int i = i0 + q * gs;
      xs[q] = i < p.n_light ? __ldg(p.cls + i) : -1;
    }
    bool any = false;
#pragma unroll
    for (int q = 0; q < kBuRows; ++q) {
      todo[q] = xs[q] >= 0 && !bfs_skip(p, xs[q]) && __ldcg(p.lab + xs[q]) == p.n;
      if (xs[q] >= 0) ++verts;
      any |= todo[q];
    }
#pragma unroll
    for (int q = 0; q < kBuRows; ++q) {
      rr[q].b0 = rr[q].d0 = rr[q].b1 = rr[q].deg = 0;
      if (todo[q]) rr[q] = vrow(p.g, xs[q]);
    }
#pragma unroll 1
    for (int v0 = 0; any; v0 += kBuArcs) {
      int dst[kBuRows][kBuArcs], cf[kBuRows][kBuArcs];
#pragma unroll
      for (int q = 0; q < kBuRows; ++q)
#pragma unroll
        for (int w = 0; w < kBuArcs; ++w) {
          cf[q][w] = 0;
          dst[q][w] = 0;
          if (todo[q] && v0 + w < rr[q].deg) {
            int kk, aa;
            vidx(rr[q], v0 + w, kk, aa);
            p.g.load(kk, aa, dst[q][w], cf[q][w]);
            if (DIR == 1) cf[q][w] = p.g.twin_cf(kk, aa);
            ++arcs;
          }
        }
      any = false;
#pragma unroll
      for (int q = 0; q < kBuRows; ++q) {
        bool hit = false;
#pragma unroll
        for (int w = 0; w < kBuArcs; ++w)
          if (cf[q][w] > 0 && __ldcg(p.lab + dst[q][w]) == level) hit = true;
        if (todo[q] && hit) {
          p.lab[xs[q]] = level + 1;
          ++found;
          fdeg += (unsigned long long)rr[q].deg;
        }
        if (hit || v0 + kBuArcs >= rr[q].deg) todo[q] = false;
        any |= todo[q];
      }
    }
  }
  if (p.trace && threadIdx.x == 0) p.bt2[blockIdx.x] = gtime();  // light rows done
  // medium rows: the warp checks a batch of rows' labels at once (32 rows, or
  // 8 when there are too few rows to give every warp several batches); 8-lane
  // tiles scan the open rows four at a time over their first kBuTile arcs
  // (where most hits are), and the whole warp finishes the rows that are
  // longer and have not hit yet
  {
    constexpr int kBuTile = 128;
    const int sub = lane >> 3, sl = lane & 7;
    const unsigned smask = 0xffu << (sub * 8);
    const int B = p.n_medium >= 64 * nwarps ? 32 : 8;
    // batches are claimed, not dealt: rows of one batch are neighbours in
    // vertex order, and R-MAT puts its longer rows together, so a static deal
    // left some warps many long unlabelled rows (the slowest block of the
    // level's medium part took 4x the fastest)
    int* next = &c->bu_med[level % 3];
    for (int base = gw * B;;) {
      if (base >= p.n_medium) break;
      const int i = base + lane;
      int x = -1;
      if (lane < B && i < p.n_medium) {
        x = __ldg(p.cls + p.n_light + i);
        ++verts;
      }
      const bool open = x >= 0 && !bfs_skip(p, x) && __ldcg(p.lab + x) == p.n;
      VRow r;
      r.b0 = r.d0 = r.b1 = r.deg = 0;
      if (open) r = vrow(p.g, x);
      unsigned todo = __ballot_sync(0xffffffffu, open);
      unsigned big = 0;
      while (todo) {
        // this tile's row: the (sub+1)-th open one; `rest` drops the first four
        unsigned rest = todo, pick = 32;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (j == sub && rest) pick = __ffs(rest) - 1;
          rest &= rest - 1u;
        }
        const int src = pick < 32 ? (int)pick : lane;
        const int xr = __shfl_sync(0xffffffffu, x, src);
        VRow q;
        q.b0 = __shfl_sync(0xffffffffu, r.b0, src);
        q.d0 = __shfl_sync(0xffffffffu, r.d0, src);
        q.b1 = __shfl_sync(0xffffffffu, r.b1, src);
        q.deg = __shfl_sync(0xffffffffu, r.deg, src);
        todo = rest;
        bool defer = false;
        if (pick < 32) {
          const int lim = min(q.deg, kBuTile);
          bool hit = false;
          for (int v0 = 0; v0 < lim && !hit; v0 += 32) {
            bool h = false;
#pragma unroll
            for (int w = 0; w < 4; ++w) {
              const int vi = v0 + w * 8 + sl;
              if (vi < lim) {
                int kk, aa;
                vidx(q, vi, kk, aa);
                ++arcs;
                h |= bu_arc<Topo, DIR>(p, kk, aa, level);
              }
            }
            hit = __any_sync(smask, h);
          }
          if (hit && sl == 0) {
            p.lab[xr] = level + 1;
            ++found;
            fdeg += (unsigned long long)q.deg;
          }
          defer = !hit && q.deg > kBuTile && sl == 0;
        }
        big |= __reduce_or_sync(0xffffffffu, defer ? (1u << pick) : 0u);
      }
      while (big) {
        const int src = __ffs(big) - 1;
        big &= big - 1u;
        const int xr = __shfl_sync(0xffffffffu, x, src);
        VRow q;
        q.b0 = __shfl_sync(0xffffffffu, r.b0, src);
        q.d0 = __shfl_sync(0xffffffffu, r.d0, src);
        q.b1 = __shfl_sync(0xffffffffu, r.b1, src);
        q.deg = __shfl_sync(0xffffffffu, r.deg, src);
        bool hit = false;
        for (int v0 = kBuTile; v0 < q.deg && !hit; v0 += 128) {
          bool h = false;
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            const int vi = v0 + w * 32 + lane;
            if (vi < q.deg) {
              int kk, aa;
              vidx(q, vi, kk, aa);
              ++arcs;
              h |= bu_arc<Topo, DIR>(p, kk, aa, level);
            }
          }
          hit = __any_sync(0xffffffffu, h);
        }
        if (hit && lane == 0) {
          p.lab[xr] = level + 1;
          ++found;
          fdeg += (unsigned long long)q.deg;
        }
      }
      // the first batch of every warp is its own, the rest are claimed
      int nb = 0;
      if (lane == 0) nb = nwarps * B + atomicAdd(next, B);
      base = __shfl_sync(0xffffffffu, nb, 0);
    }
  }
  if (p.trace) {
    __syncwarp();
    if (threadIdx.x == 0) p.bt2[gridDim.x + blockIdx.x] = gtime();  // medium rows done (warp 0's view)
  }
  // long rows: blocks over static 2048-arc chunks; first chunk to hit wins
  unsigned long long ha = 0;
  // chunk k of the list goes to block k % blocks; warp 0 checks 32 of the
  // block's chunks at once (their vertex still unlabelled), one block
  // barrier per 32 chunks, and only those chunks are scanned
  __shared__ unsigned s_live;
  for (int k0 = 0; (long long)blockIdx.x + (long long)k0 * gridDim.x < p.n_bch; k0 += 32) {
    if (threadIdx.x < 32) {
      const long long it = blockIdx.x + (long long)(k0 + (int)threadIdx.x) * gridDim.x;
      bool live = false;
      if (it < p.n_bch) {
        const int v = __ldg(&p.bch[it].x);
        live = !bfs_skip(p, v) && __ldcg(p.lab + v) == p.n;
      }
      const unsigned m = __ballot_sync(0xffffffffu, live);
      if (threadIdx.x == 0) s_live = m;
    }
    __syncthreads();
    unsigned live = s_live;
    __syncthreads();
    while (live) {
      const int j = __ffs(live) - 1;
      live &= live - 1;
      const int4 ch = __ldg(p.bch + blockIdx.x + (long long)(k0 + j) * gridDim.x);  // {vertex, segment, begin, end}
      bool hit = false;
      for (int base = ch.z; base < ch.w; base += blockDim.x * 4) {
        bool h = false;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int a = base + q * blockDim.x + threadIdx.x;
          if (a < ch.w) {
            ++ha;
            h |= bu_arc<Topo, DIR>(p, ch.y, a, level);
          }
        }
        if (__syncthreads_or(h)) {
          hit = true;
          break;
        }
      }
      if (hit && threadIdx.x == 0 && atomicCAS(p.lab + ch.x, p.n, level + 1) == p.n) {
        ++found;
        fdeg += (unsigned long long)p.g.deg(ch.x);
      }
    }
  }
  arcs += ha;
  // one atomic per block for the level's count and arcs
  for (int o = 16; o > 0; o >>= 1) {
    found += __shfl_down_sync(0xffffffffu, found, o);
    fdeg += __shfl_down_sync(0xffffffffu, fdeg, o);
    arcs += __shfl_down_sync(0xffffffffu, arcs, o);
    verts += __shfl_down_sync(0xffffffffu, verts, o);
  }
  __shared__ unsigned long long s_f, s_d, s_a, s_v;
  if (threadIdx.x == 0) s_f = s_d = s_a = s_v = 0;
  __syncthreads();
  if (lane == 0) {
    if (found) atomicAdd(&s_f, found);
    if (fdeg) atomicAdd(&s_d, fdeg);
    if (arcs) atomicAdd(&s_a, arcs);
    if (verts) atomicAdd(&s_v, verts);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_f) atomicAdd(&c->bu_found[level % 3], (int)s_f);
    if (s_d) atomicAdd((unsigned long long*)&acc.fdeg, s_d);
    if (s_a) atomicAdd(&acc.bfs_arcs, s_a);
    if (s_v) atomicAdd(&acc.bfs_vertices, s_v);
  }
}

// Full BFS; on return every block has passed the closing barrier.  When
// `queues` is set, the active lists `cur` are rebuilt from the new labels
// (vertices with excess and label < n, other than s and t).
template <class Topo, int DIR>
__device__ bool bfs(const Params<Topo>& p, int root, bool queues, int cur, BlockAcc& acc,
                    bool keep_dead = false) {
  Ctl* c = p.ctl;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  // root < 0: every sink of the terminal sets is a root.  With keep_dead,
  // vertices an earlier global relabel of this launch marked dead (label
  // n + 1, see the end of this function) keep the mark: both directions
  // look only for label n, so their rows are never scanned again.
  for (int v = gt; v < p.n; v += gs) {
    if (root >= 0 ? v == root : is_sink(p, v)) p.lab[v] = 0;
    else if (!keep_dead || __ldcg(p.lab + v) <= p.n) p.lab[v] = p.n;
  }
  const long long dead = keep_dead ? ldv64(&c->dead_deg) : 0;
  if (gt == 0) {
    const int d = root >= 0 ? p.g.deg(root) : 0;
    if (root < 0) {
      c->fhcount[0] = 0;
      c->fcount[0] = 0;
    } else if (d > kTdHeavy) {
      const int nch = (d + kTdChunk - 1) / kTdChunk;
      for (int j = 0; j < nch; ++j) p.frh[0][j] = make_int2(root, j);
      c->fhcount[0] = nch;
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
    c->bu_found[0] = c->bu_found[1] = c->bu_found[2] = 0;
    c->bu_med[0] = c->bu_med[1] = c->bu_med[2] = 0;
    c->mcount = c->mhcount = 0;
    if (queues) {
      c->dpack = 0;
      c->light_next = 0;
      c->heavy_next = 0;
    }
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return false;
  // The active counts are cleared only now: a relabel that the plateau test
  // starts was decided on them at the top of the round, and a block may not
  // have read them yet when global thread 0 enters this function.
  if (queues && gt == 0) {
    c->lcount[cur] = 0;
    c->hcount[cur] = 0;
  }
  if (root < 0) {  // the sinks form level 0
    for (int base = gt - lane; base < p.n_sinks; base += gs) {
      const int i = base + lane;
      const int v = i < p.n_sinks ? __ldg(p.sinks + i) : -1;
      warp_frontier(p, &c->fcount[0], &c->fhcount[0], 0, v, v >= 0, acc);
    }
    __syncthreads();
    if (threadIdx.x == 0 && acc.fdeg) {
      atomicAdd((unsigned long long*)&c->fdeg[0], (unsigned long long)acc.fdeg);
      acc.fdeg = 0;
    }
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
  }
  // Every block derives the direction from values that are final at the
  // barrier (frontier size and arcs of this level), so all blocks agree.
  bool bu = false, prev_bu = false;
  long long visited = 0;
  for (int level = 0;; ++level) {
    const int fc = level % 3, fn = (level + 1) % 3, fr = (level + 2) % 3;
    // frontier size: list counters after top-down, found count after bottom-up
    const int nf = prev_bu ? ldv(&c->bu_found[(level + 2) % 3])
                           : ldv(&c->fcount[fc]) + ldv(&c->fhcount[fc]);
    if (nf == 0) break;
    const long long fdeg = ldv64(&c->fdeg[fc]);
    visited += fdeg;
    const long long rem = p.total_deg - dead - visited;
    if (!bu && fdeg * p.bfs_alpha > rem) bu = true;
    else if (bu && (long long)nf * kBfsBeta < (long long)p.n) bu = false;
    const bool mat = !bu && prev_bu;
    int nl = 0, nlh = 0;
    if (mat) {
      // the list of the bottom-up level's finds is built by a label scan
      bfs_materialise(p, level, fc, acc);
      if (!grid_sync(c, p.bar_timeout_ns)) return false;
      nl = ldv(&c->mcount);
      nlh = ldv(&c->mhcount);
    } else if (!bu) {
      nl = ldv(&c->fcount[fc]);
      nlh = ldv(&c->fhcount[fc]);
    }
    if (gt == 0) {
      // Each counter reset here was last read before the previous barrier
      // and is next written after the coming one.
      c->fcount[fr] = 0;
      c->fhcount[fr] = 0;
      c->fdeg[fr] = 0;
      c->bu_found[fn] = 0;
      c->bu_med[fn] = 0;
      if (!mat) c->mcount = c->mhcount = 0;
      atomicAdd(&p.st->bfs_levels, 1);
      if (bu) atomicAdd(&p.st->bu_levels, 1);
      TRACE(p, kTrLevel, bu ? 1 : 0, nf, fdeg);
    }
    if (threadIdx.x == 0) acc.fdeg = 0;
    __syncthreads();
    const unsigned long long tb = gtime();
    if (p.trace && threadIdx.x == 0) p.bt2[2 * gridDim.x + blockIdx.x] = tb;
    if (bu) bfs_bottom_up<Topo, DIR>(p, level, acc);
    else bfs_top_down<Topo, DIR>(p, level, nl, nlh, fc, fn, acc);
    TRACE_BLOCK(p, tb);
    __syncthreads();
    if (threadIdx.x == 0 && acc.fdeg)
      atomicAdd((unsigned long long*)&c->fdeg[fn], (unsigned long long)acc.fdeg);
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
    if (p.trace && bu && gt == 0) {
      // longest light-row part and longest medium-row part of any block
      unsigned long long ml = 0, mm = 0;
      for (int b2 = 0; b2 < (int)gridDim.x; ++b2) {
        const unsigned long long t1 = ldv64u(p.bt2 + b2), t2 = ldv64u(p.bt2 + gridDim.x + b2);
        const unsigned long long t0b = ldv64u(p.bt2 + 2 * gridDim.x + b2);
        ml = max(ml, t1 > t0b ? t1 - t0b : 0ull);
        mm = max(mm, t2 > t1 ? t2 - t1 : 0ull);
      }
      TRACE(p, kTrBuSplit, level, (long long)ml, (long long)mm);
    }
    prev_bu = bu;
  }
  if (queues) {
    // File the active vertices, and mark dead the ones left unreached: the
    // vertices that cannot reach a sink form a closed set (no residual arc
    // leaves it), and a push into or out of it would need an active vertex
    // labelled above n, so it stays closed for the rest of the phase.
    const int nall = p.n_light + p.n_medium + p.n_heavy;
    unsigned long long dd = 0;
    for (int base = gt - lane; base < nall; base += gs) {
      const int i = base + lane;
      int v = -1, ev = 0;
      bool pred = false;
      if (i < nall) {
        v = __ldg(p.cls + i);
        if (!is_terminal(p, v)) {
          const int lv = __ldcg(p.lab + v);
          if (lv == p.n) {
            p.lab[v] = p.n + 1;
            dd += (unsigned long long)p.g.deg(v);
          }
          ev = ldv(p.e + v);
          pred = ev > 0 && lv < p.n;
        }
      }
      warp_file(p, cur, v, ev, pred);
    }
    for (int o = 16; o > 0; o >>= 1) dd += __shfl_down_sync(0xffffffffu, dd, o);
    __shared__ unsigned long long s_dd;
    if (threadIdx.x == 0) s_dd = 0;
    __syncthreads();
    if (lane == 0 && dd) atomicAdd(&s_dd, dd);
    __syncthreads();
    if (threadIdx.x == 0 && s_dd) atomicAdd((unsigned long long*)&c->dead_deg, s_dd);
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Greedy two-hop routing, right after the preflow of a fresh solve with one
// sink on the BCSR layout: every vertex x that the preflow gave excess sends
// what it can straight on to t, along x->t and along x->y->t, taking the
// residual of each arc by compare-and-swap so that concurrent walkers never
// take more than an arc holds.  Every such move is a valid push of a preflow
// (a path of residual arcs whose middle vertex y keeps its excess), and labels
// are not consulted: the global relabel that opens the first round computes
// valid labels for whatever state this leaves.  So the maximum flow found is
// the same.  In a CPU model of this pass (vertices in order, arcs in row
// order) these moves carry 93% of the maximum flow of R-MAT scale 20 and 90%
// of the 2M x 2M matching before the first round.
// The y->t arc of each vertex y comes from the twins in t's row (an arc of
// capacity 0 whose twin has positive capacity), kept in `esnap` until the
// first global relabel files the active vertices (which overwrites it).
#ifndef WBPR_GREEDY_ARCS
#define WBPR_GREEDY_ARCS 1024
#endif
constexpr int kGreedyArcs = WBPR_GREEDY_ARCS;  // arcs of x's row a walker tries
#ifndef WBPR_GREEDY_SHORT
#define WBPR_GREEDY_SHORT 32
#endif
constexpr int kGreedyShort = WBPR_GREEDY_SHORT;  // of them by the walker's own thread,
constexpr int kGreedyBatch = 8;                  //   eight in flight; the rest by a warp

template <class Topo>
__device__ __forceinline__ bool greedy_applies(const Params<Topo>& p) {
  return p.greedy && !p.term && p.t >= 0;
}

// Take up to `want` from the residual word *r (0 if it holds none); `hint`
// is the value last read there (a guess for the first compare-and-swap), or
// -1 to read it first.
__device__ __forceinline__ int claim_residual(int* r, int want, int hint = -1) {
  int cur = hint >= 0 ? hint : ldv(r);
  while (cur > 0 && want > 0) {
    const int take = min(cur, want);
    const int prev = atomicCAS(r, cur, cur - take);
    if (prev == cur) return take;
    cur = prev;
  }
  return 0;
}

// The y->t arc of every vertex y into esnap[y].  RCSR: t's reverse entries
// are {y, forward id of y->t}.
__device__ __forceinline__ void two_hop_arcs(const Params<TopoR>& p) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  int b, e;
  p.g.seg(p.t, 1, b, e);
  for (int a = b + gt; a < e; a += gs) {
    const int2 r = __ldg(p.g.rarc + a);  // {tail y, forward arc y->t}
    if (r.x != p.s && p.g.cap_of(r.y) > 0) p.esnap[r.x] = r.y;
  }
}
// BCSR16: t's records that are twins of arcs into t.
__device__ __forceinline__ void two_hop_arcs(const Params<TopoB>& p) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  int b, e;
  p.g.seg(p.t, 0, b, e);
  for (int a = b + gt; a < e; a += gs) {
    const int2 x = __ldg(p.g.arx + a);  // {twin, capacity}
    if (x.y != 0) continue;             // t's own arc, not the twin of an arc into t
    if (__ldg(&p.g.arx[x.x].y) <= 0) continue;
    const int y = p.g.head(0, a);
    if (y != p.s) p.esnap[y] = x.x;
  }
}

// Move up to `want` units out of x along arc a (x->y) and on along arc yt
// (y->t), or straight along a when y is t (yt < 0).  Each residual is taken
// by compare-and-swap; what y->t cannot take goes back to x->y.  Returns
// the amount that reached t.
template <class Topo>
__device__ __forceinline__ int route_to_sink(const Params<Topo>& p, int a, int yt, int want, int cf_hint) {
  int* ra = p.g.resid(a);
  const int got1 = claim_residual(ra, want, cf_hint);
  if (got1 <= 0) return 0;
  int got = got1;
  if (yt >= 0) {
    got = claim_residual(p.g.resid(yt), got1);
    if (got < got1) atomicAdd(ra, got1 - got);  // hand back what y->t could not take
    if (got <= 0) return 0;
    atomicAdd(p.g.twin_resid(yt), got);
    p.g.log_push(yt);
  }
  atomicAdd(p.g.twin_resid(a), got);
  p.g.log_push(a);
  return got;
}

// The walker of arc sa of s: its vertex x and the excess that arc delivered.
// Only s's own arcs carried preflow (a twin in s's row is the reverse of an
// arc into s, with capacity 0), and a fresh solve's preflow pushed each one's
// whole capacity.  Returns the budget, 0 if the arc is no walker.
template <class Topo>
__device__ __forceinline__ int walker_of(const Params<Topo>& p, int sa, int& x) {
  const int cap = p.g.cap_of(sa);
  x = p.g.head(0, sa);
  if (cap <= 0 || x == p.t || x == p.s) return 0;
  return cap;
}

// Stage 1: a thread per walker over the first kGreedyShort arcs of x's row,
// eight in flight.  A walker with excess and arcs left joins the list of long
// walkers (fr[1]: its arc of s, fr[2]: its excess left).
template <class Topo>
__device__ __forceinline__ void two_hop_short(const Params<Topo>& p, BlockAcc& acc) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  int sb, se;
  p.g.seg(p.s, 0, sb, se);
  unsigned long long pushes = 0, scanned = 0;
  int sink = 0;
  for (int base = sb + gt - lane; base < se; base += gs) {  // whole warps, for the aggregated append
    const int sa = base + lane;
    int x = -1, budget = 0;
    if (sa < se) budget = walker_of(p, sa, x);
    const int budget0 = budget;
    int xb = 0, xe = 0;
    if (budget > 0) p.g.seg(x, 0, xb, xe);
    const int xend = min(xe, xb + kGreedyShort);
    for (int a0 = xb; a0 < xend && budget > 0; a0 += kGreedyBatch) {
      int y[kGreedyBatch], cf[kGreedyBatch], yt[kGreedyBatch];
#pragma unroll
      for (int q = 0; q < kGreedyBatch; ++q) {
        y[q] = -1;
        cf[q] = 0;
        if (a0 + q < xend) {
          p.g.load(0, a0 + q, y[q], cf[q]);
          ++scanned;
        }
      }
#pragma unroll
      for (int q = 0; q < kGreedyBatch; ++q)
        yt[q] = (cf[q] > 0 && y[q] >= 0 && y[q] != p.s && y[q] != p.t) ? __ldcg(p.esnap + y[q]) : -1;
#pragma unroll
      for (int q = 0; q < kGreedyBatch; ++q) {
        if (budget <= 0 || cf[q] <= 0 || y[q] < 0 || y[q] == p.s) continue;
        if (y[q] != p.t && yt[q] < 0) continue;
        const int got = route_to_sink(p, a0 + q, y[q] == p.t ? -1 : yt[q], min(budget, cf[q]), cf[q]);
        if (got > 0) {
          budget -= got;
          sink += got;
          pushes += y[q] == p.t ? 1 : 2;
        }
      }
    }
    if (budget < budget0) atomicSub(p.e + x, budget0 - budget);
    const bool more = budget > 0 && xe > xend && kGreedyArcs > kGreedyShort;
    const unsigned m = __ballot_sync(0xffffffffu, more);
    if (m) {
      int at = 0;
      const int leader = __ffs(m) - 1;
      if (lane == leader) at = atomicAdd(&p.ctl->glong, __popc(m));
      at = __shfl_sync(0xffffffffu, at, leader) + __popc(m & ((1u << lane) - 1u));
      if (more && at < p.n) {  // the lists hold n entries (parallel arcs of s could make more walkers)
        p.fr[1][at] = sa;
        p.fr[2][at] = budget;
      }
    }
  }
  if (sink) atomicAdd(&acc.sink, sink);
  if (pushes) atomicAdd(&acc.pushes, pushes);
  if (scanned) atomicAdd(&acc.scanned, scanned);
}

// Stage 2: a warp per long walker over arcs kGreedyShort .. kGreedyArcs of
// x's row, 128 at a time.  The lanes' shares of the excess left follow arc
// order by a saturating prefix sum (each capped at what the arc and its
// y->t arc hold when read), and all lanes route their shares together.
template <class Topo>
__device__ __forceinline__ void two_hop_long(const Params<Topo>& p, BlockAcc& acc) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nl = min(ldv(&p.ctl->glong), p.n);
  unsigned long long pushes = 0, scanned = 0;
  int sink = 0;
  // first walker by warp index, the rest claimed (walks differ in length)
  for (int w = gw; w < nl;) {
    int nx = 0;
    if (lane == 0) nx = nwarps + atomicAdd(&p.ctl->glong_next, 1);
    nx = __shfl_sync(0xffffffffu, nx, 0);
    const int sa = __ldcg(p.fr[1] + w);
    int budget = __ldcg(p.fr[2] + w);
    const int budget0 = budget;
    const int x = p.g.head(0, sa);
    int xb, xe;
    p.g.seg(x, 0, xb, xe);
    const int xend = min(xe, xb + kGreedyArcs);
    // 128 arcs a step, four consecutive ones per lane: a walk is at most
    // eight dependent steps instead of 31
    for (int a0 = xb + kGreedyShort; a0 < xend && budget > 0; a0 += 128) {
      int y[4], cf[4], yt[4], room[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int a = a0 + 4 * lane + k;
        y[k] = -1;
        cf[k] = 0;
        if (a < xend) p.g.load(0, a, y[k], cf[k]);
      }
      if (lane == 0) scanned += (unsigned long long)min(128, xend - a0);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        yt[k] = -1;
        if (cf[k] > 0 && y[k] != p.s && y[k] != p.t && y[k] >= 0) yt[k] = __ldcg(p.esnap + y[k]);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        room[k] = 0;
        if (cf[k] > 0 && y[k] != p.s && y[k] >= 0) {
          if (y[k] == p.t) room[k] = cf[k];
          else if (yt[k] >= 0) room[k] = min(cf[k], ldv(p.g.resid(yt[k])));
        }
      }
      // saturating prefix of the rooms in arc order: the lane's own four,
      // then over the lanes
      unsigned own = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        own += room[k] > 0 ? (unsigned)room[k] : 0u;
        if (own > (unsigned)budget) own = (unsigned)budget;
      }
      unsigned incl = own;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) {
          incl += v;
          if (incl > (unsigned)budget) incl = (unsigned)budget;
        }
      }
      unsigned before = __shfl_up_sync(0xffffffffu, incl, 1);
      if (lane == 0) before = 0;
      int got = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        unsigned upto = before + (room[k] > 0 ? (unsigned)room[k] : 0u);
        if (upto > (unsigned)budget) upto = (unsigned)budget;
        const int share = (int)(upto - before);
        before = upto;
        if (share > 0) {
          const int g1 = route_to_sink(p, a0 + 4 * lane + k, y[k] == p.t ? -1 : yt[k], share, cf[k]);
          if (g1 > 0) pushes += y[k] == p.t ? 1 : 2;
          got += g1;
        }
      }
      int tot = got;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
      budget -= tot;
      sink += got;
    }
    if (lane == 0 && budget < budget0) atomicSub(p.e + x, budget0 - budget);
    w = nx;
  }
  if (sink) atomicAdd(&acc.sink, sink);
  if (pushes) atomicAdd(&acc.pushes, pushes);
  if (scanned) atomicAdd(&acc.scanned, scanned);
}

__device__ __forceinline__ void clear_log(const TopoB& g, int gt) {
  if (g.ulog && gt < kLogSlots) {
    g.ulog_n[gt * kLogStride] = 0;
    g.ulog_n[gt * kLogStride + 1] = 0;
  }
}
__device__ __forceinline__ void clear_log(const TopoR&, int) {}

// ---------------------------------------------------------------------------
// Resident blocks per SM the register allocation is sized for: 4 blocks of
// 256 threads, 64 registers a thread (a few hundred bytes spilled).  Against
// 3 blocks at 80 registers, measured on GB300: R-MAT scale 22 3.97 -> 3.71 ms
// (the global relabels' latency-bound levels gain most), the 2M x 2M matching
// on this solver 9.70 -> 9.38 ms, 512 x 512 grids, layered networks and
// GENRMF within noise.
#ifndef WBPR_PR_MIN_BLOCKS
#define WBPR_PR_MIN_BLOCKS 4
#endif

template <class Topo, int W>
__global__ void __launch_bounds__(256, WBPR_PR_MIN_BLOCKS) pr_persistent(const __grid_constant__ Params<Topo> p) {
  __shared__ BlockAcc acc;
  Ctl* c = p.ctl;
  if (threadIdx.x == 0) {
    acc.scanned = acc.pushes = acc.relabels = acc.visits = acc.bfs_arcs = acc.bfs_vertices = acc.wmark = 0;
    acc.deep = 0;
    acc.fdeg = 0;
    acc.sink = 0;
  }
  __syncthreads();
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const unsigned long long t_start = gtime();
  if (gt == 0) p.st->t0 = t_start;

  if (p.mode == kModeBfsOnly) {
    if (p.bfs_dir == 0) bfs<Topo, 0>(p, p.bfs_root, false, 0, acc);
    else bfs<Topo, 1>(p, p.bfs_root, false, 0, acc);
    flush_acc(acc, p.st);
    return;
  }

  if (p.mode == kModeFresh) {
    // heights 0, excess 0, no pending relabel; residuals are reset by the
    // host-side reset kernel before this launch
    const bool greedy = greedy_applies(p);
    for (int v = gt; v < p.n; v += gs) {
      p.lab[v] = 0;
      p.e[v] = 0;
      p.rl_min[v] = kNone;
      if (greedy) p.esnap[v] = -1;  // the y->t arc of every vertex, filled below
    }
    // the residuals were restored before this launch: the undo log starts empty
    clear_log(p.g, gt);
    if (!grid_sync(c, p.bar_timeout_ns)) return;
    // preflow: saturate every residual arc out of s (reference preflow.cu:3-31,
    // with excess accumulated so parallel source arcs are kept)
    if (p.term) {  // terminal sets: a block per source
      for (int i = blockIdx.x; i < p.n_sources; i += gridDim.x) {
        const int src = __ldg(p.sources + i);
        for (int k = 0; k < Topo::kSeg; ++k) {
          int b, e;
          p.g.seg(src, k, b, e);
          for (int a = b + threadIdx.x; a < e; a += blockDim.x) {
            int dst, cf;
            p.g.load(k, a, dst, cf);
            if (cf > 0 && p.term[dst] != 1) {
              p.g.push(k, a, cf, cf);
              atomicAdd(p.e + dst, cf);
            }
          }
        }
      }
    } else {
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
      if (greedy) two_hop_arcs(p);
    }
    if (greedy) {
      if (!grid_sync(c, p.bar_timeout_ns)) return;
      unsigned long long tb = gtime();
      two_hop_short(p, acc);
      TRACE_BLOCK(p, tb);
      if (!grid_sync(c, p.bar_timeout_ns)) return;
      if (gt == 0) TRACE(p, kTrGreedy, 1, ldv(&c->glong), 0);
      tb = gtime();
      two_hop_long(p, acc);
      TRACE_BLOCK(p, tb);
      flush_sink(p.e + p.t, acc);
    }
  } else {
    for (int v = gt; v < p.n; v += gs) p.rl_min[v] = kNone;
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return;
  if (p.mode == kModeFresh && greedy_applies(p) && gt == 0) TRACE(p, kTrGreedy, 2, ldv(p.e + p.t), 0);

  int cur = 0, raw = 0, rounds = 0;
  bool need_gr = true;
  int gr_why = 0;  // trace only: what started the coming global relabel (bit 0 work, 1 rounds, 2 no
                   // flow, 3 active set not shrinking)
  int act_hist[kMaxPlateau];  // active counts of the last gr_plateau rounds, by since_gr % gr_plateau
  // work since the last global relabel: every block adds the per-round
  // counter of the finished round (final at the barrier), so all agree
  unsigned long long work = 0;
  int since_gr = 0;
  unsigned long long gr_ns = 0, round_ns = 0, push_ns = 0, deep_ns = 0;
  unsigned long long gr_end = 0, gr_last = 0;  // global thread 0 only
  bool marked = false;  // a global relabel has marked dead vertices (label n + 1)
  // global thread 0: rounds in a row after which excess(t) had not changed
  int stall = 0, et_prev = 0;
  for (;;) {
    if (need_gr) {
      const unsigned long long t0 = gtime();
      if (!bfs<Topo, 0>(p, p.term ? -1 : p.t, true, cur, acc, marked)) break;
      marked = true;
      if (gt == 0) {
        stall = 0;
        if (p.t >= 0) et_prev = ldv(p.e + p.t);
      }
      if (threadIdx.x == 0 && blockIdx.x == 0) {
        gr_end = gtime();
        gr_last = gr_end - t0;
        gr_ns += gr_last;
        atomicAdd(&p.st->grs, 1);
        TRACE(p, kTrGrEnd, gr_why, (long long)work, since_gr);
      }
      need_gr = false;
      work = 0;
      since_gr = 0;
    }
    const int nL = ldv(&c->lcount[cur]), nH = ldv(&c->hcount[cur]);
    const int nact = nL + nH;
    if (nact == 0) break;
    // An active set that stopped shrinking is excess circling without
    // reaching t (its labels climb a step or two a round): a global relabel
    // retires what cannot reach t at once.  The counts are final at the
    // barrier, so every block takes the same branch.
    if (p.gr_plateau > 0 && since_gr >= p.gr_plateau &&
        (long long)nact * 10 >= (long long)act_hist[since_gr % p.gr_plateau] * 9 && ldv(&c->gr_ok)) {
      need_gr = true;
      if (p.trace) gr_why = 8;
      continue;
    }
    if (p.gr_plateau > 0) act_hist[since_gr % p.gr_plateau] = nact;
    if (ldv(&c->stop)) {
      if (gt == 0) atomicCAS(&c->err, 0, (int)WBPR_ERR_NO_CONVERGENCE);
      break;
    }
    const unsigned long long t0 = gtime();
    if (gt == 0) TRACE(p, kTrRound, rounds, nL, nH);
    unsigned long long tb = gtime(), tdeep = 0;
    if (p.trace && threadIdx.x == 0) p.bt2[gridDim.x + blockIdx.x] = tb;
    push_first<Topo, W>(p, cur, raw, acc);
    if (nH > 0) {
      TRACE_BLOCK(p, tb);
      if (!grid_sync(c, p.bar_timeout_ns)) break;
      const unsigned long long dp = *(volatile unsigned long long*)&c->dpack;
      const int nD = (int)(dp & 0xffffffffu);
      if (gt == 0) {
        TRACE(p, kTrPassA, rounds, (long long)(dp >> 32), nD);
        if (p.trace) {  // longest heavy part and longest light part of any block
          unsigned long long mh = 0, ml = 0;
          for (int b = 0; b < (int)gridDim.x; ++b) {
            const unsigned long long t0b = ldv64u(p.bt2 + gridDim.x + b), th = ldv64u(p.bt2 + b);
            const unsigned long long tot = p.bt[b];
            mh = max(mh, th - t0b);
            ml = max(ml, tot > th - t0b ? tot - (th - t0b) : 0ull);
          }
          TRACE(p, kTrSplit, rounds, (long long)mh, (long long)ml);
        }
      }
      tb = gtime();
      if (nD > 0) {
        push_deep<Topo>(p, 0, nD, raw, acc);
        if (!grid_sync(c, p.bar_timeout_ns)) break;
        push_deep<Topo>(p, 1, nD, raw, acc);
        tdeep = tb;
      }
    }
    TRACE_BLOCK(p, tb);
    if (p.t >= 0) flush_sink(p.e + p.t, acc);
    flush_work(acc, c, raw);
    if (!grid_sync(c, p.bar_timeout_ns)) break;
    if (gt == 0) {
      const unsigned long long now = gtime();
      push_ns += now - t0;
      if (tdeep) deep_ns += now - tdeep;  // pass A start to the push phase's closing barrier
      TRACE(p, kTrPassB, rounds, 0, 0);
    }
    tb = gtime();
    relabel_phase<Topo>(p, cur, cur ^ 1, raw, acc);
    TRACE_BLOCK(p, tb);
    flush_work(acc, c, raw);
    if (gt == 0) {
      round_ns += gtime() - t0;
      if ((p.max_rounds > 0 && rounds + 1 >= p.max_rounds) || time_past(t_start, p.budget_ns))
        c->stop = 1;
      c->gr_ok = 2 * (gtime() - gr_end) >= gr_last;
      // excess(t) is final once the push phase's barrier has passed: every
      // block flushed its pushes into t before it
      if (p.gr_stall > 0 && p.t >= 0) {
        const int et = ldv(p.e + p.t);
        stall = et == et_prev ? stall + 1 : 0;
        et_prev = et;
        c->stalled = stall >= p.gr_stall;
      }
    }
    if (!grid_sync(c, p.bar_timeout_ns)) break;
    if (gt == 0) TRACE(p, kTrRelabel, rounds, ldv(&c->qraw_count[raw]), p.t >= 0 ? ldv(p.e + p.t) : 0);
    work += work_total(c, raw);
    ++rounds;
    ++since_gr;
    cur ^= 1;
    raw ^= 1;
    // Work-based trigger (Cherkassky-Goldberg) plus a round cap: tails where
    // a few stranded vertices ping-pong excess do little work per round
    // while their labels climb towards n two at a time.
    // Both triggers wait until the rounds since the last relabel have taken
    // at least half as long as that relabel did, so relabelling stays at
    // most about two thirds of the time on graphs whose BFS is deep (512 x
    // 512 grids: 38 -> 27 ms; a 20,000-vertex path whose one unit of excess
    // walks 20,000 rounds: 60 s of relabels every 48 rounds without it).
    // A run of rounds that moved no flow into t suggests the remaining
    // excess is cut off from t; a global relabel then retires it at once
    // instead of letting it climb towards n over many rounds.
    // (published by global thread 0 before the barrier, read by all after it)
    const bool stalled = ldv(&c->stalled) != 0;
    if ((work > p.gr_threshold || since_gr >= p.gr_rounds || stalled) && ldv(&c->gr_ok)) {
      need_gr = true;
      if (p.trace) gr_why = (work > p.gr_threshold) | (since_gr >= p.gr_rounds) << 1 | (int)stalled << 2;
    }
  }
  // callers see label n for every vertex that cannot reach the sink (every
  // block has left the loop after the same barrier and reads no label now)
  if (marked)
    for (int v = gt; v < p.n; v += gs)
      if (__ldcg(p.lab + v) > p.n) p.lab[v] = p.n;
  flush_acc(acc, p.st);
  if (gt == 0) {
    p.st->rounds = rounds;
    p.st->gr_ns = gr_ns;
    p.st->round_ns = round_ns;
    p.st->push_ns = push_ns;
    p.st->deep_ns = deep_ns;
  }
}

// Count vertices left with excess that cannot reach t (label n).
template <class Topo>
__global__ void count_stranded(Params<Topo> p) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  int cnt = 0;
  for (int v = gt; v < p.n; v += gs)
    if (!is_terminal(p, v) && p.e[v] > 0 && p.lab[v] >= p.n) ++cnt;
  if (cnt) atomicAdd(&p.st->stranded, cnt);
}

}  // namespace wbpr_dev
