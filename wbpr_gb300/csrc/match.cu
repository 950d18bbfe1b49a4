// Push-relabel specialised to unit-capacity bipartite matching networks.
//
// A network of the super-source / super-sink construction (s -> x for every
// left vertex x, x -> y for every edge, y -> t for every right vertex y, all
// capacities 1) has only three kinds of residual state, so the kernel keeps a
// matching instead of residuals.  One 64-bit word per right vertex y,
//   mate[y] = (x << 32) | label(y)     (x = kNoMate while y is free),
// stands for the flow on s -> x, x -> y and y -> t and for y's distance
// label.  A left vertex's label is implied: 1 + the least label over its
// residual arcs.  Every unmatched left vertex holds one unit of excess (the
// preflow saturated s -> x).  A round discharges each one by a double push:
// x pushes to its neighbour y of least label, and y passes its unit on at
// once -- into t when y was free, else back to its previous mate x', which
// becomes active.  The push is one compare-and-swap of y's word from the
// value x read during its scan to (x, label + 2): y's only residual arc then
// leads to x, one label above x's least label.  A lost race (another claim
// reached y first) makes x scan again.  So a right vertex's label rises
// exactly when its mate changes, from the value its new mate saw, and labels
// never fall between global relabels: the labelling stays valid (label(u) <=
// label(v) + 1 on every residual arc), and a left vertex whose least
// neighbour label is n cannot reach t.  When no active vertex is left, the
// matching is maximum (Goldberg-Tarjan phase 1 on this network).
//
// The global relabel is a BFS over alternating paths (free right vertices at
// label 1, a left x at k + 1 from a right y at k when x -> y is residual, x's
// mate at k + 2), direction-optimising as in the general solver.  It runs
// when the active set stops shrinking (its unmatched vertices that cannot
// reach t circle, their labels climbing two a round); the unmatched left
// vertices it reaches form the next active set, the rest are retired.
//
// At the end the matching is written into the residuals of either layout:
// three arcs per matched edge (on BCSR16 the host then has the next solve
// rewrite every residual in one streaming pass, cheaper than restoring three
// scattered arc pairs per matched edge from the undo log; RCSR rewrites them
// before every solve anyway).  excess(t) is the matching's
// size, every other excess is 0 (the residual graph of a maximum flow), and
// the right vertices' labels are written out from their words.  A left
// vertex's label is kept as it goes: 1 + its least neighbour label at its
// last push, k + 1 when a global relabel reached it at level k, n when it was
// found unable to reach t -- valid throughout, as right labels only rise and
// a push raises exactly the label of the vertex pushed to.  A label of n or
// more therefore proves a vertex dead for the rest of the solve (the set that
// cannot reach t is closed under pushes): global relabels mark such vertices
// n + 1 and never scan them again.  This specialises the general solver
// (maxflow-cuda/src/push_relabel_kernel.cu:400-537 and
// maxflow-cuda/src/global_relabel.cu:4-178 of the reference) to the
// bipartite inputs of the WBPR paper's matching experiments.
#include "match.h"

namespace wbpr_dev {

namespace {

constexpr int kRetry = 2;  // scans again after a lost claim before waiting a round

__device__ __forceinline__ unsigned long long mword(unsigned x, int lab) {
  return ((unsigned long long)x << 32) | (unsigned)lab;
}
__device__ __forceinline__ int wlab(unsigned long long w) { return (int)(unsigned)w; }
__device__ __forceinline__ int wmate(unsigned long long w) { return (int)(w >> 32); }  // -1 when free

struct MAcc {
  unsigned long long scanned, claims, visits, bfs_arcs, bfs_vertices;
};

// one atomic per converged group
__device__ __forceinline__ void count_one(int* cnt) {
  cg::coalesced_group g = cg::coalesced_threads();
  if (g.thread_rank() == 0) atomicAdd(cnt, (int)g.size());
}

__device__ __forceinline__ void add_block(long long* dst, long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long*)dst, (unsigned long long)v);
}

// arcs of left vertex x to right vertices: [b, b + d)
__device__ __forceinline__ int left_row(const MatchParams& p, int x, int& b) {
  b = __ldg(p.lrow + x);
  return __ldg(p.lrow + x + 1) - b - p.ltrim;
}
// arcs of right vertex y from left vertices: [b, e)
__device__ __forceinline__ void right_row(const MatchParams& p, int y, int& b, int& e) {
  b = __ldg(p.rrow + y) + p.rskip;
  e = __ldg(p.rrow + y + 1);
}
__device__ __forceinline__ int right_deg(const MatchParams& p, int y) {
  return __ldg(p.rrow + y + 1) - __ldg(p.rrow + y) - p.rskip;
}

// queue x for the next round by its row length
__device__ __forceinline__ void file_left(const MatchParams& p, int x, int nb, int* qc, int* hc) {
  int b;
  if (left_row(p, x, b) > p.heavy_deg) append(p.hq[nb], hc, x);
  else append(p.q[nb], qc, x);
}

// the right vertex x is matched to, -1 if none
__device__ __forceinline__ int mate_of_left(const MatchParams& p, int x) {
  const int y = __ldcg(p.cy + x);
  return y >= 0 && wmate(__ldcg(p.mate + y)) == x ? y : -1;
}

// x's push over arc a to the right vertex whose word x read as w (label < n):
// false when another claim changed the word first.  `evicted` is y's
// previous mate (-1: y was free, one more unit into t).
__device__ __forceinline__ bool take(const MatchParams& p, int x, int a, unsigned long long w, int& evicted) {
  const int y = __ldg(&p.lhd[a].x);
  const int l = wlab(w);
  if (atomicCAS(p.mate + y, w, mword((unsigned)x, min(l + 2, p.n))) != w) return false;
  p.claim[x] = a;
  p.cy[x] = y;
  p.lmin[x] = l;
  p.lab[x] = l + 1;  // x's label: 1 + its least neighbour label
  evicted = wmate(w);
  return true;
}

// Discharge of active left vertex x by a whole warp, 128 arcs in flight.
__device__ __forceinline__ void discharge_warp(const MatchParams& p, int x, int nb, int* qc, int* hc, MAcc& acc) {
  const int lane = threadIdx.x & 31;
  int b;
  const int d = left_row(p, x, b);
  int bound = max(__ldcg(p.lmin + x), 1);
  if (lane == 0) ++acc.visits;
  for (int tries = 0;; ++tries) {
    unsigned long long best = ~0ull, bw = 0;
    for (int k0 = 0; k0 < d; k0 += 128) {
      int y[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j * 32 + lane;
        y[j] = k < d ? __ldg(&p.lhd[b + k].x) : -1;
      }
      unsigned long long kl = ~0ull, wl = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (y[j] >= 0) {
          ++acc.scanned;
          const unsigned long long w = __ldcg(p.mate + y[j]);
          const unsigned long long key =
              ((unsigned long long)(unsigned)wlab(w) << 32) | (unsigned)(k0 + j * 32 + lane);
          if (key < kl) {
            kl = key;
            wl = w;
          }
        }
      unsigned long long km = kl;
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long q = __shfl_xor_sync(0xffffffffu, km, o);
        km = q < km ? q : km;
      }
      if (km < best) {
        const int src = __ffs(__ballot_sync(0xffffffffu, kl == km)) - 1;
        bw = __shfl_sync(0xffffffffu, wl, src);
        best = km;
      }
      if ((int)(best >> 32) <= bound) break;
    }
    const int ml = (int)(best >> 32);
    if (best == ~0ull || ml >= p.n) {  // cannot reach t
      if (lane == 0) p.lab[x] = p.n;
      break;
    }
    int ok = 0, ev = -1;
    if (lane == 0) {
      ok = take(p, x, b + (int)(unsigned)best, bw, ev);
      if (ok) {
        ++acc.claims;
        if (ev >= 0) file_left(p, ev, nb, qc, hc);
      } else if (tries == kRetry) {
        p.lab[x] = ml + 1;  // at most 1 + its least label now
        file_left(p, x, nb, qc, hc);
      }
    }
    if (__shfl_sync(0xffffffffu, ok, 0) || tries == kRetry) break;
    bound = ml;
  }
}

// Discharge of active left vertex x (row [b, b + d), early-exit bound) by
// its own thread, given the least key and word over its first four arcs:
// the rest of the row four arcs at a time unless the bound is already met,
// then the compare-and-swap, rescanning after a lost race.
__device__ __forceinline__ void discharge_thread(const MatchParams& p, int x, int b, int d, int bound,
                                                 unsigned long long best, unsigned long long bw, int nb, int* qc,
                                                 int* hc, MAcc& acc) {
  ++acc.visits;
  int from = 4;  // arcs already scanned into best
  for (int tries = 0;; ++tries) {
    for (int k0 = from; k0 < d && (best >> 32) > (unsigned long long)bound; k0 += 4) {
      int y[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) y[j] = k0 + j < d ? __ldg(&p.lhd[b + k0 + j].x) : -1;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (y[j] >= 0) {
          ++acc.scanned;
          const unsigned long long w = __ldcg(p.mate + y[j]);
          const unsigned long long key = ((unsigned long long)(unsigned)wlab(w) << 32) | (unsigned)(k0 + j);
          if (key < best) {
            best = key;
            bw = w;
          }
        }
    }
    const int ml = (int)(best >> 32);
    if (best == ~0ull || ml >= p.n) {  // cannot reach t
      p.lab[x] = p.n;
      return;
    }
    int ev;
    if (take(p, x, b + (int)(unsigned)best, bw, ev)) {
      ++acc.claims;
      if (ev >= 0) file_left(p, ev, nb, qc, hc);
      return;
    }
    if (tries == kRetry) {
      p.lab[x] = ml + 1;  // at most 1 + its least label now
      file_left(p, x, nb, qc, hc);
      return;
    }
    bound = ml;  // the label just lost to can only have risen
    best = ~0ull;
    from = 0;
  }
}

// One round: every active left vertex finds its first arc of least label and
// pushes over it.  A scan stops early at the least label the vertex saw last
// time (labels never fall between relabels).  Evicted mates, and vertices
// that lost kRetry + 1 races, go to the queues of buffer nb, counts slot rc.
// Long rows take a warp each; short rows a thread each, or a warp each when
// the whole active set fits one per warp (a tail round is then one vertex's
// dependent loads long, not a thread's walk of its row four arcs at a time).
__device__ void match_round(const MatchParams& p, const int* L, int nL, const int* H, int nH, int nb, int rc,
                            MAcc& acc) {
  MCtl* c = p.ctl;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const int gw = gt >> 5, nw = gs >> 5;
  int* qc = &c->qn[rc];
  int* hc = &c->hn[rc];
  if (nL + nH <= nw) {
    for (int i = gw; i < nL + nH; i += nw) discharge_warp(p, __ldcg(i < nH ? H + i : L + (i - nH)), nb, qc, hc, acc);
    return;
  }
  for (int i = gw; i < nH; i += nw) discharge_warp(p, __ldcg(H + i), nb, qc, hc, acc);
  // short rows: a thread each, two rows at a time (their first four arcs
  // and the heads' mate words in flight together), then each row on its own
  for (int i0 = gt; i0 < nL; i0 += 2 * gs) {
    int x[2], b[2], d[2], bound[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) x[q] = i0 + q * gs < nL ? __ldcg(L + i0 + q * gs) : -1;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      d[q] = 0;
      b[q] = 0;
      bound[q] = 1;
      if (x[q] >= 0) {
        d[q] = left_row(p, x[q], b[q]);
        bound[q] = max(__ldcg(p.lmin + x[q]), 1);
      }
    }
    int y[2][4];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int j = 0; j < 4; ++j) y[q][j] = j < d[q] ? __ldg(&p.lhd[b[q] + j].x) : -1;
    unsigned long long w[2][4];
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int j = 0; j < 4; ++j) w[q][j] = y[q][j] >= 0 ? __ldcg(p.mate + y[q][j]) : ~0ull;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (x[q] < 0) continue;
      unsigned long long best = ~0ull, bw = 0;
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (y[q][j] >= 0) {
          ++acc.scanned;
          const unsigned long long key = ((unsigned long long)(unsigned)wlab(w[q][j]) << 32) | (unsigned)j;
          if (key < best) {
            best = key;
            bw = w[q][j];
          }
        }
      discharge_thread(p, x[q], b[q], d[q], bound[q], best, bw, nb, qc, hc, acc);
    }
  }
}

// x has just been labelled k + 1 by level li: its mate (if any) gets k + 2
// and joins the next frontier; an unmatched x joins the active queue qb.
__device__ __forceinline__ void visit_left(const MatchParams& p, int x, int k, int li, bool list, int qb,
                                           long long& seen, long long& fdeg) {
  MCtl* c = p.ctl;
  int b;
  seen += left_row(p, x, b);
  p.lmin[x] = k;
  const int y = mate_of_left(p, x);
  if (y >= 0) {
    p.mate[y] = mword((unsigned)x, k + 2);  // y's only residual arc leads to x: reached through x alone
    fdeg += right_deg(p, y);
    if (list) append(p.fr[(li + 1) & 1], &c->fn[(li + 1) % 3], y);
    else count_one(&c->fn[(li + 1) % 3]);
  } else {
    file_left(p, x, qb, &c->gq[0], &c->gq[1]);
  }
}

// Bottom-up check of unlabelled left vertex x at level k, given whether its
// first four arcs hit: the rest of its row four arcs at a time until a
// neighbour labelled k is found; then x is labelled k + 1.
__device__ __forceinline__ void bu_finish(const MatchParams& p, int x, int b, int d, bool hit, int k, int li,
                                          int qb, long long& seen, long long& fdeg, MAcc& acc) {
  for (int k0 = 4; k0 < d && !hit; k0 += 4) {
    int y[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) y[j] = k0 + j < d ? __ldg(&p.lhd[b + k0 + j].x) : -1;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (y[j] >= 0) {
        ++acc.bfs_arcs;
        hit |= wlab(__ldcg(p.mate + y[j])) == k;
      }
  }
  if (hit) {
    p.lab[x] = k + 1;
    visit_left(p, x, k, li, false, qb, seen, fdeg);
  }
}

// Global relabel (see the file comment); the active queue it builds is
// buffer qb with counts gq.  False when a barrier failed.
__device__ bool match_gr(const MatchParams& p, int qb, MAcc& acc, int& levels, int& bu_levels) {
  MCtl* c = p.ctl;
  const int n = p.n;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  if (gt == 0) {
    c->gq[0] = c->gq[1] = 0;
    c->mcnt[0] = c->mcnt[1] = 0;
    for (int i = 0; i < 3; ++i) {
      c->fn[i] = 0;
      c->fdeg[i] = 0;
      c->seen[i] = 0;
    }
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return false;
  // unlabelled: n; proven dead (label n or more): n + 1, skipped by every
  // level and counted as seen arcs
  long long fd = 0, dead = 0;
  for (int i = gt; i < p.nl; i += gs) {
    const int x = __ldg(p.lv + i);
    if (__ldcg(p.lab + x) >= n) {
      p.lab[x] = n + 1;
      int b;
      dead += left_row(p, x, b);
    } else {
      p.lab[x] = n;
    }
  }
  for (int i = gt; i < p.nr; i += gs) {
    const int y = __ldg(p.rv + i);
    const unsigned long long w = __ldcg(p.mate + y);
    const int x = wmate(w);
    p.mate[y] = mword((unsigned)x, x < 0 ? 1 : (wlab(w) >= n ? n + 1 : n));
    if (x < 0) {
      append(p.fr[0], &c->fn[0], y);
      fd += right_deg(p, y);
    }
  }
  add_block(&c->fdeg[0], fd);
  add_block(&c->seen[0], dead);
  if (!grid_sync(c, p.bar_timeout_ns)) return false;
  bool listed = true;  // the current level's frontier is a list
  int mats = 0;        // materialised lists so far
  long long seen_all = 0;
  for (int li = 0, k = 1;; ++li, k += 2) {
    const int cur = li % 3, zz = (li + 2) % 3;
    const int nf = ldv(&c->fn[cur]);
    const long long fdeg = ldv64(&c->fdeg[cur]);
    seen_all += ldv64(&c->seen[cur]);
    if (nf == 0) break;
    ++levels;
    if (gt == 0) TRACE(p, kTrLevel, listed ? 0 : 1, nf, fdeg);
    const long long rem = p.left_arcs - seen_all;
    const bool bu = listed ? fdeg * p.bfs_alpha > rem : !((long long)nf * kBfsBeta < p.nr);
    int nlist = nf;
    if (!bu && !listed) {  // back to top-down: list the frontier first
      if (gt == 0) c->mcnt[(mats + 1) & 1] = 0;
      for (int i = gt; i < p.nr; i += gs) {
        const int y = __ldg(p.rv + i);
        if (wlab(__ldcg(p.mate + y)) == k) append(p.fr[li & 1], &c->mcnt[mats & 1], y);
      }
      if (!grid_sync(c, p.bar_timeout_ns)) return false;
      nlist = ldv(&c->mcnt[mats & 1]);
      ++mats;
    }
    if (gt == 0) {
      c->fn[zz] = 0;
      c->fdeg[zz] = 0;
      c->seen[zz] = 0;
    }
    long long seen = 0, nfd = 0;
    const unsigned long long tb = gtime();
    if (!bu) {
      // top-down: a thread per frontier vertex over its reverse arcs (slot 0
      // of a right row is y -> t), 4 in flight; rows longer than 32 arcs go
      // to the whole warp afterwards
      const int* F = p.fr[li & 1];
      if (nlist <= (gs >> 5)) {
        // a small frontier: a warp per vertex, lanes over its arcs (a tail
        // level is then one arc's dependent loads long)
        for (int i = gt >> 5; i < nlist; i += gs >> 5) {
          const int y = __ldcg(F + i);
          int b, e;
          right_row(p, y, b, e);
          if (lane == 0) ++acc.bfs_vertices;
          for (int a = b + lane; a < e; a += 32) {
            const int x = __ldg(&p.rhd[a].x);
            ++acc.bfs_arcs;
            if (__ldcg(p.lab + x) == n && atomicCAS(p.lab + x, n, k + 1) == n)
              visit_left(p, x, k, li, true, qb, seen, nfd);
          }
        }
      } else {
        for (int base = gt - lane; base < nlist; base += gs) {
          const int i = base + lane;
          int b = 0, e = 0;
          if (i < nlist) {
            const int y = __ldcg(F + i);
            right_row(p, y, b, e);
            ++acc.bfs_vertices;
          }
          const bool big = e - b > 32;
          if (!big)
            for (int a0 = b; a0 < e; a0 += 4) {
              int x[4];
#pragma unroll
              for (int j = 0; j < 4; ++j) x[j] = a0 + j < e ? __ldg(&p.rhd[a0 + j].x) : -1;
#pragma unroll
              for (int j = 0; j < 4; ++j)
                if (x[j] >= 0) {
                  ++acc.bfs_arcs;
                  if (__ldcg(p.lab + x[j]) == n && atomicCAS(p.lab + x[j], n, k + 1) == n)
                    visit_left(p, x[j], k, li, true, qb, seen, nfd);
                }
            }
          for (unsigned bm = __ballot_sync(0xffffffffu, big); bm; bm &= bm - 1) {
            const int src = __ffs(bm) - 1;
            const int bb = __shfl_sync(0xffffffffu, b, src), ee = __shfl_sync(0xffffffffu, e, src);
            for (int a = bb + lane; a < ee; a += 32) {
              const int x = __ldg(&p.rhd[a].x);
              ++acc.bfs_arcs;
              if (__ldcg(p.lab + x) == n && atomicCAS(p.lab + x, n, k + 1) == n)
                visit_left(p, x, k, li, true, qb, seen, nfd);
            }
          }
        }
      }
    } else {
      ++bu_levels;
      // bottom-up: every unlabelled left vertex looks for a neighbour at k
      // (its mate is unlabelled too, so it cannot be the one found)
      const int nh = p.nl - p.nl_light;
      for (int i = gt >> 5; i < nh; i += gs >> 5) {
        const int x = __ldg(p.lv + p.nl_light + i);
        if (__ldcg(p.lab + x) != n) continue;
        if (lane == 0) ++acc.bfs_vertices;
        int b;
        const int d = left_row(p, x, b);
        bool hit = false;
        for (int k0 = 0; k0 < d && !hit; k0 += 128) {
          int y[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int kk = k0 + j * 32 + lane;
            y[j] = kk < d ? __ldg(&p.lhd[b + kk].x) : -1;
          }
          bool h = false;
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (y[j] >= 0) {
              ++acc.bfs_arcs;
              h |= wlab(__ldcg(p.mate + y[j])) == k;
            }
          hit = __any_sync(0xffffffffu, h);
        }
        if (hit && lane == 0) {
          p.lab[x] = k + 1;
          visit_left(p, x, k, li, false, qb, seen, nfd);
        }
      }
      // short rows: a thread each, two at a time (labels, rows and the
      // first four heads' words of both in flight), then each on its own
      for (int i0 = gt; i0 < p.nl_light; i0 += 2 * gs) {
        int x[2], b[2], d[2];
        bool open[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) x[q] = i0 + q * gs < p.nl_light ? __ldg(p.lv + i0 + q * gs) : -1;
#pragma unroll
        for (int q = 0; q < 2; ++q) open[q] = x[q] >= 0 && __ldcg(p.lab + x[q]) == n;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          b[q] = 0;
          d[q] = 0;
          if (open[q]) {
            ++acc.bfs_vertices;
            d[q] = left_row(p, x[q], b[q]);
          }
        }
        int y[2][4];
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
          for (int j = 0; j < 4; ++j) y[q][j] = j < d[q] ? __ldg(&p.lhd[b[q] + j].x) : -1;
        bool hit[2] = {false, false};
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (y[q][j] >= 0) {
              ++acc.bfs_arcs;
              hit[q] |= wlab(__ldcg(p.mate + y[q][j])) == k;
            }
#pragma unroll
        for (int q = 0; q < 2; ++q)
          if (open[q]) bu_finish(p, x[q], b[q], d[q], hit[q], k, li, qb, seen, nfd, acc);
      }
    }
    add_block(&c->seen[(li + 1) % 3], seen);
    add_block(&c->fdeg[(li + 1) % 3], nfd);
    TRACE_BLOCK(p, tb);
    if (!grid_sync(c, p.bar_timeout_ns)) return false;
    listed = !bu;
  }
  return true;
}

// Four blocks of 256 per SM (64 registers): at three (80 registers, what the
// compiler picks unbounded) the relabels' latency-bound levels ran 1.7 ms
// instead of 0.9 on the 2M x 2M matching.
__global__ void __launch_bounds__(256, 4) pr_match(MatchParams p) {
  MCtl* c = p.ctl;
  const int n = p.n;
  const int lane = threadIdx.x & 31;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, gs = gridDim.x * blockDim.x;
  const unsigned long long t_start = gtime();
  if (gt == 0) p.st->t0 = t_start;
  MAcc acc{};
  // every label n (isolated vertices keep it; the first round, which visits
  // every left vertex, sets theirs), excess 0, right vertices free at label
  // 1, their exact distance to t
  for (int v = gt; v < n; v += gs) {
    p.lab[v] = n;
    p.e[v] = 0;
  }
  for (int i = gt; i < p.nr; i += gs) p.mate[__ldg(p.rv + i)] = mword(kNoMate, 1);
  for (int i = gt; i < p.nl; i += gs) {
    const int x = __ldg(p.lv + i);
    p.claim[x] = -1;
    p.cy[x] = -1;
    p.lmin[x] = 0;
  }
  if (p.ulog_n && gt < kLogSlots) {  // BCSR16: the undo log starts empty
    p.ulog_n[gt * kLogStride] = 0;
    p.ulog_n[gt * kLogStride + 1] = 0;
  }
  if (!grid_sync(c, p.bar_timeout_ns)) return;

  int rounds = 0, since_gr = 0, grs = 0, levels = 0, bu_levels = 0;
  unsigned long long work = 0, gr_ns = 0, round_ns = 0;
  unsigned long long gr_end = t_start, gr_last = 0;  // global thread 0 only
  int act_hist[kMaxPlateau];  // active counts of the last gr_plateau rounds
  bool need_gr = false, done = false, stopped = false, first = true;
  // the stop and time-balance words as read after the last round's barrier:
  // global thread 0 rewrites both during the next round, which it may enter
  // while another block is still deciding whether to run it
  bool stop = false, gr_ok = true;
  int nL = p.nl_light, nH = p.nl - p.nl_light;  // the first round takes every left vertex
  for (;;) {
    if (need_gr) {
      const unsigned long long t0 = gtime();
      if (!match_gr(p, rounds & 1, acc, levels, bu_levels)) break;
      nL = ldv(&c->gq[0]);
      nH = ldv(&c->gq[1]);
      ++grs;
      if (gt == 0) {
        gr_end = gtime();
        gr_last = gr_end - t0;
        gr_ns += gr_last;
        TRACE(p, kTrGrEnd, 0, nL, nH);
      }
      need_gr = false;
      work = 0;
      since_gr = 0;
    }
    const int nact = nL + nH;
    if (nact == 0) {  // every unmatched left vertex cannot reach t
      done = true;
      break;
    }
    if (stop) {
      if (gt == 0) atomicCAS(&c->err, 0, (int)WBPR_ERR_NO_CONVERGENCE);
      stopped = true;
      break;
    }
    // A set of active vertices that stopped shrinking is mostly excess that
    // cannot reach t circling (labels climbing two a round); a global relabel
    // retires it at once.  The counts are final at the barrier, so every
    // block takes the same branch.
    if (p.gr_plateau > 0 && since_gr >= p.gr_plateau &&
        (long long)nact * 10 >= (long long)act_hist[since_gr % p.gr_plateau] * 9 && gr_ok) {
      need_gr = true;
      continue;
    }
    if (p.gr_plateau > 0) act_hist[since_gr % p.gr_plateau] = nact;
    const unsigned long long t0 = gtime();
    const int b = rounds & 1;
    if (gt == 0) {
      c->qn[(rounds + 2) % 3] = 0;
      c->hn[(rounds + 2) % 3] = 0;
      c->work[(rounds + 1) % 3] = 0;
    }
    const unsigned long long w0 = acc.scanned + acc.visits, tb = gtime();
    match_round(p, first ? p.lv : p.q[b], nL, first ? p.lv + p.nl_light : p.hq[b], nH, b ^ 1, (rounds + 1) % 3,
                acc);
    add_block((long long*)&c->work[rounds % 3], (long long)(acc.scanned + acc.visits - w0));
    TRACE_BLOCK(p, tb);
    if (gt == 0) {
      if ((p.max_rounds > 0 && rounds + 1 >= p.max_rounds) || time_past(t_start, p.budget_ns)) c->stop = 1;
      c->gr_ok = 2 * (gtime() - gr_end) >= gr_last;
    }
    if (!grid_sync(c, p.bar_timeout_ns)) break;
    stop = ldv(&c->stop) != 0;
    gr_ok = ldv(&c->gr_ok) != 0;
    nL = ldv(&c->qn[(rounds + 1) % 3]);
    nH = ldv(&c->hn[(rounds + 1) % 3]);
    work += ldv64u(&c->work[rounds % 3]);
    if (gt == 0) {
      round_ns += gtime() - t0;
      TRACE(p, kTrRound, rounds, nL, nH);
    }
    ++rounds;
    ++since_gr;
    first = false;
    if ((work > p.gr_threshold || since_gr >= p.gr_rounds) && gr_ok) need_gr = true;
  }
  if (done || stopped) {
    // the matching as residuals: x -> y, y -> t and s -> x saturated (a
    // stopped solve leaves the matching it had, a flow all the same), and
    // the labels of the right vertices
    int cnt = 0;
    for (int i = gt; i < p.nr; i += gs) {
      const int y = __ldg(p.rv + i);
      const unsigned long long w = __ldcg(p.mate + y);
      p.lab[y] = min(wlab(w), n);
      const int x = wmate(w);
      if (x < 0) continue;
      const int a = __ldcg(p.claim + x);  // x -> y
      const int ay = __ldg(p.lrow + y);   // y -> t, the first arc of y's row
      if (p.arx) {
        // BCSR16: each arc and its twin; the twin of s -> x ends x's row
        const int ax = __ldg(p.lrow + x + 1) - 1;
        p.lhd[a].y = 0;
        p.lhd[__ldg(&p.arx[a].x)].y = 1;
        p.lhd[ay].y = 0;
        p.lhd[__ldg(&p.arx[ay].x)].y = 1;
        p.lhd[ax].y = 1;
        p.lhd[__ldg(&p.arx[ax].x)].y = 0;
      } else {
        // RCSR: forward residual 0, reverse residual 1; s -> x is the
        // forward arc of x's one reverse entry
        const int sx = __ldg(&p.rhd[__ldg(p.rrow + x)].y);
        p.lhd[a].y = 0;
        p.fcb[a] = 1;
        p.lhd[ay].y = 0;
        p.fcb[ay] = 1;
        p.lhd[sx].y = 0;
        p.fcb[sx] = 1;
      }
      ++cnt;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0 && cnt) atomicAdd(p.e + p.t, cnt);
    for (int i = gt; i < p.nl; i += gs) {  // callers see labels in [0, n]
      const int x = __ldg(p.lv + i);
      if (__ldcg(p.lab + x) > n) p.lab[x] = n;
    }
    if (gt == 0) {
      p.lab[p.s] = n;
      p.lab[p.t] = 0;
    }
  }
  unsigned long long* dst[5] = {&p.st->arcs_scanned, &p.st->pushes, &p.st->vertex_visits, &p.st->bfs_arcs,
                                &p.st->bfs_vertices};
  unsigned long long val[5] = {acc.scanned, acc.claims, acc.visits, acc.bfs_arcs, acc.bfs_vertices};
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    unsigned long long v = val[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0 && v) atomicAdd(dst[j], v);
  }
  if (gt == 0) {
    p.st->rounds = rounds;
    p.st->grs = grs;
    p.st->gr_ns = gr_ns;
    p.st->round_ns = round_ns;
    p.st->push_ns = round_ns;
    p.st->bfs_levels = levels;
    p.st->bu_levels = bu_levels;
  }
}

}  // namespace

cudaError_t launch_match(const MatchParams& p, int blocks, int threads, cudaStream_t st) {
  void* args[] = {(void*)&p};
  return cudaLaunchCooperativeKernel((const void*)pr_match, dim3(blocks), dim3(threads), args, 0, st);
}

int occupancy_match(int threads) {
  int nb = 0;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pr_match, threads, 0) == cudaSuccess ? nb : 0;
}

}  // namespace wbpr_dev
