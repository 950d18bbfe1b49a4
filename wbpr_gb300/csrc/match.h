// Unit-capacity bipartite matching networks (s -> left -> right -> t, every
// capacity 1): the solver specialised to them, declared for the host code of
// the graph handle.
#pragma once

#include <cuda_runtime.h>

#include "pr_kernel.cuh"

namespace wbpr_dev {

// Mate word of a right vertex y: (x << 32) | label of y, x = kNoMate while y
// is free.  A claim replaces the whole word with one compare-and-swap, so a
// right vertex's label changes only together with its mate.
constexpr unsigned kNoMate = 0xffffffffu;

// Control block of the matching kernel (zeroed before every launch).  Words
// every block touches in the same phase sit on their own 128-byte lines.
struct MCtl {
  alignas(128) unsigned bar;  // grid barrier word
  alignas(128) int err;
  int stop;
  alignas(128) int qn[3];     // light active queue counts, by round % 3
  alignas(128) int hn[3];     // heavy active queue counts, by round % 3
  alignas(128) int gq[2];     // the queue a global relabel builds: light, heavy
  alignas(128) int fn[3];     // right vertices labelled by a BFS level, by level % 3
  alignas(128) int mcnt[2];   // materialised frontier lists
  alignas(128) long long fdeg[3];  // their reverse arcs
  alignas(128) long long seen[3];  // forward arcs of the left vertices a level labelled
  alignas(128) unsigned long long work[3];  // arcs scanned + visits of a round, by round % 3
  alignas(128) int gr_ok;     // the rounds since the last global relabel took half as long as it
  // detection (wbpr_graph side): shape violations, list counters
  alignas(128) int bad;
  int nlist[3];  // light left, heavy left, right
  long long larcs;
};

struct MatchParams {
  // The rows as either layout holds them, heads in .x: left vertex x's arcs
  // to right vertices are lhd[lrow[x], lrow[x + 1] - ltrim), right vertex y's
  // arcs from left vertices are rhd[rrow[y] + rskip, rrow[y + 1]).  BCSR16:
  // both are the residual rows (row, arc), a left row ends with the twin of
  // s -> x (ltrim 1) and a right row starts with y -> t (rskip 1).  RCSR: the
  // forward rows (frow, farc) and the reverse entries (rrow, rarc {tail,
  // forward arc id}), ltrim = rskip = 0.
  const int* lrow;
  int2* lhd;
  int ltrim;
  const int* rrow;
  const int2* rhd;
  int rskip;
  // where the matching is written back: BCSR16 twins (arx, fcb null) or RCSR
  // reverse residuals (fcb, arx null)
  const int2* arx;
  int* fcb;
  int* ulog_n;  // BCSR16 undo-log counters, cleared at the start (null for RCSR)
  int n, s, t;
  int nl, nl_light, nr;
  const int* lv;   // left vertices: rows of at most heavy_deg arcs first, then the longer ones
  const int* rv;   // right vertices
  long long left_arcs;  // forward arcs of all left vertices
  unsigned long long* mate;  // right vertex -> mate word
  // per left vertex, kept in three arrays (one 16-byte record per vertex
  // measured 40% slower on the 2M x 2M matching: the global relabel reads
  // only cy, and the rounds only lmin)
  int* claim;      // slot of the arc of its last claim (-1: none)
  int* cy;         // the right vertex of that claim (-1: none)
  int* lmin;       // the least label it found last
  int* lab;        // labels of the left vertices (BFS marks), and all labels at the end
  int* e;          // excess
  int* q[2];       // active left vertices, rows of at most heavy_deg arcs
  int* hq[2];      // active left vertices, longer rows
  int* fr[2];      // BFS frontier lists (right vertices)
  MCtl* ctl;
  Stats* st;
  int heavy_deg;
  int bfs_alpha;
  unsigned long long gr_threshold;  // global relabel after this much round work
  int gr_rounds;                    // or at the latest after this many rounds
  int gr_plateau;                   // or when the active set shrank by < 10% over this many rounds
  long long max_rounds;
  unsigned long long budget_ns;
  unsigned long long bar_timeout_ns;
  long long* trace;        // optional event records (the general solver's format)
  unsigned long long* bt;  // per-block time of the current phase (trace only)
  int trace_cap;
};

cudaError_t launch_match(const MatchParams& p, int blocks, int threads, cudaStream_t st);
int occupancy_match(int threads);

}  // namespace wbpr_dev
