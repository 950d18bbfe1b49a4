/*
 * wbpr.h -- C ABI of the GB300 push-relabel maximum-flow library (libwbpr.so).
 *
 * This is the only surface through which host code reaches CUDA.  Every
 * signature uses plain C types: pointers, sizes and the structs below.  The
 * library owns all device memory it allocates; inputs are copied at
 * create time; no entry point calls exit().  One handle per host thread.
 *
 * Reference interfaces replaced (paths inside the WBPR project):
 *   - preflow(...)        maxflow-cuda/include/parallel_graph.cuh:44-46,
 *                         maxflow-cuda/src/preflow.cu:3-31
 *   - push_relabel(...)   maxflow-cuda/include/parallel_graph.cuh:47-54,
 *                         maxflow-cuda/src/push_relabel.cu:35-221
 *   - global_relabel / global_relabel_gpu
 *                         maxflow-cuda/src/global_relabel.cu:4-178,
 *                         maxflow-bcsr/src/global_relabel_gpu.cu:4-189
 *   - CSRGraph readers    maxflow-cuda/src/graph.cpp:28-67,151-214,219-233,292-314
 *   - ResidualGraph::buildFromCSRGraph
 *                         maxflow-cuda/src/graph.cpp:317-402 (RCSR),
 *                         maxflow-bcsr/src/graph.cpp:317-360 (BCSR),
 *                         maxflow-bcsr2/src/graph.cpp:326-362 (BCSR2)
 */
#ifndef WBPR_H_
#define WBPR_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WBPR_ABI_VERSION 2

typedef enum wbpr_status {
  WBPR_OK = 0,
  WBPR_ERR_INVALID_ARG = 1,    /* bad pointer, vertex id, size or enum      */
  WBPR_ERR_CUDA = 2,           /* a CUDA runtime call failed                */
  WBPR_ERR_NO_CONVERGENCE = 3, /* round / time budget exhausted             */
  WBPR_ERR_OVERFLOW = 4,       /* int32 excess or arc index would overflow  */
  WBPR_ERR_VERIFY = 5,         /* device invariant check failed             */
  WBPR_ERR_IO = 6,             /* file missing, truncated or malformed      */
  WBPR_ERR_NO_DEVICE = 7,      /* no CUDA device visible                    */
  WBPR_ERR_TIMEOUT = 8         /* a bounded grid-wide wait gave up          */
} wbpr_status;

/* Residual-graph layout kept on the device. */
typedef enum wbpr_layout {
  WBPR_LAYOUT_RCSR = 0,  /* forward CSR + reversed CSR with flow index        */
  WBPR_LAYOUT_BCSR = 1,  /* one row per vertex holding forward and reverse    */
                         /* arcs; 16-byte arc record {dst, cf | rev, cap}     */
  WBPR_LAYOUT_BCSR2 = 2  /* accepted alias of BCSR: the reference's BCSR2     */
                         /* {cf, rev} pair is the same record                 */
} wbpr_layout;

typedef enum wbpr_algo {
  WBPR_ALGO_TC = 0, /* thread-centric: one thread discharges one vertex       */
  WBPR_ALGO_VC = 1  /* vertex-centric: one 8/16/32-lane tile per vertex       */
} wbpr_algo;

/* Input graph in CSR form (the reference's CSRGraph, graph.h:28-58).
 * Arc i of vertex u is offsets[u] <= i < offsets[u+1], head destinations[i],
 * capacity capacities[i] >= 0.  capacities may be NULL (all capacities 1). */
typedef struct wbpr_csr {
  int32_t num_nodes;
  int64_t num_edges;
  const int32_t* offsets;      /* num_nodes + 1 */
  const int32_t* destinations; /* num_edges     */
  const int32_t* capacities;   /* num_edges or NULL */
  int32_t source;              /* -1 if the file did not name one */
  int32_t sink;
} wbpr_csr;

/* Host-owned CSR returned by the readers and generators; free with
 * wbpr_host_csr_free. */
typedef struct wbpr_host_csr {
  int32_t num_nodes;
  int64_t num_edges;
  int64_t num_edges_declared; /* value of the file header (DIMACS p / SNAP #) */
  int32_t* offsets;
  int32_t* destinations;
  int32_t* capacities;
  int32_t source;
  int32_t sink;
} wbpr_host_csr;

typedef struct wbpr_tuning {
  int32_t tile;          /* VC tile width: 8, 16 or 32 (0 = auto)                 */
  int32_t block;         /* threads per block: 64..256, multiple of 32 (0 = 256)  */
  int32_t heavy_degree;  /* rows longer than this are discharged by a whole warp  */
                         /* (128 arcs in flight) instead of a tile (0 = 32)       */
  int32_t blocks_per_sm; /* resident blocks per SM for the persistent grid (0=max) */
  double gr_alpha;       /* global relabel after alpha*(n + arcs) units of work   */
                         /* (0 = 1.0)                                             */
  int64_t max_rounds;    /* push/relabel round budget (0 = unlimited)             */
  double max_ms;         /* wall-clock budget of one solve in ms (0 = 120000)     */
  int32_t verify;        /* 1: run the device certificate check after the solve  */
  int32_t trace;         /* 1: record a per-level / per-phase event trace         */
  int32_t gr_rounds;     /* also relabel globally after this many rounds (0 = 48) */
  int32_t grid_blocks;   /* blocks of the persistent grid (0 = auto by size:      */
                         /* n + arcs <= 16384: one block, block barriers only;    */
                         /* <= 2^21: SMs / 2; <= 2^22: SMs; <= 2^24: 2 x SMs;     */
                         /* larger: every SM x blocks_per_sm)                     */
  int32_t gr_stall;      /* also relabel globally after this many rounds in a row */
                         /* that moved no flow into t (0 = auto: 1 when n + arcs  */
                         /* > 2^22, else never; -1 = never)                       */
  int64_t barrier_timeout_ns; /* a grid-barrier wait gives up after this long and */
                         /* the solve returns WBPR_ERR_TIMEOUT (0 = 10 s)         */
  int32_t greedy;        /* solves with one sink: 0 = route excess along           */
                         /* x->t and x->y->t paths right after the preflow (the   */
                         /* same maximum flow, fewer rounds); -1 = off            */
  int32_t bfs_alpha;     /* a global relabel's BFS turns bottom-up when the        */
                         /* frontier's arcs x this exceed the unvisited arcs      */
                         /* (0 = 14; 4 in the matching kernel)                    */
  int32_t gr_plateau;    /* also relabel globally when the active set shrank by   */
                         /* less than 10% over this many rounds, 1..8 (0 or -1 =  */
                         /* never, the default)                                   */
  int32_t matching;      /* 0 = a terminal pair whose network is a                */
                         /* unit-capacity bipartite matching network (s -> left,  */
                         /* left -> right, right -> t, every capacity 1, no other */
                         /* arc) is solved by the matching kernel; -1 = always    */
                         /* the general solver                                    */
  int32_t pad2;
  int64_t batch_cluster; /* batches: instances of at least this many units (n +   */
                         /* residual arcs) run on 8-block thread-block clusters, */
                         /* the rest one block each (0 = 3 x 2^17, -1 = none)     */
} wbpr_tuning;

typedef struct wbpr_result {
  int64_t flow;            /* maximum-flow value: excess of the sink         */
  float solve_ms;          /* device time, reset + preflow + solve           */
  float kernel_ms;         /* push/relabel rounds only (reference's timer)   */
  float gr_ms;             /* global relabel BFS time                        */
  uint64_t arcs_scanned;   /* residual arcs read by discharges               */
  uint64_t pushes;         /* arcs that carried a push                       */
  uint64_t relabels;       /* vertex relabels                                */
  uint64_t vertex_visits;  /* active-vertex discharges                       */
  uint64_t bfs_arcs;       /* arcs inspected by global relabels              */
  uint64_t bfs_vertices;   /* vertex checks by global relabels               */
  uint64_t alg_bytes;      /* algorithmic bytes of the persistent solver     */
                           /* launch (bytes_push + bytes_relabel + bytes_gr  */
                           /* + 12 n of initialisation)                      */
  int32_t rounds;          /* push/relabel supersteps                        */
  int32_t global_relabels; /* BFS passes                                     */
  int32_t stranded;        /* vertices left with excess unable to reach t    */
  float launch_ms;         /* CUDA-event time of the persistent solver kernel */
  float push_ms;           /* push phases of the rounds (rest: relabel)      */
  int32_t bfs_levels;      /* BFS levels over all global relabels            */
  int32_t bfs_bottom_up_levels; /* of which bottom-up                        */
  uint64_t heavy_visits;   /* discharges of rows handled by a whole block    */
  uint64_t bytes_push;     /* algorithmic bytes of the push phases: 12 per   */
                           /* arc scanned, 16 per visit, 24 per push (28     */
                           /* with the undo-log entry)                       */
  uint64_t bytes_deep;     /* of which the deep passes: 12 per arc           */
  uint64_t bytes_relabel;  /* relabel phases: 12 per relabel                 */
  uint64_t bytes_gr;       /* global relabels: 12 per arc inspected, 8 per   */
                           /* vertex check, 4 n per relabel                  */
  float deep_ms;           /* deep passes of the push phases (in push_ms)    */
  int32_t matching;        /* 1: solved by the matching kernel (rounds are   */
                           /* double-push rounds, pushes their claims)       */
  uint64_t deep_arcs_scanned; /* arcs read by the deep passes (in arcs_scanned) */
} wbpr_result;

typedef struct wbpr_verify_report {
  int32_t ok;                 /* 1 when every check passed                 */
  int32_t capacity_violations;/* arcs with cf < 0 or cf > cap + cap(rev)   */
  int32_t conservation_violations; /* vertices whose excess != in - out    */
  int32_t source_reaches_sink;/* 1 if a residual s->t path exists          */
  int32_t excess_reaches_sink;/* vertices with excess that reach t         */
  int32_t label_violations;   /* residual arcs u->v with h(u) > h(v) + 1 and
                                 h(u) < n (solver labelling; informational) */
  int64_t cut_value;          /* capacity of the sink-side residual cut    */
  int64_t flow_value;         /* excess of the sink                        */
} wbpr_verify_report;

typedef struct wbpr_graph wbpr_graph;

/* ---- status / version ---------------------------------------------------- */
const char* wbpr_status_str(wbpr_status s);
int32_t wbpr_abi_version(void);
void wbpr_default_tuning(wbpr_tuning* t);
/* Number of CUDA devices (0 when none); never fails. */
int32_t wbpr_device_count(void);
/* Text of the last CUDA failure seen by this host thread ("" if none). */
const char* wbpr_last_error(void);

/* ---- graph readers (replace CSRGraph::build* / loadFromBinary) ----------- */
/* -v 0: SNAP text, "# Nodes: N Edges: M" header, capacity 1 (graph.cpp:28-67) */
wbpr_status wbpr_read_snap_txt(const char* path, wbpr_host_csr** out);
/* -v 1: SNAP binary [n][m][m_processed][dst...][offsets...] (graph.cpp:292-314) */
wbpr_status wbpr_read_snap_bin(const char* path, wbpr_host_csr** out);
/* -v 2: DIMACS max-flow "p max / n s|t / a u v c", 1-based (graph.cpp:151-214) */
wbpr_status wbpr_read_dimacs(const char* path, wbpr_host_csr** out);
/* Writers: SNAP binary (graph.cpp:219-233) and DIMACS text. */
wbpr_status wbpr_write_snap_bin(const char* path, const wbpr_csr* g);
wbpr_status wbpr_write_dimacs(const char* path, const wbpr_csr* g);
/* -v 3: graph cache, new (the SNAP .bin above has no capacities and no
 * terminals): "WBPRCSR1", int32 version 1, int32 flags (bit 0: capacities
 * present), int64 n, m, m_declared, int32 s, t, then int32 offsets[n+1],
 * destinations[m], capacities[m]; little endian.  Reading is one copy. */
wbpr_status wbpr_write_graph_cache(const char* path, const wbpr_csr* g);
wbpr_status wbpr_read_graph_cache(const char* path, wbpr_host_csr** out);
/* Maximum-flow solution in DIMACS form: "s <flow>" and one "f u v x" line
 * (1-based) per input arc with x = arc_flow[i] > 0, in input order.  Give it
 * the flows of a completed flow (wbpr_complete_flow, then wbpr_read_state). */
wbpr_status wbpr_write_dimacs_flow(const char* path, const wbpr_csr* g, int64_t flow,
                                   const int32_t* arc_flow);
/* Bipartite matching as maximum flow (WBPR paper, section IV-A): left
 * vertices 0..L-1, right L..L+R-1, s = L+R, t = L+R+1; arcs s->l, l->r for
 * every listed pair (left[k], right[k]) (ids 0-based within their side;
 * duplicates kept once) and r->t, all of capacity 1.  The matching is the set
 * of l->r arcs that carry flow in a completed flow. */
wbpr_status wbpr_bipartite_network(int32_t L, int32_t R, int64_t num_pairs,
                                   const int32_t* left, const int32_t* right,
                                   wbpr_host_csr** out);
/* Copy a caller CSR into a library-owned one. */
wbpr_status wbpr_host_csr_copy(const wbpr_csr* in, wbpr_host_csr** out);
void wbpr_host_csr_free(wbpr_host_csr* g);

/* ---- seeded synthetic generators (integer arithmetic, same bits on x86 and
 *      aarch64) ---------------------------------------------------------- */
/* GENRMF-shaped frames: b frames of a x a grids; in-frame 4-neighbour arcs of
 * capacity c2*a*a, one inter-frame arc per vertex to a seeded permutation of
 * the next frame with capacity uniform in [c1, c2]; s = 0, t = n - 1. */
wbpr_status wbpr_gen_genrmf(int32_t a, int32_t b, int32_t c1, int32_t c2,
                            uint64_t seed, wbpr_host_csr** out);
/* R-MAT scale/edge-factor with quadrant probabilities a,b,c (d = rest),
 * self loops and duplicates removed, capacities uniform in [cap_lo, cap_hi];
 * s = max out-degree vertex, t = max in-degree vertex (lowest id on ties). */
wbpr_status wbpr_gen_rmat(int32_t scale, int32_t edge_factor, double a,
                          double b, double c, int32_t cap_lo, int32_t cap_hi,
                          uint64_t seed, wbpr_host_csr** out);
/* Unit-capacity bipartite matching network: s=0, left 1..L, right L+1..L+R,
 * t=L+R+1; left degrees ~ Zipf(zipf_s) clipped to [1, dmax]. */
wbpr_status wbpr_gen_bipartite(int32_t left, int32_t right, double zipf_s,
                               int32_t dmax, uint64_t seed,
                               wbpr_host_csr** out);
/* Layered network: s=0, `layers` layers of `width` vertices, each vertex has
 * deg_lo..deg_hi arcs into the next layer, t = n-1; caps in [cap_lo, cap_hi]. */
wbpr_status wbpr_gen_layered(int32_t layers, int32_t width, int32_t deg_lo,
                             int32_t deg_hi, int32_t cap_lo, int32_t cap_hi,
                             uint64_t seed, wbpr_host_csr** out);
/* Vision graph-cut grid w x h, 4-connected n-links, t-links; s = w*h,
 * t = w*h + 1 (smooth seeded field, see the generator for the formulas). */
wbpr_status wbpr_gen_grid(int32_t w, int32_t h, uint64_t seed,
                          wbpr_host_csr** out);

/* ---- residual-graph builders (exact reverse pairing, O(n + m)) ----------- */
/* (wbpr_graph_create builds the same arrays on the device; these host
 * builders are for callers that want them in host memory.) */
/* RCSR (maxflow-cuda/src/graph.cpp:317-402): roffsets[n+1], rdestinations[m],
 * flow_index[m] (reverse entry -> forward arc id).  Caller-allocated. */
wbpr_status wbpr_build_rcsr(const wbpr_csr* g, int32_t* roffsets,
                            int32_t* rdestinations, int32_t* flow_index);
/* BCSR (maxflow-bcsr/src/graph.cpp:317-360): every input arc gets its own
 * reverse twin.  offsets[n+1], destinations[2m], capacities[2m] (0 for a
 * twin), backward_idx[2m].  Caller-allocated. */
wbpr_status wbpr_build_bcsr(const wbpr_csr* g, int32_t* offsets,
                            int32_t* destinations, int32_t* capacities,
                            int32_t* backward_idx);
/* BCSR2 (maxflow-bcsr2/src/graph.cpp:326-362): as BCSR, with the interleaved
 * flows[2a] = residual, flows[2a+1] = reverse arc id.  flows is 4m ints. */
wbpr_status wbpr_build_bcsr2(const wbpr_csr* g, int32_t* offsets,
                             int32_t* destinations, int32_t* flows);

/* ---- device graph and solve --------------------------------------------- */
wbpr_status wbpr_graph_create(const wbpr_csr* g, wbpr_layout layout,
                              wbpr_graph** out);
wbpr_status wbpr_graph_destroy(wbpr_graph* g);
/* Bytes of device memory held by the handle. */
int64_t wbpr_graph_device_bytes(const wbpr_graph* g);
/* Device memory of graphs and batches comes from a stream-ordered pool per
 * device owned by the library.  Memory freed by wbpr_graph_destroy /
 * wbpr_batch_destroy (and the build's temporaries) stays reserved in the pool
 * up to max_bytes (16 GiB by default), so the next graph of a similar size is
 * created without mapping memory, and destroyed without unmapping it.  This
 * sets max_bytes for the current device's pool (and for pools created later)
 * and releases reserved memory above it now; 0 returns all free memory to the
 * driver.  Negative max_bytes: WBPR_ERR_INVALID_ARG. */
wbpr_status wbpr_memory_cache(int64_t max_bytes);
/* Replace the m capacities (input order; host or device buffer) of a built
 * graph without rebuilding it: the same topology with new capacities, e.g.
 * the next frame of a graph-cut pipeline.  Checked first (capacities >= 0:
 * INVALID_ARG; incoming sums within int32: OVERFLOW), and the graph is left
 * unchanged when a check fails.  Takes effect at the next wbpr_solve. */
wbpr_status wbpr_graph_set_capacities(wbpr_graph* g, const int32_t* capacities);
/* Queue the handle's device work on the caller's stream (a cudaStream_t of
 * the handle's device; NULL returns to the handle's own stream).  Work queued
 * before the switch is finished first.  Calls still return once their
 * results are on the host. */
wbpr_status wbpr_graph_set_stream(wbpr_graph* g, void* stream);
/* Copy a BCSR handle's residual graph, as built on the device, back to host
 * buffers in the format of wbpr_build_bcsr (offsets[n+1], destinations[2m],
 * capacities[2m], backward_idx[2m]; any may be NULL).  The device build is
 * the same arrays as the host build, entry for entry.  INVALID_ARG for an
 * RCSR handle. */
wbpr_status wbpr_graph_read_bcsr(const wbpr_graph* g, int32_t* offsets, int32_t* destinations,
                                 int32_t* capacities, int32_t* backward_idx);
/* The same for an RCSR handle, in the format of wbpr_build_rcsr (roffsets[n+1],
 * rdestinations[m], flow_index[m]; the forward arrays are the input CSR).
 * INVALID_ARG for a BCSR handle. */
wbpr_status wbpr_graph_read_rcsr(const wbpr_graph* g, int32_t* roffsets, int32_t* rdestinations,
                                 int32_t* flow_index);
/* Fresh solve: reset residuals to capacities, preflow from s, push/relabel to
 * a maximum preflow.  Result flow = excess(t). s/t = -1 use the graph's. */
wbpr_status wbpr_solve(wbpr_graph* g, int32_t s, int32_t t, wbpr_algo algo,
                       const wbpr_tuning* tuning, wbpr_result* out);
/* Many (source, sink) pairs in one solve, new: the preflow saturates the arcs
 * of every source, every sink absorbs flow and roots the global relabel, and
 * flows[i] receives the flow that ended at sinks[i].  When each pair lies in
 * its own connected component -- many instances stored as one disjoint-union
 * graph -- flows[i] is the maximum flow from sources[i] to sinks[i], and all
 * instances are solved by the whole GPU at once.  Every vertex may hold at
 * most one terminal role.  The handle's single-pair state (wbpr_verify,
 * wbpr_mincut_adjoint, wbpr_complete_flow) does not apply to this solve. */
wbpr_status wbpr_solve_pairs(wbpr_graph* g, int32_t k, const int32_t* sources, const int32_t* sinks,
                             wbpr_algo algo, const wbpr_tuning* tuning, int64_t* flows, wbpr_result* out);
/* Try tile widths {8, 16, 32} (VC; TC has one), global-relabel work factors
 * {0.5, 1, 1.5, 3} and long-row thresholds {32, 64} on this graph and
 * these terminals (the faster of two solves each), then the best of those
 * with bfs_alpha 4, gr_plateau 4 and both; return the fastest tuning and its
 * solve time.  Every tuning must give the same flow (WBPR_ERR_VERIFY
 * otherwise).  The graph's state afterwards is that of the last solve. */
wbpr_status wbpr_autotune(wbpr_graph* g, int32_t s, int32_t t, wbpr_algo algo, wbpr_tuning* best,
                          float* best_ms);
/* Read back the state after a solve (host buffers, any may be NULL):
 * height[n], excess[n], and per input arc flow = cap - residual (m). */
wbpr_status wbpr_read_state(wbpr_graph* g, int32_t* height, int32_t* excess,
                            int32_t* arc_flow);
/* Event trace of the last solve run with tuning.trace = 1: the last `cap`
 * records of 6 int64 {kind | aux << 32, ns since kernel start, v0, v1, longest
 * and shortest block work time (ns) of the phase that the record closes};
 * kinds 1 BFS level (aux bottom-up, v0 frontier, v1 frontier arcs), 2 round
 * start (aux round, v0 light list, v1 heavy entries << 32 | chunks), 3 pass A
 * end, 4 push phase end, 5 relabel end (v0 next raw queue), 6 global relabel
 * end.  Returns the number of records copied. */
int32_t wbpr_read_trace(wbpr_graph* g, int64_t* out, int32_t cap);
/* Certificate check on the device: capacities, conservation, and that no
 * residual path leads from s or from any excess vertex to t (so the value is
 * maximal), and cut value == flow value. */
wbpr_status wbpr_verify(wbpr_graph* g, wbpr_verify_report* rep);
/* Min-cut adjoint: per input arc int8 indicator g[e] of the exact
 * (super)gradient d maxflow / d cap(e).  side 0: sink-side cut (vertices that
 * can reach t form T, g = [u not in T and v in T]); side 1: source-side cut
 * (S = vertices reachable from s once the stranded excess is returned,
 * g = [u in S and v not in S]).  `indicator` is a host or device buffer of
 * m bytes. */
wbpr_status wbpr_mincut_adjoint(wbpr_graph* g, int32_t side, int8_t* indicator,
                                float* adjoint_ms);
/* Turn the maximum preflow of the last solve into a maximum flow: the excess
 * left at vertices that cannot reach t is pushed back to s (a second solve
 * with s as the sink), so every vertex other than s and t conserves flow.
 * Per-arc flows read afterwards (wbpr_read_state) form a valid maximum flow;
 * the flow value is unchanged.  `ms` (may be NULL) receives the device time. */
wbpr_status wbpr_complete_flow(wbpr_graph* g, float* ms);
/* Vertex sides of the two extreme minimum cuts: side 0 -> in_set[v] = 1 iff v
 * can reach t in the residual graph (the sink side T); side 1 -> in_set[v] = 1
 * iff v is reachable from s after wbpr_complete_flow (the source side S).
 * `in_set` is a host buffer of n bytes. */
wbpr_status wbpr_cut_sides(wbpr_graph* g, int32_t side, int8_t* in_set);

/* ---- batched solver ---------------------------------------------------------- */
/* No counterpart in the reference (its CLI solves one graph per process).
 * Many independent instances, each with its own source and sink, solved in one
 * launch: every thread block claims a whole instance (largest first) and runs
 * preflow, global relabels and push/relabel rounds with block-level barriers
 * only, scheduling its own global relabels.  The launch is captured into a
 * CUDA graph on the first solve with a given tuning and replayed afterwards. */
typedef struct wbpr_batch wbpr_batch;
wbpr_status wbpr_batch_create(const wbpr_csr* graphs, int32_t count, wbpr_batch** out);
wbpr_status wbpr_batch_destroy(wbpr_batch* b);
int64_t wbpr_batch_device_bytes(const wbpr_batch* b);
/* flows (host, count entries, may be NULL): maximum-flow values, -1 for an
 * instance that hit its budget (then WBPR_ERR_NO_CONVERGENCE).  Uses
 * tuning.tile (8/16/32), .block (64..512), .gr_alpha, .gr_rounds, .max_rounds,
 * .max_ms (per instance). */
wbpr_status wbpr_batch_solve(wbpr_batch* b, const wbpr_tuning* tuning, int64_t* flows, float* solve_ms);
/* Per-instance device time (ms) and rounds of the last solve (either may be NULL). */
wbpr_status wbpr_batch_instance_stats(wbpr_batch* b, float* inst_ms, int32_t* inst_rounds);
/* Try tile widths, block sizes and global-relabel frequencies on this batch,
 * then which instances run on clusters (batch_cluster: none, 2^18 or 2^19
 * units); return the fastest tuning and its time. */
wbpr_status wbpr_batch_autotune(wbpr_batch* b, wbpr_tuning* best, float* best_ms);

/* ---- solve without any device allocation --------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory (code running inside a caller-owned memory pool or arena, or a
 * framework that forbids cudaMalloc on its hot path): the caller passes the
 * BCSR residual graph in device buffers it owns and receives the maximum flow
 * in *flow (host).  The buffers interleave the arrays wbpr_build_bcsr writes:
 *   d_row[n+1]  = offsets;
 *   d_arc[2a]   = destinations[a], d_arc[2a+1] = residual of arc a (reset
 *                 to the capacity at the start, the final residual on return);
 *   d_arx[2a]   = backward_idx[a], d_arx[2a+1] = capacities[a].
 * They are checked on the device before the solve: d_row must start at 0, end
 * at num_residual_arcs and never decrease; heads must lie in [0, n), twins be
 * paired, capacities be >= 0 (WBPR_ERR_INVALID_ARG otherwise); and no vertex's
 * incoming capacities may sum past int32 (WBPR_ERR_OVERFLOW).  All solver
 * scratch lives in one fixed file-scope device array (about 5.6 MB per device,
 * held until exit), so no allocation happens.  Limits: n <= 65536 vertices and
 * num_residual_arcs <= 1048576; larger inputs return WBPR_ERR_INVALID_ARG (see
 * wbpr_last_error).  The first call on a device looks up the array's address;
 * make it before any stream capture.  Calls share the array: calls that
 * overlap on the GPU race and must be serialised by the caller.  `stream` is
 * a cudaStream_t or NULL; the call synchronises it before returning. */
wbpr_status wbpr_solve_bcsr_noalloc(int32_t n, int64_t num_residual_arcs, const int32_t* d_row,
                                    int32_t* d_arc, const int32_t* d_arx, int32_t s, int32_t t,
                                    int32_t algo, void* stream, int64_t* flow);

/* ---- drop-ins for the reference host functions (RCSR arrays, in place) --- */
/* Same arguments and meaning as preflow() in maxflow-cuda/src/preflow.cu:3-31,
 * except that excess is accumulated (+=) so parallel source arcs are not lost.
 * Returns a wbpr_status. */
int32_t wbpr_rcsr_preflow(int32_t V, int32_t source, int32_t sink,
                          int32_t* cpu_height, int32_t* cpu_excess_flow,
                          const int32_t* offsets, const int32_t* destinations,
                          const int32_t* capacities, int32_t* forward_flows,
                          int32_t* backward_flows, const int32_t* roffsets,
                          const int32_t* rdestinations, const int32_t* flow_idx,
                          int32_t* Excess_total);
/* Same arguments and in-place contract as push_relabel() in
 * maxflow-cuda/src/push_relabel.cu:35-221 (host arrays only: the library owns
 * the device copies).  On return cpu_height, cpu_excess_flow, cpu_fflows and
 * cpu_bflows hold the final state, cpu_excess_flow[sink] is the maximum flow,
 * *Excess_total = e(s) + e(t), and *kernel_ms (may be NULL) the push/relabel
 * kernel time.  Returns a wbpr_status. */
int32_t wbpr_rcsr_push_relabel(int32_t algo_type, int32_t V, int32_t E,
                               int32_t source, int32_t sink,
                               int32_t* cpu_height, int32_t* cpu_excess_flow,
                               const int32_t* cpu_offsets,
                               const int32_t* cpu_destinations,
                               const int32_t* cpu_capacities,
                               int32_t* cpu_fflows, int32_t* cpu_bflows,
                               const int32_t* cpu_roffsets,
                               const int32_t* cpu_rdestinations,
                               const int32_t* cpu_flow_idx,
                               int32_t* Excess_total, float* kernel_ms);

#ifdef __cplusplus
}
#endif
#endif /* WBPR_H_ */
