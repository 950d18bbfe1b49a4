/*
 * oracle.c -- CPU oracle for the WBPR push-relabel path.  TEST
 * INFRASTRUCTURE ONLY: tests, the smoke check and the CPU-baseline leg of
 * the benchmark call it as the checker; the product never links it.
 *
 * Three independent computations of the maximum-flow value:
 *   oracle_serial_maxflow  restatement of the reference CPU solver
 *                          (maxflow-serial/graph.cpp:316-401 residual build,
 *                          :463-479 preflow, :482-518 push, :521-524 relabel,
 *                          :527-540 findActiveNode, :555-589 maxflow,
 *                          :592-619 checkPath).  O(n) per operation: small
 *                          graphs only.
 *   oracle_dinic           Dinic's blocking-flow algorithm (BFS levels,
 *                          iterative DFS with current arcs), int64 flows.
 *   oracle_fifo_pr         FIFO push-relabel with global relabelling and the
 *                          gap heuristic (Cherkassky-Goldberg), int64 excess.
 * Parity pin: the serial restatement reproduces the reference binary's
 * "Max flow" output on the reference's own fixtures and on seeded graphs (see
 * tests/golden/make_golden.py, which runs the reference compiled from its
 * sources by oracle/build_oracle.py).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_NO_PATH 1
#define ORC_BUDGET 2
#define ORC_NOMEM 3

/* ------------------------------------------------------------------------ */
/* Restatement of maxflow-serial.  Reverse CSR in the same fill order as the
 * reference (tails ascending); flow_index takes the FIRST forward arc u->v
 * for a reverse entry, as graph.cpp:386-399 does.  Preflow assigns the excess
 * (excesses[dest] = cap, graph.cpp:474).  Returns excess(t) as the reference
 * prints it; *status = ORC_NO_PATH when checkPath fails (the reference then
 * prints no value; the flow is 0). */
int64_t oracle_serial_maxflow(int32_t n, const int32_t* off, const int32_t* dst,
                              const int32_t* cap, int32_t s, int32_t t,
                              int64_t max_ops, int32_t* status) {
  int64_t m = off[n];
  int32_t *roff = calloc((size_t)n + 1, 4), *rdst = malloc(4 * (size_t)(m + 1)),
          *fidx = malloc(4 * (size_t)(m + 1)), *ff = malloc(4 * (size_t)(m + 1)),
          *bf = malloc(4 * (size_t)(m + 1)), *h = calloc((size_t)n, 4),
          *ex = calloc((size_t)n, 4), *cnt = calloc((size_t)n, 4);
  char* vis = calloc((size_t)n, 1);
  int32_t* stack = malloc(4 * (size_t)n + 4);
  int64_t result = 0;
  *status = ORC_OK;
  if (!roff || !rdst || !fidx || !ff || !bf || !h || !ex || !cnt || !vis || !stack) {
    *status = ORC_NOMEM;
    goto done;
  }
  for (int64_t i = 0; i < m; ++i) {
    ff[i] = cap[i];
    bf[i] = 0;
    roff[dst[i] + 1]++;
  }
  for (int32_t v = 0; v < n; ++v) roff[v + 1] += roff[v];
  for (int32_t u = 0; u < n; ++u)
    for (int32_t j = off[u]; j < off[u + 1]; ++j) {
      int32_t v = dst[j];
      rdst[roff[v] + cnt[v]++] = u;
    }
  for (int32_t u = 0; u < n; ++u)
    for (int32_t i = roff[u]; i < roff[u + 1]; ++i) {
      int32_t v = rdst[i];
      fidx[i] = -1;
      for (int32_t j = off[v]; j < off[v + 1]; ++j)
        if (dst[j] == u) {
          fidx[i] = j;
          break;
        }
    }
  /* checkPath: DFS over forward arcs */
  {
    int32_t sp = 0, found = 0;
    stack[sp++] = s;
    vis[s] = 1;
    while (sp && !found) {
      int32_t u = stack[--sp];
      for (int32_t i = off[u]; i < off[u + 1]; ++i) {
        int32_t v = dst[i];
        if (!vis[v]) {
          if (v == t) {
            found = 1;
            break;
          }
          stack[sp++] = v;
          vis[v] = 1;
        }
      }
    }
    if (!found && !vis[t]) {
      *status = ORC_NO_PATH;
      goto done;
    }
  }
  /* preflow */
  h[s] = n;
  for (int32_t i = off[s]; i < off[s + 1]; ++i) {
    ex[dst[i]] = cap[i];
    ff[i] = 0;
    bf[i] = cap[i];
  }
  for (int64_t ops = 0;; ++ops) {
    if (max_ops > 0 && ops >= max_ops) {
      *status = ORC_BUDGET;
      break;
    }
    /* findActiveNode: lowest label < n among vertices with excess */
    int32_t a = -1, best = n;
    for (int32_t i = 0; i < n; ++i)
      if (ex[i] > 0 && i != s && i != t && h[i] < best) {
        best = h[i];
        a = i;
      }
    if (a < 0) break;
    /* push along the first arc with h(v) == h(w) + 1 and flow > 0 */
    int pushed = 0;
    for (int32_t i = off[a]; i < off[a + 1] && !pushed; ++i) {
      int32_t w = dst[i];
      if (h[a] == h[w] + 1) {
        int32_t f = ex[a] < ff[i] ? ex[a] : ff[i];
        if (f == 0) continue;
        ff[i] -= f;
        bf[i] += f;
        ex[a] -= f;
        ex[w] += f;
        pushed = 1;
      }
    }
    for (int32_t i = roff[a]; i < roff[a + 1] && !pushed; ++i) {
      int32_t w = rdst[i];
      if (h[a] == h[w] + 1) {
        int32_t pi = fidx[i];
        int32_t f = ex[a] < bf[pi] ? ex[a] : bf[pi];
        if (f == 0) continue;
        bf[pi] -= f;
        ff[pi] += f;
        ex[a] -= f;
        ex[w] += f;
        pushed = 1;
      }
    }
    if (!pushed) h[a] += 1; /* relabel */
  }
  result = ex[t];
done:
  free(roff);
  free(rdst);
  free(fidx);
  free(ff);
  free(bf);
  free(h);
  free(ex);
  free(cnt);
  free(vis);
  free(stack);
  return result;
}

/* ------------------------------------------------------------------------ */
/* Residual graph with paired arcs for the exact solvers. */
typedef struct {
  int32_t n;
  int64_t na;
  int64_t* first; /* n + 1 */
  int32_t* head;
  int64_t* res;
  int64_t* rev;
  int64_t* fwd_of_input; /* input arc -> residual slot */
} RG;

static void rg_free(RG* g) {
  free(g->first);
  free(g->head);
  free(g->res);
  free(g->rev);
  free(g->fwd_of_input);
}

static int rg_build(RG* g, int32_t n, const int32_t* off, const int32_t* dst, const int32_t* cap) {
  int64_t m = off[n];
  memset(g, 0, sizeof(*g));
  g->n = n;
  g->na = 2 * m;
  g->first = calloc((size_t)n + 1, 8);
  g->head = malloc(4 * (size_t)(2 * m + 1));
  g->res = malloc(8 * (size_t)(2 * m + 1));
  g->rev = malloc(8 * (size_t)(2 * m + 1));
  g->fwd_of_input = malloc(8 * (size_t)(m + 1));
  int64_t* cur = calloc((size_t)n + 1, 8);
  if (!g->first || !g->head || !g->res || !g->rev || !g->fwd_of_input || !cur) {
    free(cur);
    rg_free(g);
    return ORC_NOMEM;
  }
  for (int32_t u = 0; u < n; ++u) {
    g->first[u + 1] += off[u + 1] - off[u];
    for (int32_t i = off[u]; i < off[u + 1]; ++i) g->first[dst[i] + 1]++;
  }
  for (int32_t u = 0; u < n; ++u) g->first[u + 1] += g->first[u];
  for (int32_t u = 0; u < n; ++u) cur[u] = g->first[u];
  for (int32_t u = 0; u < n; ++u)
    for (int32_t i = off[u]; i < off[u + 1]; ++i) {
      int32_t v = dst[i];
      int64_t a = cur[u]++, b = cur[v]++;
      g->head[a] = v;
      g->res[a] = cap ? cap[i] : 1;
      g->rev[a] = b;
      g->head[b] = u;
      g->res[b] = 0;
      g->rev[b] = a;
      g->fwd_of_input[i] = a;
    }
  free(cur);
  return ORC_OK;
}

/* Dinic. */
static int64_t dinic_run(RG* g, int32_t s, int32_t t) {
  const int32_t n = g->n;
  int32_t* level = malloc(4 * (size_t)n);
  int32_t* q = malloc(4 * (size_t)n);
  int64_t* it = malloc(8 * (size_t)n);
  int64_t* pa = malloc(8 * (size_t)n + 8); /* arc stack of the DFS path */
  int64_t flow = 0;
  if (!level || !q || !it || !pa) goto out;
  for (;;) {
    for (int32_t i = 0; i < n; ++i) level[i] = -1;
    int32_t qh = 0, qt = 0;
    level[s] = 0;
    q[qt++] = s;
    while (qh < qt) {
      int32_t u = q[qh++];
      for (int64_t a = g->first[u]; a < g->first[u + 1]; ++a)
        if (g->res[a] > 0 && level[g->head[a]] < 0) {
          level[g->head[a]] = level[u] + 1;
          q[qt++] = g->head[a];
        }
    }
    if (level[t] < 0) break;
    for (int32_t i = 0; i < n; ++i) it[i] = g->first[i];
    /* iterative DFS: walk admissible arcs, augment at t, retreat on dead ends */
    int32_t depth = 0, u = s;
    for (;;) {
      if (u == t) {
        int64_t b = INT64_MAX;
        for (int32_t k = 0; k < depth; ++k)
          if (g->res[pa[k]] < b) b = g->res[pa[k]];
        for (int32_t k = 0; k < depth; ++k) {
          g->res[pa[k]] -= b;
          g->res[g->rev[pa[k]]] += b;
        }
        flow += b;
        /* restart from the first saturated arc */
        int32_t k0 = 0;
        while (k0 < depth && g->res[pa[k0]] > 0) ++k0;
        depth = k0;
        u = depth ? g->head[pa[depth - 1]] : s;
        continue;
      }
      int64_t a;
      for (a = it[u]; a < g->first[u + 1]; ++a)
        if (g->res[a] > 0 && level[g->head[a]] == level[u] + 1) break;
      it[u] = a;
      if (a < g->first[u + 1]) {
        pa[depth++] = a;
        u = g->head[a];
      } else {
        if (u == s) break;
        level[u] = -1; /* dead end */
        --depth;
        u = depth ? g->head[pa[depth - 1]] : s;
        it[u]++;
      }
    }
  }
out:
  free(level);
  free(q);
  free(it);
  free(pa);
  return flow;
}

int64_t oracle_dinic(int32_t n, const int32_t* off, const int32_t* dst, const int32_t* cap,
                     int32_t s, int32_t t) {
  RG g;
  if (rg_build(&g, n, off, dst, cap)) return -1;
  int64_t f = dinic_run(&g, s, t);
  rg_free(&g);
  return f;
}

/* Dinic plus both extreme minimum cuts.  For every input arc i (u -> v):
 *   sink_side[i]   = [u cannot reach t in the final residual graph, v can]
 *   source_side[i] = [u reachable from s, v not]
 * Either array may be NULL. */
int64_t oracle_mincut(int32_t n, const int32_t* off, const int32_t* dst, const int32_t* cap,
                      int32_t s, int32_t t, int8_t* sink_side, int8_t* source_side) {
  RG g;
  if (rg_build(&g, n, off, dst, cap)) return -1;
  int64_t f = dinic_run(&g, s, t);
  char* rs = calloc((size_t)n, 1);
  char* rt = calloc((size_t)n, 1);
  int32_t* q = malloc(4 * (size_t)n + 4);
  if (rs && rt && q) {
    int32_t qh = 0, qt = 0;
    rs[s] = 1;
    q[qt++] = s;
    while (qh < qt) {
      int32_t u = q[qh++];
      for (int64_t a = g.first[u]; a < g.first[u + 1]; ++a)
        if (g.res[a] > 0 && !rs[g.head[a]]) {
          rs[g.head[a]] = 1;
          q[qt++] = g.head[a];
        }
    }
    qh = qt = 0;
    rt[t] = 1;
    q[qt++] = t;
    while (qh < qt) {
      int32_t v = q[qh++];
      for (int64_t a = g.first[v]; a < g.first[v + 1]; ++a) {
        int32_t u = g.head[a];
        if (!rt[u] && g.res[g.rev[a]] > 0) { /* residual u -> v */
          rt[u] = 1;
          q[qt++] = u;
        }
      }
    }
    for (int32_t u = 0; u < n; ++u)
      for (int32_t i = off[u]; i < off[u + 1]; ++i) {
        int32_t v = dst[i];
        if (sink_side) sink_side[i] = (int8_t)(!rt[u] && rt[v]);
        if (source_side) source_side[i] = (int8_t)(rs[u] && !rs[v]);
      }
  } else {
    f = -1;
  }
  free(rs);
  free(rt);
  free(q);
  rg_free(&g);
  return f;
}

/* ------------------------------------------------------------------------ */
/* FIFO push-relabel with global relabel (BFS from t) every ~n relabels and
 * the gap heuristic.  Phase 1 only: the value is the sink excess. */
int64_t oracle_fifo_pr(int32_t n, const int32_t* off, const int32_t* dst, const int32_t* cap,
                       int32_t s, int32_t t) {
  RG g;
  if (rg_build(&g, n, off, dst, cap)) return -1;
  int64_t* ex = calloc((size_t)n, 8);
  int32_t* d = malloc(4 * (size_t)n);
  int32_t* q = malloc(4 * (size_t)n + 4);
  char* inq = calloc((size_t)n, 1);
  int32_t* fifo = malloc(4 * ((size_t)n + 1));
  int64_t* cur = malloc(8 * (size_t)n);
  int32_t* cnt = calloc(2 * (size_t)n + 2, 4);
  int64_t flow = -1;
  if (!ex || !d || !q || !inq || !fifo || !cur || !cnt) goto out;
  int32_t fh = 0, ft = 0, fsz = 0; /* circular FIFO of active vertices */
#define FPUSH(v)             \
  do {                       \
    fifo[ft] = (v);          \
    ft = (ft + 1) % (n + 1); \
    ++fsz;                   \
    inq[(v)] = 1;            \
  } while (0)
  for (int64_t a = g.first[s]; a < g.first[s + 1]; ++a) {
    int64_t c = g.res[a];
    if (c <= 0) continue;
    int32_t v = g.head[a];
    g.res[a] = 0;
    g.res[g.rev[a]] += c;
    ex[v] += c;
  }
  int64_t work = 0;
  const int64_t gr_every = (int64_t)n + g.na / 2;
  int need_gr = 1;
  for (;;) {
    if (need_gr) {
      /* exact distances to t over residual arcs; unreached -> n */
      for (int32_t i = 0; i < n; ++i) d[i] = n;
      memset(cnt, 0, (2 * (size_t)n + 2) * 4);
      int32_t qh = 0, qt = 0;
      d[t] = 0;
      q[qt++] = t;
      while (qh < qt) {
        int32_t v = q[qh++];
        for (int64_t a = g.first[v]; a < g.first[v + 1]; ++a) {
          int32_t u = g.head[a];
          if (d[u] == n && u != s && g.res[g.rev[a]] > 0) {
            d[u] = d[v] + 1;
            q[qt++] = u;
          }
        }
      }
      d[s] = n;
      for (int32_t i = 0; i < n; ++i) {
        if (d[i] < n) cnt[d[i]]++;
        cur[i] = g.first[i];
        inq[i] = 0;
      }
      fh = ft = fsz = 0;
      for (int32_t i = 0; i < n; ++i)
        if (i != s && i != t && ex[i] > 0 && d[i] < n) FPUSH(i);
      need_gr = 0;
      work = 0;
    }
    if (fsz == 0) break;
    int32_t u = fifo[fh];
    fh = (fh + 1) % (n + 1);
    --fsz;
    inq[u] = 0;
    if (d[u] >= n) continue;
    /* discharge u */
    while (ex[u] > 0) {
      int64_t a = cur[u];
      if (a == g.first[u + 1]) {
        /* relabel */
        int32_t old = d[u], mn = 2 * n;
        for (int64_t b = g.first[u]; b < g.first[u + 1]; ++b)
          if (g.res[b] > 0 && d[g.head[b]] + 1 < mn) mn = d[g.head[b]] + 1;
        work += 12 + (g.first[u + 1] - g.first[u]);
        cnt[old]--;
        if (mn >= n) mn = n;
        d[u] = mn;
        cur[u] = g.first[u];
        if (mn < n) cnt[mn]++;
        if (cnt[old] == 0 && old < n) {
          /* gap: everything above `old` is cut off from t */
          for (int32_t i = 0; i < n; ++i)
            if (d[i] > old && d[i] < n && i != s) {
              cnt[d[i]]--;
              d[i] = n;
            }
          d[u] = n;
        }
        if (d[u] >= n) break;
        continue;
      }
      int32_t v = g.head[a];
      if (g.res[a] > 0 && d[u] == d[v] + 1) {
        int64_t f = ex[u] < g.res[a] ? ex[u] : g.res[a];
        g.res[a] -= f;
        g.res[g.rev[a]] += f;
        ex[u] -= f;
        ex[v] += f;
        if (v != s && v != t && !inq[v]) FPUSH(v);
      } else {
        cur[u]++;
      }
    }
    if (work > gr_every) need_gr = 1;
  }
#undef FPUSH
  flow = ex[t];
out:
  free(ex);
  free(d);
  free(q);
  free(inq);
  free(fifo);
  free(cur);
  free(cnt);
  rg_free(&g);
  return flow;
}
