// `maxflow` command line: drop-in for the reference CLI
// (maxflow-cuda/src/main.cu:7-240).  Same options and the same two lines that
// scripts parse ("Total kernel time: X ms" and the maximum-flow line); every
// device operation goes through the C ABI in wbpr.h.
//
//   maxflow [-h] -v {0,1,2,3} -f file [-s src] [-t sink] [-a {0,1}]
//           [-l {rcsr,bcsr,bcsr16,bcsr2}] [-V] [-j] [-o solution] [-c cache]
//
// Added beyond the reference: -v 3 reads the library's graph cache (with
// capacities and terminals), -c writes the loaded graph to that cache, and
// -o writes the maximum flow as a DIMACS solution ("s" and "f" lines) after
// returning stranded excess to the source.
//
// As in the reference, -f loads the file with the -v given before it, and
// -s / -t are ignored for DIMACS input (the file names the terminals).
#include <getopt.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "wbpr.h"

static void usage(const char* prog) {
  printf("Usage: %s [-h] [-v file type] [-f filename] [-s source] [-t sink]\n", prog);
  printf("Options:\n");
  printf("\t-h\t\tShow this help message and exit\n");
  printf("\t-v\t\tSpecify which kind of file to load\n");
  printf("\t\t\t\t0: SNAP txt file (default)\n");
  printf("\t\t\t\t1: SNAP binary file\n");
  printf("\t\t\t\t2: DIMACS file\n");
  printf("\t\t\t\t3: graph cache written by -c (capacities and terminals kept)\n");
  printf("\t-f filename\tSpecify the file path (binary or txt)\n");
  printf("\t-s source\tSource node\n");
  printf("\t-t sink\t\tSink node\n");
  printf("\t-a algorithm\tSpecify the algorithm to use\n");
  printf("\t\t\t\t0: Thread-centric push-relabel (default)\n");
  printf("\t\t\t\t1: Vertex-centric push-relabel\n");
  printf("\t-l layout\tbcsr (default; also bcsr16), rcsr or bcsr2\n");
  printf("\t-V\t\tVerify the result on the device (capacity, conservation, cut)\n");
  printf("\t-j\t\tAlso print one JSON line with the solve statistics\n");
  printf("\t-o file\t\tWrite the maximum flow as a DIMACS solution (s / f lines)\n");
  printf("\t-c file\t\tWrite the loaded graph to a cache file for -v 3\n");
}

// Degree statistics in the reference's format (graph.cpp:618-683).
static void print_status(const wbpr_host_csr* g) {
  const int n = g->num_nodes;
  double sum = 0;
  int maxd = 0, maxv = 0, mind = n, minv = 0;
  for (int i = 0; i < n; ++i) {
    int d = g->offsets[i + 1] - g->offsets[i];
    sum += d;
    if (d > maxd) { maxd = d; maxv = i; }
    if (d < mind) { mind = d; minv = i; }
  }
  double avg = n ? sum / n : 0, sq = 0;
  for (int i = 0; i < n; ++i) {
    double d = g->offsets[i + 1] - g->offsets[i] - avg;
    sq += d * d;
  }
  printf("---------<< Graph Status >>---------\n");
  printf("Number of nodes: %d\n", n);
  printf("Number of edges: %lld\n", (long long)g->num_edges);
  printf("Average degree: %.2f\n", avg);
  printf("Standard deviation of degree: %.2f\n", n ? std::sqrt(sq / n) : 0.0);
  printf("Maximum degree: %d (Node %d)\n", maxd, maxv);
  printf("Minimum degree: %d (Node %d)\n", mind, minv);
  printf("Source node: %d, Sink node: %d\n", g->source, g->sink);
}

int main(int argc, char** argv) {
  int file_type = 0, algo = 0, source = -1, sink = -1;
  bool verify = false, json = false;
  const char* out_path = nullptr;
  const char* cache_path = nullptr;
  // BCSR16 by default: the same results as RCSR (the reference's only layout
  // in maxflow-cuda) and the general solver's fastest path
  wbpr_layout layout = WBPR_LAYOUT_BCSR;
  wbpr_host_csr* g = nullptr;
  int ch;
  while ((ch = getopt(argc, argv, "hv:f:s:t:a:l:Vjo:c:")) != -1) {
    switch (ch) {
      case 'h':
        usage(argv[0]);
        return 0;
      case 'v':
        file_type = atoi(optarg);
        break;
      case 'f': {
        wbpr_status st;
        if (g) wbpr_host_csr_free(g), g = nullptr;
        switch (file_type) {
          case 0:
            printf("Loading from txt file: %s\n", optarg);
            st = wbpr_read_snap_txt(optarg, &g);
            break;
          case 1:
            printf("Loading from binary file: %s\n", optarg);
            st = wbpr_read_snap_bin(optarg, &g);
            break;
          case 2:
            printf("Loading from DIMACS file: %s\n", optarg);
            st = wbpr_read_dimacs(optarg, &g);
            break;
          case 3:
            printf("Loading from graph cache: %s\n", optarg);
            st = wbpr_read_graph_cache(optarg, &g);
            break;
          default:
            printf("Invalid file type\n");
            return 1;
        }
        if (st != WBPR_OK) {
          fprintf(stderr, "Cannot load %s: %s\n", optarg, wbpr_status_str(st));
          return 1;
        }
        break;
      }
      case 's':
        if (file_type != 2) source = atoi(optarg);
        break;
      case 't':
        if (file_type != 2) sink = atoi(optarg);
        break;
      case 'o':
        out_path = optarg;
        break;
      case 'c':
        cache_path = optarg;
        break;
      case 'a':
        algo = atoi(optarg);
        break;
      case 'l':
        if (!strcmp(optarg, "rcsr")) layout = WBPR_LAYOUT_RCSR;
        else if (!strcmp(optarg, "bcsr") || !strcmp(optarg, "bcsr16")) layout = WBPR_LAYOUT_BCSR;
        else if (!strcmp(optarg, "bcsr2")) layout = WBPR_LAYOUT_BCSR2;
        else {
          printf("Invalid layout\n");
          return 1;
        }
        break;
      case 'V':
        verify = true;
        break;
      case 'j':
        json = true;
        break;
      default:
        printf("Invalid option\n");
        return 1;
    }
  }
  if (!g) {
    printf("No input file (-f)\n");
    return 1;
  }
  // DIMACS names its terminals; a cache keeps them unless -s / -t are given
  if (file_type != 2 && !(file_type == 3 && source < 0 && sink < 0)) {
    g->source = source;
    g->sink = sink;
  }
  if (g->source < 0 || g->sink < 0 || g->source >= g->num_nodes || g->sink >= g->num_nodes ||
      g->source == g->sink) {
    printf("Source(-s) and sink(-t) must be distinct vertices of the graph\n");
    wbpr_host_csr_free(g);
    return 1;
  }
  print_status(g);
  if (cache_path) {
    wbpr_csr cv{g->num_nodes, g->num_edges, g->offsets, g->destinations, g->capacities, g->source, g->sink};
    wbpr_status cs = wbpr_write_graph_cache(cache_path, &cv);
    if (cs != WBPR_OK) {
      fprintf(stderr, "Cannot write %s: %s\n", cache_path, wbpr_status_str(cs));
      wbpr_host_csr_free(g);
      return 1;
    }
  }
  if (algo == 0) printf("Using thread-centric push-relabel algorithm\n");
  else if (algo == 1) printf("Using vertex-centric push-relabel algorithm\n");
  else {
    printf("Invalid algorithm type\n");
    wbpr_host_csr_free(g);
    return 1;
  }
  wbpr_csr view{g->num_nodes, g->num_edges, g->offsets, g->destinations, g->capacities,
                g->source, g->sink};
  wbpr_graph* dg = nullptr;
  wbpr_status st = wbpr_graph_create(&view, layout, &dg);
  if (st != WBPR_OK) {
    fprintf(stderr, "wbpr_graph_create: %s\n", wbpr_status_str(st));
    wbpr_host_csr_free(g);
    return 1;
  }
  wbpr_tuning tu;
  wbpr_default_tuning(&tu);
  tu.verify = verify ? 1 : 0;
  wbpr_result res;
  st = wbpr_solve(dg, g->source, g->sink, algo == 0 ? WBPR_ALGO_TC : WBPR_ALGO_VC, &tu, &res);
  if (st != WBPR_OK) {
    fprintf(stderr, "wbpr_solve: %s\n", wbpr_status_str(st));
    wbpr_graph_destroy(dg);
    wbpr_host_csr_free(g);
    return 1;
  }
  printf("Total kernel time: %.6f ms\n", res.kernel_ms);
  printf("The maximum flow value of this flow network as calculated by the parallel "
         "implementation is %lld, %lld\n",
         (long long)res.flow, (long long)res.flow);
  if (verify) printf("Verification: passed (capacity, conservation, cut == flow)\n");
  if (json) {
    printf("{\"value\": %lld, \"solve_ms\": %.4f, \"kernel_ms\": %.4f, \"gr_ms\": %.4f, "
           "\"gr_share\": %.4f, \"rounds\": %d, \"global_relabels\": %d, \"arcs_scanned\": %llu, "
           "\"pushes\": %llu, \"relabels\": %llu, \"mteps\": %.3f, \"alg_bytes\": %llu, "
           "\"hbm_gbps\": %.1f}\n",
           (long long)res.flow, res.solve_ms, res.kernel_ms, res.gr_ms,
           res.solve_ms > 0 ? res.gr_ms / res.solve_ms : 0.0, res.rounds, res.global_relabels,
           (unsigned long long)res.arcs_scanned, (unsigned long long)res.pushes,
           (unsigned long long)res.relabels,
           res.solve_ms > 0 ? (double)g->num_edges / (res.solve_ms * 1e3) : 0.0,
           (unsigned long long)res.alg_bytes,
           res.launch_ms > 0 ? (double)res.alg_bytes / (res.launch_ms * 1e6) : 0.0);
  }
  int rc = 0;
  if (out_path) {
    int32_t* flow = (int32_t*)malloc(sizeof(int32_t) * (g->num_edges > 0 ? (size_t)g->num_edges : 1));
    st = flow ? wbpr_complete_flow(dg, nullptr) : WBPR_ERR_INVALID_ARG;
    if (st == WBPR_OK) st = wbpr_read_state(dg, nullptr, nullptr, flow);
    if (st == WBPR_OK) st = wbpr_write_dimacs_flow(out_path, &view, res.flow, flow);
    if (st != WBPR_OK) {
      fprintf(stderr, "Cannot write the solution to %s: %s\n", out_path, wbpr_status_str(st));
      rc = 1;
    }
    free(flow);
  }
  wbpr_graph_destroy(dg);
  wbpr_host_csr_free(g);
  return rc;
}
