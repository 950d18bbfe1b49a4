// Host side of libwbpr: graph readers and writers, seeded generators and the
// residual-graph builders.  Plain C++17, no CUDA.  Every generator draws from
// a counter-based splitmix64 stream and uses integer thresholds, so the same
// seed gives the same graph on x86-64 and aarch64 hosts and for any number of
// host threads.
#include <algorithm>
#include <atomic>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <new>
#include <system_error>
#include <thread>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "wbpr_internal.h"

namespace wbpr {

int host_threads() {
  unsigned hc = std::thread::hardware_concurrency();
  if (hc == 0) hc = 1;
  if (hc > 32) hc = 32;
  const char* env = std::getenv("WBPR_HOST_THREADS");
  if (env) {
    int v = std::atoi(env);
    if (v >= 1 && v <= 256) return v;
  }
  return (int)hc;
}

template <class F>
static void parallel_for(int64_t n, F&& f, int64_t grain = 1 << 16) {
  int T = host_threads();
  if (n < grain * 2 || T == 1) {
    f(0, n, 0);
    return;
  }
  int64_t chunks = std::min<int64_t>(T, (n + grain - 1) / grain);
  std::vector<std::thread> th;
  th.reserve(chunks);
  for (int64_t c = 0; c < chunks; ++c) {
    int64_t b = n * c / chunks, e = n * (c + 1) / chunks;
    th.emplace_back([&f, b, e, c] { f(b, e, (int)c); });
  }
  for (auto& x : th) x.join();
}

// ---------------------------------------------------------------------------
// splitmix64 (Steele, Lea, Flood 2014): one 64-bit state step and finalizer.
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
struct Stream {
  uint64_t x;
  explicit Stream(uint64_t seed, uint64_t a = 0, uint64_t b = 0)
      : x(mix64(seed ^ mix64(a * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL) ^
                mix64(b + 0xD1B54A32D192ED03ULL))) {}
  uint64_t next() {
    x += 0x9E3779B97F4A7C15ULL;
    return mix64(x);
  }
  // uniform integer in [lo, hi] (multiply-high, no modulo)
  int64_t range(int64_t lo, int64_t hi) {
    uint64_t span = (uint64_t)(hi - lo) + 1;
    return lo + (int64_t)(((unsigned __int128)next() * span) >> 64);
  }
  // uniform double in [0, 1) with 53 random bits
  double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ---------------------------------------------------------------------------
wbpr_status check_csr_shape(const wbpr_csr* g) {
  if (!g || g->num_nodes < 0 || g->num_edges < 0) return WBPR_ERR_INVALID_ARG;
  if (g->num_nodes > 0 && (!g->offsets)) return WBPR_ERR_INVALID_ARG;
  if (g->num_edges > 0 && !g->destinations) return WBPR_ERR_INVALID_ARG;
  if (g->num_edges > (int64_t)std::numeric_limits<int32_t>::max())
    return WBPR_ERR_OVERFLOW;
  const int32_t n = g->num_nodes;
  if (n == 0) return g->num_edges == 0 ? WBPR_OK : WBPR_ERR_INVALID_ARG;
  if (g->offsets[0] != 0 || (int64_t)g->offsets[n] != g->num_edges)
    return WBPR_ERR_INVALID_ARG;
  return WBPR_OK;
}

wbpr_status check_csr(const wbpr_csr* g) {
  if (!g || g->num_nodes < 0 || g->num_edges < 0) return WBPR_ERR_INVALID_ARG;
  if (g->num_nodes > 0 && (!g->offsets)) return WBPR_ERR_INVALID_ARG;
  if (g->num_edges > 0 && !g->destinations) return WBPR_ERR_INVALID_ARG;
  if (g->num_edges > (int64_t)std::numeric_limits<int32_t>::max())
    return WBPR_ERR_OVERFLOW;
  const int32_t n = g->num_nodes;
  if (n == 0) return g->num_edges == 0 ? WBPR_OK : WBPR_ERR_INVALID_ARG;
  if (g->offsets[0] != 0 || (int64_t)g->offsets[n] != g->num_edges)
    return WBPR_ERR_INVALID_ARG;
  for (int32_t u = 0; u < n; ++u)
    if (g->offsets[u + 1] < g->offsets[u]) return WBPR_ERR_INVALID_ARG;
  std::atomic<int> bad{0};
  parallel_for(g->num_edges, [&](int64_t b, int64_t e, int) {
    for (int64_t i = b; i < e; ++i) {
      int32_t v = g->destinations[i];
      if (v < 0 || v >= n) { bad = 1; return; }
      if (g->capacities && g->capacities[i] < 0) { bad = 1; return; }
    }
  });
  return bad ? WBPR_ERR_INVALID_ARG : WBPR_OK;
}

int64_t max_in_capacity(const wbpr_csr* g) {
  std::vector<int64_t> in((size_t)g->num_nodes, 0);
  for (int64_t i = 0; i < g->num_edges; ++i)
    in[g->destinations[i]] += g->capacities ? g->capacities[i] : 1;
  int64_t mx = 0;
  for (int64_t x : in) mx = std::max(mx, x);
  return mx;
}

wbpr_status to_host_csr(Csr&& c, wbpr_host_csr** out) {
  if (!out) return WBPR_ERR_INVALID_ARG;
  auto* h = (wbpr_host_csr*)std::calloc(1, sizeof(wbpr_host_csr));
  if (!h) return WBPR_ERR_INVALID_ARG;
  h->num_nodes = c.n;
  h->num_edges = c.m;
  h->num_edges_declared = c.m_declared;
  h->source = c.s;
  h->sink = c.t;
  h->offsets = (int32_t*)std::malloc(sizeof(int32_t) * ((size_t)c.n + 1));
  h->destinations = (int32_t*)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, c.m));
  h->capacities = (int32_t*)std::malloc(sizeof(int32_t) * std::max<int64_t>(1, c.m));
  if (!h->offsets || !h->destinations || !h->capacities) {
    wbpr_host_csr_free(h);
    return WBPR_ERR_INVALID_ARG;
  }
  std::memcpy(h->offsets, c.off.data(), sizeof(int32_t) * ((size_t)c.n + 1));
  if (c.m) {
    std::memcpy(h->destinations, c.dst.data(), sizeof(int32_t) * c.m);
    std::memcpy(h->capacities, c.cap.data(), sizeof(int32_t) * c.m);
  }
  *out = h;
  return WBPR_OK;
}

// ---------------------------------------------------------------------------
// File readers.  The file's bytes are mapped (read into memory when they
// cannot be) and parsed by hand; malformed or truncated input returns
// WBPR_ERR_IO instead of the reference's undefined behaviour.
namespace {
class FileBytes {
 public:
  FileBytes() = default;
  FileBytes(const FileBytes&) = delete;
  FileBytes& operator=(const FileBytes&) = delete;
  ~FileBytes() {
    if (map_) munmap(map_, len_);
  }
  // A regular file is mapped read-only (no copy, pages fault in on the
  // threads that parse them); anything else is read.
  bool open(const char* path) {
    if (!path) return false;
    const int fd = ::open(path, O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0) {
      void* q = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE, fd, 0);
      if (q != MAP_FAILED) {
        madvise(q, (size_t)st.st_size, MADV_WILLNEED);
        map_ = q;
        len_ = (size_t)st.st_size;
        ::close(fd);
        return true;
      }
    }
    std::string buf;
    char chunk[1 << 16];
    for (;;) {
      const ssize_t r = ::read(fd, chunk, sizeof(chunk));
      if (r < 0 && errno == EINTR) continue;
      if (r < 0) {
        ::close(fd);
        return false;
      }
      if (r == 0) break;
      buf.append(chunk, (size_t)r);
    }
    ::close(fd);
    own_.swap(buf);
    return true;
  }
  const char* data() const { return map_ ? (const char*)map_ : own_.data(); }
  size_t size() const { return map_ ? len_ : own_.size(); }

 private:
  void* map_ = nullptr;
  size_t len_ = 0;
  std::string own_;
};
}  // namespace

namespace {
struct Lines {
  const char* p;
  const char* end;
  bool next(const char** b, const char** e) {
    if (p >= end) return false;
    const char* q = p;
    while (q < end && *q != '\n') ++q;
    *b = p;
    *e = (q > p && q[-1] == '\r') ? q - 1 : q;
    p = q < end ? q + 1 : q;
    return true;
  }
};
// Parse a signed decimal integer; advances *p; false on no digits/overflow.
bool parse_int(const char** p, const char* e, int64_t* v) {
  const char* q = *p;
  while (q < e && (*q == ' ' || *q == '\t')) ++q;
  bool neg = false;
  if (q < e && (*q == '-' || *q == '+')) { neg = *q == '-'; ++q; }
  if (q >= e || *q < '0' || *q > '9') return false;
  int64_t x = 0;
  while (q < e && *q >= '0' && *q <= '9') {
    x = x * 10 + (*q - '0');
    if (x > (int64_t)1 << 40) return false;
    ++q;
  }
  *v = neg ? -x : x;
  *p = q;
  return true;
}
bool parse_word(const char** p, const char* e, const char** wb, const char** we) {
  const char* q = *p;
  while (q < e && (*q == ' ' || *q == '\t')) ++q;
  if (q >= e) return false;
  *wb = q;
  while (q < e && *q != ' ' && *q != '\t') ++q;
  *we = q;
  *p = q;
  return true;
}

// Group (u, v, c) triples into CSR, keeping per-row order of appearance
// (the reference's adjacency-list append order).
wbpr_status triples_to_csr(int32_t n, const std::vector<int32_t>& us,
                           const std::vector<int32_t>& vs,
                           const std::vector<int32_t>& cs, Csr* c) {
  c->n = n;
  c->m = (int64_t)us.size();
  c->off.assign((size_t)n + 1, 0);
  for (int32_t u : us) c->off[(size_t)u + 1]++;
  for (int32_t i = 0; i < n; ++i) c->off[i + 1] += c->off[i];
  c->dst.resize(us.size());
  c->cap.resize(us.size());
  std::vector<int32_t> cur(c->off.begin(), c->off.end() - 1);
  for (size_t k = 0; k < us.size(); ++k) {
    int32_t pos = cur[us[k]]++;
    c->dst[pos] = vs[k];
    c->cap[pos] = cs[k];
  }
  return WBPR_OK;
}

// Arcs parsed by one host thread from one piece of a file.
struct ArcPiece {
  std::vector<int32_t> us, vs, cs;  // cs left empty when every capacity is 1
  bool sorted = true;               // tails non-decreasing inside the piece
};

// Run f(k) for every piece k, piece 0 on the calling thread.
template <class F>
bool run_pieces(int P, F&& f) {
  try {
    std::vector<std::thread> th;
    for (int k = 1; k < P; ++k) th.emplace_back(f, k);
    if (P > 0) f(0);
    for (auto& x : th) x.join();
  } catch (const std::system_error&) {
    return false;
  }
  return true;
}

// Join pieces parsed in file order into c's CSR with n rows, keeping file
// order inside each row.  When the tails run non-decreasing through the whole
// file (the usual layout), every piece is copied straight into place by its
// own thread, which also writes the row offsets of the tails it starts
// (off[x] for previous tail < x <= tail); any other order goes through a
// counting sort.
wbpr_status pieces_to_csr(int64_t n, std::vector<ArcPiece>& pc, Csr* c) {
  const int P = (int)pc.size();
  size_t total = 0;
  bool sorted = true;
  int32_t prev_last = -1;
  std::vector<size_t> at((size_t)P + 1, 0);
  std::vector<int32_t> tail_before((size_t)P, -1);  // tail of the arc before each piece
  for (int k = 0; k < P; ++k) {
    const ArcPiece& q = pc[(size_t)k];
    at[(size_t)k] = total;
    tail_before[(size_t)k] = prev_last;
    total += q.us.size();
    if (!q.sorted || (!q.us.empty() && q.us.front() < prev_last)) sorted = false;
    if (!q.us.empty()) prev_last = q.us.back();
  }
  at[(size_t)P] = total;
  if (total > (size_t)std::numeric_limits<int32_t>::max()) return WBPR_ERR_OVERFLOW;
  if (sorted) {
    c->n = (int32_t)n;
    c->m = (int64_t)total;
    c->off.assign((size_t)n + 1, 0);
    c->dst.resize(total);
    c->cap.resize(total);
    auto place = [&](int k) {
      const ArcPiece& q = pc[(size_t)k];
      const size_t base = at[(size_t)k];
      std::copy(q.vs.begin(), q.vs.end(), c->dst.begin() + (std::ptrdiff_t)base);
      if (q.cs.empty())
        std::fill(c->cap.begin() + (std::ptrdiff_t)base, c->cap.begin() + (std::ptrdiff_t)(base + q.vs.size()), 1);
      else
        std::copy(q.cs.begin(), q.cs.end(), c->cap.begin() + (std::ptrdiff_t)base);
      int32_t prev = tail_before[(size_t)k];
      for (size_t j = 0; j < q.us.size(); ++j) {
        const int32_t u = q.us[j];
        for (int32_t x = prev + 1; x <= u; ++x) c->off[(size_t)x] = (int32_t)(base + j);
        prev = u;
      }
    };
    if (!run_pieces(P, place)) return WBPR_ERR_IO;
    for (int64_t x = (int64_t)prev_last + 1; x <= n; ++x) c->off[(size_t)x] = (int32_t)total;
    return WBPR_OK;
  }
  std::vector<int32_t> us(total), vs(total), cs(total);
  auto join = [&](int k) {
    ArcPiece& q = pc[(size_t)k];
    const std::ptrdiff_t base = (std::ptrdiff_t)at[(size_t)k];
    std::copy(q.us.begin(), q.us.end(), us.begin() + base);
    std::copy(q.vs.begin(), q.vs.end(), vs.begin() + base);
    if (q.cs.empty())
      std::fill(cs.begin() + base, cs.begin() + base + (std::ptrdiff_t)q.us.size(), 1);
    else
      std::copy(q.cs.begin(), q.cs.end(), cs.begin() + base);
  };
  if (!run_pieces(P, join)) return WBPR_ERR_IO;
  std::vector<ArcPiece>().swap(pc);
  return triples_to_csr((int32_t)n, us, vs, cs, c);
}
}  // namespace

// Split [b, e) into up to T pieces that start at line starts.
static std::vector<const char*> line_splits(const char* b, const char* e, int T) {
  std::vector<const char*> cut{b};
  const size_t len = (size_t)(e - b);
  for (int k = 1; k < T; ++k) {
    const char* q = b + len * k / T;
    if (q <= cut.back()) continue;
    while (q < e && q[-1] != '\n') ++q;
    if (q > cut.back() && q < e) cut.push_back(q);
  }
  cut.push_back(e);
  return cut;
}

// -v 2 : DIMACS max-flow (reference graph.cpp:151-214).  1-based ids are
// shifted to 0-based; "n ID s" / "n ID t" set the terminals (the last one of
// each kind counts); arcs keep file order inside each tail row.  The header
// ("c", "p", "n" lines up to the first arc) is read in order; the arc lines
// are parsed by all host threads, each over a piece of the file that starts
// at a line start, and joined in file order.
wbpr_status read_dimacs(const char* path, Csr* c) {
  FileBytes buf;
  if (!buf.open(path)) return WBPR_ERR_IO;
  Lines L{buf.data(), buf.data() + buf.size()};
  const char *b, *e;
  int64_t n = -1, mdecl = -1;
  int32_t s = -1, t = -1;
  auto parse_n = [&](const char* p, const char* e2, int32_t* ss, int32_t* tt) {
    int64_t id;
    const char *wb, *we;
    if (n < 0 || !parse_int(&p, e2, &id) || !parse_word(&p, e2, &wb, &we)) return false;
    if (id < 1 || id > n) return false;
    if (*wb == 's') *ss = (int32_t)(id - 1);
    else if (*wb == 't') *tt = (int32_t)(id - 1);
    return true;
  };
  const char* arcs_from = buf.data() + buf.size();
  while (L.next(&b, &e)) {
    const char* p = b;
    while (p < e && (*p == ' ' || *p == '\t')) ++p;
    if (p >= e || *p == 'c') continue;
    char kind = *p++;
    if (kind == 'p') {
      const char *wb, *we;
      if (!parse_word(&p, e, &wb, &we)) return WBPR_ERR_IO;
      if (!parse_int(&p, e, &n) || !parse_int(&p, e, &mdecl)) return WBPR_ERR_IO;
      if (n <= 0 || n > std::numeric_limits<int32_t>::max() - 2 || mdecl < 0) return WBPR_ERR_IO;
    } else if (kind == 'n') {
      if (!parse_n(p, e, &s, &t)) return WBPR_ERR_IO;
    } else if (kind == 'a') {
      if (n < 0) return WBPR_ERR_IO;
      arcs_from = b;
      break;
    } else {
      return WBPR_ERR_IO;
    }
  }
  if (n < 0) return WBPR_ERR_IO;
  const std::vector<const char*> cut = line_splits(arcs_from, buf.data() + buf.size(), host_threads());
  const int P = (int)cut.size() - 1;
  struct Piece {
    int32_t s = -1, t = -1;
    bool bad = false;
  };
  std::vector<Piece> pc((size_t)std::max(P, 0));
  std::vector<ArcPiece> arcs((size_t)std::max(P, 0));
  // One pass per line: "a u v c" lines are parsed where they stand (a newline
  // is neither blank nor a digit, so a short line fails its own parse);
  // comment lines are skipped to their newline.
  auto work = [&](int k) {
    Piece& q = pc[(size_t)k];
    ArcPiece& a = arcs[(size_t)k];
    const size_t guess = (size_t)((cut[k + 1] - cut[k]) / 12 + 16);
    a.us.reserve(guess);
    a.vs.reserve(guess);
    a.cs.reserve(guess);
    const char* p = cut[k];
    const char* const end = cut[k + 1];
    auto to_next_line = [&]() {
      const void* nl = std::memchr(p, '\n', (size_t)(end - p));
      p = nl ? (const char*)nl + 1 : end;
    };
    int32_t last = -1;
    while (p < end) {
      while (p < end && (*p == ' ' || *p == '\t')) ++p;
      if (p >= end) break;
      const char kind = *p;
      if (kind == '\n' || (kind == '\r' && (p + 1 == end || p[1] == '\n')) || kind == 'c') {
        to_next_line();
        continue;
      }
      ++p;
      if (kind == 'a') {
        int64_t u, v, cap;
        if (!parse_int(&p, end, &u) || !parse_int(&p, end, &v) || !parse_int(&p, end, &cap) || u < 1 || u > n ||
            v < 1 || v > n || cap < 0 || cap > std::numeric_limits<int32_t>::max()) {
          q.bad = true;
          return;
        }
        const int32_t tu = (int32_t)(u - 1);
        if (tu < last) a.sorted = false;
        last = tu;
        a.us.push_back(tu);
        a.vs.push_back((int32_t)(v - 1));
        a.cs.push_back((int32_t)cap);
        to_next_line();  // the rest of the line is ignored
      } else if (kind == 'n') {
        const char* le = (const char*)std::memchr(p, '\n', (size_t)(end - p));
        if (!le) le = end;
        if (le > p && le[-1] == '\r') --le;
        if (!parse_n(p, le, &q.s, &q.t)) {
          q.bad = true;
          return;
        }
        p = le;
        to_next_line();
      } else {
        q.bad = true;  // a second problem line or an unknown line kind
        return;
      }
    }
  };
  if (!run_pieces(P, work)) return WBPR_ERR_IO;
  for (const Piece& q : pc) {
    if (q.bad) return WBPR_ERR_IO;
    if (q.s >= 0) s = q.s;
    if (q.t >= 0) t = q.t;
  }
  const wbpr_status st = pieces_to_csr(n, arcs, c);
  if (st) return st;
  c->m_declared = mdecl;
  c->s = s;
  c->t = t;
  return WBPR_OK;
}

// -v 0 : SNAP text (reference graph.cpp:28-67).  "# Nodes: N Edges: M" gives
// n (the last such header counts); other '#' lines are comments; every row is
// sorted by head; capacity 1.  Without the header, n = 1 + largest id seen.
// Parsed like DIMACS: one piece of the file per host thread, one pass per
// line, headers searched within their own line only.
wbpr_status read_snap_txt(const char* path, Csr* c) {
  FileBytes buf;
  if (!buf.open(path)) return WBPR_ERR_IO;
  const char* const data = buf.data();
  const std::vector<const char*> cut = line_splits(data, data + buf.size(), host_threads());
  const int P = (int)cut.size() - 1;
  struct Piece {
    int64_t n = -1, mdecl = -1;  // the piece's last "# Nodes: N Edges: M" header
    int64_t maxid = -1;
    bool bad = false;
  };
  std::vector<Piece> pc((size_t)std::max(P, 0));
  std::vector<ArcPiece> arcs((size_t)std::max(P, 0));
  static const char kNodes[] = "Nodes:";
  static const char kEdges[] = "Edges:";
  constexpr int32_t kMaxId = std::numeric_limits<int32_t>::max() - 2;
  auto work = [&](int k) {
    Piece& q = pc[(size_t)k];
    ArcPiece& a = arcs[(size_t)k];
    const size_t guess = (size_t)((cut[k + 1] - cut[k]) / 10 + 16);
    a.us.reserve(guess);
    a.vs.reserve(guess);
    const char* p = cut[k];
    const char* const end = cut[k + 1];
    auto to_next_line = [&]() {
      const void* nl = std::memchr(p, '\n', (size_t)(end - p));
      p = nl ? (const char*)nl + 1 : end;
    };
    int32_t last = -1;
    while (p < end) {
      while (p < end && (*p == ' ' || *p == '\t')) ++p;
      if (p >= end) break;
      const char ch = *p;
      if (ch == '\n' || (ch == '\r' && (p + 1 == end || p[1] == '\n'))) {
        to_next_line();
        continue;
      }
      if (ch == '#') {
        const char* le = (const char*)std::memchr(p, '\n', (size_t)(end - p));
        if (!le) le = end;
        if (le > p && le[-1] == '\r') --le;
        const char* kn = std::search(p, le, kNodes, kNodes + 6);
        if (kn != le) {
          const char* r = kn + 6;
          int64_t nn, mm;
          if (!parse_int(&r, le, &nn)) {
            q.bad = true;
            return;
          }
          const char* ke = std::search(r, le, kEdges, kEdges + 6);
          if (ke == le) {
            q.bad = true;
            return;
          }
          r = ke + 6;
          if (!parse_int(&r, le, &mm) || nn <= 0 || nn > kMaxId) {
            q.bad = true;
            return;
          }
          q.n = nn;
          q.mdecl = mm;
        }
        p = le;
        to_next_line();
        continue;
      }
      int64_t u, v;
      if (!parse_int(&p, end, &u) || !parse_int(&p, end, &v) || u < 0 || v < 0 || u > kMaxId || v > kMaxId) {
        q.bad = true;
        return;
      }
      q.maxid = std::max(q.maxid, std::max(u, v));
      if ((int32_t)u < last) a.sorted = false;
      last = (int32_t)u;
      a.us.push_back((int32_t)u);
      a.vs.push_back((int32_t)v);
      to_next_line();  // the rest of the line is ignored
    }
  };
  if (!run_pieces(P, work)) return WBPR_ERR_IO;
  int64_t n = -1, mdecl = -1, maxid = -1;
  for (const Piece& q : pc) {
    if (q.bad) return WBPR_ERR_IO;
    if (q.n >= 0) {
      n = q.n;
      mdecl = q.mdecl;
    }
    maxid = std::max(maxid, q.maxid);
  }
  if (n < 0) n = maxid + 1;
  if (n <= 0) return WBPR_ERR_IO;
  if (maxid >= n) return WBPR_ERR_IO;
  const wbpr_status st = pieces_to_csr(n, arcs, c);
  if (st) return st;
  parallel_for(c->n, [&](int64_t lo, int64_t hi, int) {
    for (int64_t u = lo; u < hi; ++u) {
      const auto b = c->dst.begin() + c->off[(size_t)u], e = c->dst.begin() + c->off[(size_t)u + 1];
      if (!std::is_sorted(b, e)) std::sort(b, e);
    }
  });
  c->m_declared = mdecl < 0 ? c->m : mdecl;
  return WBPR_OK;
}

// -v 1 : SNAP binary (reference graph.cpp:219-233 writer, 292-314 reader):
// int32 n, m, m_processed, destinations[m_processed], offsets[n+1]; cap 1.
wbpr_status read_snap_bin(const char* path, Csr* c) {
  FileBytes buf;
  if (!buf.open(path)) return WBPR_ERR_IO;
  if (buf.size() < 12) return WBPR_ERR_IO;
  int32_t hdr[3];
  std::memcpy(hdr, buf.data(), 12);
  int32_t n = hdr[0], mdecl = hdr[1], mp = hdr[2];
  if (n <= 0 || mp < 0) return WBPR_ERR_IO;
  size_t need = 12 + 4 * ((size_t)mp + (size_t)n + 1);
  if (buf.size() < need) return WBPR_ERR_IO;
  c->n = n;
  c->m = mp;
  c->m_declared = mdecl;
  c->dst.resize((size_t)mp);
  c->off.resize((size_t)n + 1);
  std::memcpy(c->dst.data(), buf.data() + 12, 4 * (size_t)mp);
  std::memcpy(c->off.data(), buf.data() + 12 + 4 * (size_t)mp, 4 * ((size_t)n + 1));
  c->cap.assign((size_t)mp, 1);
  wbpr_csr view{c->n, c->m, c->off.data(), c->dst.data(), c->cap.data(), -1, -1};
  if (check_csr(&view) != WBPR_OK) return WBPR_ERR_IO;
  return WBPR_OK;
}

// Graph cache (new; the reference's .bin has no capacities and no
// terminals): "WBPRCSR1", int32 version 1, int32 flags (bit 0: capacities
// present), int64 n, int64 m, int64 m_declared, int32 s, int32 t, then int32
// offsets[n+1], destinations[m] and, with bit 0, capacities[m]; little endian.
constexpr char kCacheMagic[8] = {'W', 'B', 'P', 'R', 'C', 'S', 'R', '1'};
struct CacheHeader {
  char magic[8];
  int32_t version;
  int32_t flags;
  int64_t n, m, m_declared;
  int32_t s, t;
};
static_assert(sizeof(CacheHeader) == 48, "cache header layout");

wbpr_status read_graph_cache(const char* path, Csr* c) {
  FileBytes buf;
  if (!buf.open(path)) return WBPR_ERR_IO;
  CacheHeader h;
  if (buf.size() < sizeof(h)) return WBPR_ERR_IO;
  std::memcpy(&h, buf.data(), sizeof(h));
  if (std::memcmp(h.magic, kCacheMagic, 8) != 0 || h.version != 1) return WBPR_ERR_IO;
  if (h.n < 1 || h.n > std::numeric_limits<int32_t>::max() - 2 || h.m < 0 ||
      h.m > std::numeric_limits<int32_t>::max())
    return WBPR_ERR_IO;
  const bool caps = h.flags & 1;
  const size_t need = sizeof(h) + 4 * ((size_t)h.n + 1 + (size_t)h.m * (caps ? 2 : 1));
  if (buf.size() != need) return WBPR_ERR_IO;
  c->n = (int32_t)h.n;
  c->m = h.m;
  c->m_declared = h.m_declared;
  c->s = h.s;
  c->t = h.t;
  const char* p = buf.data() + sizeof(h);
  c->off.resize((size_t)h.n + 1);
  std::memcpy(c->off.data(), p, 4 * ((size_t)h.n + 1));
  p += 4 * ((size_t)h.n + 1);
  c->dst.resize((size_t)h.m);
  std::memcpy(c->dst.data(), p, 4 * (size_t)h.m);
  p += 4 * (size_t)h.m;
  if (caps) {
    c->cap.resize((size_t)h.m);
    std::memcpy(c->cap.data(), p, 4 * (size_t)h.m);
  } else {
    c->cap.assign((size_t)h.m, 1);
  }
  if ((c->s < -1 || c->s >= c->n) || (c->t < -1 || c->t >= c->n)) return WBPR_ERR_IO;
  wbpr_csr view{c->n, c->m, c->off.data(), c->dst.data(), c->cap.data(), c->s, c->t};
  return check_csr(&view) == WBPR_OK ? WBPR_OK : WBPR_ERR_IO;
}

// ---------------------------------------------------------------------------
// Parallel LSD radix sort of 64-bit keys on the low `bits` bits.
static void radix_sort_u64(std::vector<uint64_t>& a, int bits) {
  std::vector<uint64_t> tmp(a.size());
  const int T = host_threads();
  const int64_t N = (int64_t)a.size();
  for (int shift = 0; shift < bits; shift += 8) {
    std::vector<std::vector<int64_t>> hist(T, std::vector<int64_t>(256, 0));
    auto range = [&](int k, int64_t* b, int64_t* e) {
      *b = N * k / T;
      *e = N * (k + 1) / T;
    };
    {
      std::vector<std::thread> th;
      for (int k = 0; k < T; ++k)
        th.emplace_back([&, k] {
          int64_t b, e;
          range(k, &b, &e);
          auto& h = hist[k];
          for (int64_t i = b; i < e; ++i) h[(a[i] >> shift) & 255]++;
        });
      for (auto& x : th) x.join();
    }
    int64_t base = 0;
    for (int d = 0; d < 256; ++d)
      for (int k = 0; k < T; ++k) {
        int64_t c = hist[k][d];
        hist[k][d] = base;
        base += c;
      }
    {
      std::vector<std::thread> th;
      for (int k = 0; k < T; ++k)
        th.emplace_back([&, k] {
          int64_t b, e;
          range(k, &b, &e);
          auto& h = hist[k];
          for (int64_t i = b; i < e; ++i) tmp[h[(a[i] >> shift) & 255]++] = a[i];
        });
      for (auto& x : th) x.join();
    }
    a.swap(tmp);
  }
}

// Sorted unique (u << 32 | v) keys -> CSR with capacities from a stream
// keyed by the final arc index.
static void keys_to_csr(int32_t n, const std::vector<uint64_t>& keys, int32_t cap_lo,
                        int32_t cap_hi, uint64_t seed, Csr* c) {
  c->n = n;
  c->m = (int64_t)keys.size();
  c->m_declared = c->m;
  c->off.assign((size_t)n + 1, 0);
  c->dst.resize(keys.size());
  c->cap.resize(keys.size());
  for (uint64_t k : keys) c->off[(size_t)(k >> 32) + 1]++;
  for (int32_t i = 0; i < n; ++i) c->off[i + 1] += c->off[i];
  parallel_for((int64_t)keys.size(), [&](int64_t b, int64_t e, int) {
    for (int64_t i = b; i < e; ++i) {
      c->dst[i] = (int32_t)(keys[i] & 0xffffffffu);
      Stream r(seed, 0xCA9ULL, (uint64_t)i);
      c->cap[i] = (int32_t)r.range(cap_lo, cap_hi);
    }
  });
}

// ---------------------------------------------------------------------------
// Generators.
wbpr_status gen_genrmf(int32_t a, int32_t b, int32_t c1, int32_t c2, uint64_t seed, Csr* c) {
  if (a < 1 || b < 1 || c1 < 0 || c2 < c1) return WBPR_ERR_INVALID_ARG;
  int64_t A2 = (int64_t)a * a;
  int64_t n = A2 * b;
  if (n > std::numeric_limits<int32_t>::max() / 8) return WBPR_ERR_OVERFLOW;
  if ((int64_t)c2 * A2 > std::numeric_limits<int32_t>::max()) return WBPR_ERR_OVERFLOW;
  const int32_t incap = (int32_t)(c2 * A2);
  // one seeded Fisher-Yates permutation per frame boundary
  std::vector<int32_t> perm((size_t)A2);
  c->n = (int32_t)n;
  c->off.assign((size_t)n + 1, 0);
  c->dst.clear();
  c->cap.clear();
  c->dst.reserve((size_t)(n * 5));
  c->cap.reserve((size_t)(n * 5));
  for (int32_t z = 0; z < b; ++z) {
    if (z < b - 1) {
      for (int64_t i = 0; i < A2; ++i) perm[i] = (int32_t)i;
      Stream r(seed, 0x5EED0001ULL, (uint64_t)z);
      for (int64_t i = A2 - 1; i > 0; --i) std::swap(perm[i], perm[r.range(0, i)]);
    }
    Stream rc(seed, 0x5EED0002ULL, (uint64_t)z);
    int64_t base = A2 * z;
    for (int32_t x = 0; x < a; ++x)
      for (int32_t y = 0; y < a; ++y) {
        int64_t loc = (int64_t)x * a + y;
        int64_t v = base + loc;
        if (z < b - 1) {
          c->dst.push_back((int32_t)(base + A2 + perm[loc]));
          c->cap.push_back((int32_t)rc.range(c1, c2));
        }
        const int dx[4] = {0, 0, 1, -1}, dy[4] = {1, -1, 0, 0};
        for (int k = 0; k < 4; ++k) {
          int32_t nx = x + dx[k], ny = y + dy[k];
          if (nx < 0 || ny < 0 || nx >= a || ny >= a) continue;
          c->dst.push_back((int32_t)(base + (int64_t)nx * a + ny));
          c->cap.push_back(incap);
        }
        c->off[(size_t)v + 1] = (int32_t)c->dst.size();
      }
  }
  c->m = (int64_t)c->dst.size();
  c->m_declared = c->m;
  c->s = 0;
  c->t = (int32_t)(n - 1);
  return WBPR_OK;
}

wbpr_status gen_rmat(int32_t scale, int32_t ef, double pa, double pb, double pc, int32_t cap_lo,
                     int32_t cap_hi, uint64_t seed, Csr* c) {
  if (scale < 1 || scale > 30 || ef < 1 || cap_lo < 0 || cap_hi < cap_lo) return WBPR_ERR_INVALID_ARG;
  if (pa < 0 || pb < 0 || pc < 0 || pa + pb + pc > 1.0) return WBPR_ERR_INVALID_ARG;
  const int64_t n = (int64_t)1 << scale;
  const int64_t M = n * ef;
  if (M > ((int64_t)1 << 31) - 1) return WBPR_ERR_OVERFLOW;
  // integer quadrant thresholds on 32-bit draws
  const uint64_t TA = (uint64_t)std::floor(pa * 4294967296.0);
  const uint64_t TB = (uint64_t)std::floor((pa + pb) * 4294967296.0);
  const uint64_t TC = (uint64_t)std::floor((pa + pb + pc) * 4294967296.0);
  std::vector<uint64_t> keys((size_t)M);
  parallel_for(M, [&](int64_t b, int64_t e, int) {
    for (int64_t k = b; k < e; ++k) {
      Stream r(seed, 0x4D41ULL, (uint64_t)k);
      uint64_t u = 0, v = 0, w = 0;
      for (int lvl = 0; lvl < scale; ++lvl) {
        if ((lvl & 1) == 0) w = r.next();
        uint64_t x = (lvl & 1) ? (w >> 32) : (w & 0xffffffffu);
        uint64_t bit = (uint64_t)1 << (scale - 1 - lvl);
        if (x >= TB) u |= bit;                      // quadrants c, d
        if ((x >= TA && x < TB) || x >= TC) v |= bit;  // quadrants b, d
      }
      keys[k] = (u << 32) | v;
    }
  });
  radix_sort_u64(keys, 32 + scale);
  // drop self loops and duplicates
  int64_t w = 0;
  for (int64_t i = 0; i < M; ++i) {
    uint64_t k = keys[i];
    if ((k >> 32) == (k & 0xffffffffu)) continue;
    if (w > 0 && keys[w - 1] == k) continue;
    keys[w++] = k;
  }
  keys.resize((size_t)w);
  keys_to_csr((int32_t)n, keys, cap_lo, cap_hi, seed, c);
  // terminals: max out-degree and max in-degree (lowest id on ties)
  std::vector<int32_t> indeg((size_t)n, 0);
  for (int32_t v : c->dst) indeg[v]++;
  int32_t s = 0, t = -1;
  for (int32_t u = 1; u < (int32_t)n; ++u)
    if (c->off[u + 1] - c->off[u] > c->off[s + 1] - c->off[s]) s = u;
  for (int32_t u = 0; u < (int32_t)n; ++u)
    if (u != s && (t < 0 || indeg[u] > indeg[t])) t = u;
  c->s = s;
  c->t = t;
  return WBPR_OK;
}

wbpr_status gen_bipartite(int32_t L, int32_t R, double zs, int32_t dmax, uint64_t seed, Csr* c) {
  if (L < 1 || R < 1 || dmax < 1 || zs <= 0) return WBPR_ERR_INVALID_ARG;
  if ((int64_t)L + R + 2 > std::numeric_limits<int32_t>::max() / 2) return WBPR_ERR_OVERFLOW;
  dmax = std::min(dmax, R);
  // Zipf CDF over 1..dmax by plain sums (no libm beyond pow on exact ints)
  std::vector<double> cdf((size_t)dmax);
  double acc = 0;
  for (int32_t k = 1; k <= dmax; ++k) {
    double w = (zs == 2.0) ? 1.0 / ((double)k * (double)k) : 1.0 / std::pow((double)k, zs);
    acc += w;
    cdf[k - 1] = acc;
  }
  const int32_t n = L + R + 2, s = 0, t = L + R + 1;
  std::vector<std::vector<int32_t>> rows((size_t)L);
  parallel_for(L, [&](int64_t b, int64_t e, int) {
    for (int64_t l = b; l < e; ++l) {
      Stream r(seed, 0xB1ULL, (uint64_t)l);
      double u = r.unit() * acc;
      int32_t d = (int32_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) + 1;
      if (d > dmax) d = dmax;
      auto& row = rows[l];
      row.resize((size_t)d);
      for (int32_t k = 0; k < d; ++k) row[k] = L + 1 + (int32_t)r.range(0, R - 1);
      std::sort(row.begin(), row.end());
      row.erase(std::unique(row.begin(), row.end()), row.end());
    }
  }, 4096);
  c->n = n;
  c->off.assign((size_t)n + 1, 0);
  c->dst.clear();
  c->cap.clear();
  for (int32_t l = 1; l <= L; ++l) c->dst.push_back(l);
  c->off[1] = L;
  for (int32_t l = 0; l < L; ++l) {
    for (int32_t v : rows[l]) c->dst.push_back(v);
    c->off[l + 2] = (int32_t)c->dst.size();
  }
  for (int32_t r = 0; r < R; ++r) {
    c->dst.push_back(t);
    c->off[L + 2 + r] = (int32_t)c->dst.size();
  }
  c->off[n] = (int32_t)c->dst.size();
  c->m = (int64_t)c->dst.size();
  c->m_declared = c->m;
  c->cap.assign(c->dst.size(), 1);
  c->s = s;
  c->t = t;
  return WBPR_OK;
}

wbpr_status gen_layered(int32_t layers, int32_t width, int32_t dlo, int32_t dhi, int32_t clo,
                        int32_t chi, uint64_t seed, Csr* c) {
  if (layers < 1 || width < 1 || dlo < 1 || dhi < dlo || clo < 0 || chi < clo)
    return WBPR_ERR_INVALID_ARG;
  int64_t n64 = (int64_t)layers * width + 2;
  if (n64 > std::numeric_limits<int32_t>::max() / 8) return WBPR_ERR_OVERFLOW;
  const int32_t n = (int32_t)n64, s = 0, t = n - 1;
  c->n = n;
  c->off.assign((size_t)n + 1, 0);
  c->dst.clear();
  c->cap.clear();
  Stream rs(seed, 0x1A0ULL, 0);
  for (int32_t j = 0; j < width; ++j) {
    c->dst.push_back(1 + j);
    c->cap.push_back((int32_t)rs.range(clo, chi));
  }
  c->off[1] = (int32_t)c->dst.size();
  std::vector<int32_t> tmp;
  for (int32_t i = 0; i < layers; ++i)
    for (int32_t j = 0; j < width; ++j) {
      int32_t v = 1 + i * width + j;
      Stream r(seed, 0x1A1ULL, (uint64_t)v);
      if (i == layers - 1) {
        c->dst.push_back(t);
        c->cap.push_back((int32_t)r.range(clo, chi));
      } else {
        int32_t d = (int32_t)std::min<int64_t>(r.range(dlo, dhi), width);
        tmp.clear();
        for (int32_t k = 0; k < d; ++k) tmp.push_back(1 + (i + 1) * width + (int32_t)r.range(0, width - 1));
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        for (int32_t x : tmp) {
          c->dst.push_back(x);
          c->cap.push_back((int32_t)r.range(clo, chi));
        }
      }
      c->off[(size_t)v + 1] = (int32_t)c->dst.size();
    }
  c->off[(size_t)n] = (int32_t)c->dst.size();
  c->m = (int64_t)c->dst.size();
  c->m_declared = c->m;
  c->s = s;
  c->t = t;
  return WBPR_OK;
}

// Vision graph-cut grid.  field = seeded noise (Irwin-Hall sum of 12
// uniforms, a unit-variance Gaussian stand-in) blurred with a sigma = 4
// Gaussian and scaled to [0, 1].  n-link cap = round(1000 exp(-d^2 / 0.02)),
// d = field difference; t-links round(1000 u), round(1000 (1 - u)),
// u = clip(field + 0.2 * noise, 0, 1).
wbpr_status gen_grid(int32_t w, int32_t h, uint64_t seed, Csr* c) {
  if (w < 2 || h < 2) return WBPR_ERR_INVALID_ARG;
  int64_t P = (int64_t)w * h;
  if (P + 2 > std::numeric_limits<int32_t>::max() / 8) return WBPR_ERR_OVERFLOW;
  auto gauss = [&](uint64_t tag, uint64_t i) {
    Stream r(seed, tag, i);
    double acc = 0;
    for (int k = 0; k < 12; ++k) acc += r.unit();
    return acc - 6.0;
  };
  std::vector<double> f((size_t)P), g((size_t)P);
  for (int64_t i = 0; i < P; ++i) f[i] = gauss(0x6A1ULL, (uint64_t)i);
  const int R = 12;
  double kw[2 * R + 1], ks = 0;
  for (int k = -R; k <= R; ++k) ks += (kw[k + R] = std::exp(-(double)(k * k) / (2.0 * 16.0)));
  for (int k = 0; k <= 2 * R; ++k) kw[k] /= ks;
  for (int32_t y = 0; y < h; ++y)
    for (int32_t x = 0; x < w; ++x) {
      double a = 0;
      for (int k = -R; k <= R; ++k) {
        int32_t xx = std::min(std::max(x + k, 0), w - 1);
        a += kw[k + R] * f[(int64_t)y * w + xx];
      }
      g[(int64_t)y * w + x] = a;
    }
  for (int32_t y = 0; y < h; ++y)
    for (int32_t x = 0; x < w; ++x) {
      double a = 0;
      for (int k = -R; k <= R; ++k) {
        int32_t yy = std::min(std::max(y + k, 0), h - 1);
        a += kw[k + R] * g[(int64_t)yy * w + x];
      }
      f[(int64_t)y * w + x] = a;
    }
  double lo = f[0], hi = f[0];
  for (double v : f) { lo = std::min(lo, v); hi = std::max(hi, v); }
  double span = hi > lo ? hi - lo : 1.0;
  for (double& v : f) v = (v - lo) / span;
  const int32_t n = (int32_t)(P + 2), s = (int32_t)P, t = (int32_t)P + 1;
  auto ncap = [&](int64_t p, int64_t q) {
    double d = f[p] - f[q];
    return (int32_t)std::lround(1000.0 * std::exp(-d * d / 0.02));
  };
  // arc lists: pixel rows hold n-links (right, left, down, up) then p->t
  c->n = n;
  c->off.assign((size_t)n + 1, 0);
  c->dst.clear();
  c->cap.clear();
  std::vector<int32_t> tcap((size_t)P), scap((size_t)P);
  for (int64_t p = 0; p < P; ++p) {
    double u = f[p] + 0.2 * gauss(0x6A2ULL, (uint64_t)p);
    u = std::min(1.0, std::max(0.0, u));
    scap[p] = (int32_t)std::lround(1000.0 * u);
    tcap[p] = (int32_t)std::lround(1000.0 * (1.0 - u));
  }
  for (int32_t y = 0; y < h; ++y)
    for (int32_t x = 0; x < w; ++x) {
      int64_t p = (int64_t)y * w + x;
      const int dx[4] = {1, -1, 0, 0}, dy[4] = {0, 0, 1, -1};
      for (int k = 0; k < 4; ++k) {
        int32_t nx = x + dx[k], ny = y + dy[k];
        if (nx < 0 || ny < 0 || nx >= w || ny >= h) continue;
        int64_t q = (int64_t)ny * w + nx;
        c->dst.push_back((int32_t)q);
        c->cap.push_back(ncap(p, q));
      }
      c->dst.push_back(t);
      c->cap.push_back(tcap[p]);
      c->off[(size_t)p + 1] = (int32_t)c->dst.size();
    }
  for (int64_t p = 0; p < P; ++p) {
    c->dst.push_back((int32_t)p);
    c->cap.push_back(scap[p]);
  }
  c->off[(size_t)s + 1] = (int32_t)c->dst.size();
  c->off[(size_t)t + 1] = (int32_t)c->dst.size();
  c->m = (int64_t)c->dst.size();
  c->m_declared = c->m;
  c->s = s;
  c->t = t;
  return WBPR_OK;
}

// ---------------------------------------------------------------------------
// Residual builders.  Pairing is by construction (input arc i and its twin),
// O(n + m), replacing the reference's first-match search, which costs
// O(sum deg^2) and pairs antiparallel or parallel arcs with the wrong twin.
wbpr_status build_bcsr16(const wbpr_csr* g, Bcsr16* out) {
  const int32_t n = g->num_nodes;
  const int64_t m = g->num_edges;
  if (2 * m > std::numeric_limits<int32_t>::max()) return WBPR_ERR_OVERFLOW;
  std::vector<int32_t> indeg((size_t)n, 0);
  for (int64_t i = 0; i < m; ++i) indeg[g->destinations[i]]++;
  out->row.assign((size_t)n + 1, 0);
  for (int32_t u = 0; u < n; ++u)
    out->row[u + 1] = out->row[u] + (g->offsets[u + 1] - g->offsets[u]) + indeg[u];
  out->arc.resize((size_t)(4 * m));
  out->arx.resize((size_t)(4 * m));
  // reverse cursor of v starts after v's forward arcs
  std::vector<int32_t> cur((size_t)n);
  for (int32_t v = 0; v < n; ++v) cur[v] = out->row[v] + (g->offsets[v + 1] - g->offsets[v]);
  for (int32_t u = 0; u < n; ++u) {
    for (int32_t i = g->offsets[u]; i < g->offsets[u + 1]; ++i) {
      int32_t v = g->destinations[i];
      int32_t c = g->capacities ? g->capacities[i] : 1;
      int32_t f = out->row[u] + (i - g->offsets[u]);
      int32_t r = cur[v]++;
      out->arc[2 * (size_t)f] = v;
      out->arc[2 * (size_t)f + 1] = c;
      out->arx[2 * (size_t)f] = r;
      out->arx[2 * (size_t)f + 1] = c;
      out->arc[2 * (size_t)r] = u;
      out->arc[2 * (size_t)r + 1] = 0;
      out->arx[2 * (size_t)r] = f;
      out->arx[2 * (size_t)r + 1] = 0;
    }
  }
  return WBPR_OK;
}

wbpr_status build_rcsr_dev(const wbpr_csr* g, Rcsr* out) {
  const int32_t n = g->num_nodes;
  const int64_t m = g->num_edges;
  out->frow.assign(g->offsets, g->offsets + n + 1);
  out->farc.resize((size_t)(2 * m));
  out->fcap.resize((size_t)m);
  out->rrow.assign((size_t)n + 1, 0);
  out->rarc.resize((size_t)(2 * m));
  for (int64_t i = 0; i < m; ++i) {
    int32_t c = g->capacities ? g->capacities[i] : 1;
    out->farc[2 * i] = g->destinations[i];
    out->farc[2 * i + 1] = c;
    out->fcap[i] = c;
    out->rrow[(size_t)g->destinations[i] + 1]++;
  }
  for (int32_t v = 0; v < n; ++v) out->rrow[v + 1] += out->rrow[v];
  std::vector<int32_t> cur(out->rrow.begin(), out->rrow.end() - 1);
  for (int32_t u = 0; u < n; ++u)
    for (int32_t i = g->offsets[u]; i < g->offsets[u + 1]; ++i) {
      int32_t j = cur[g->destinations[i]]++;
      out->rarc[2 * (size_t)j] = u;
      out->rarc[2 * (size_t)j + 1] = i;
    }
  return WBPR_OK;
}

namespace {
// "<kind> x y z\n" appended to s.
void append_line(std::string& s, char kind, int64_t x, int64_t y, int64_t z) {
  char b[80];
  char* p = b;
  *p++ = kind;
  for (int64_t v : {x, y, z}) {
    *p++ = ' ';
    p = std::to_chars(p, b + sizeof(b), v).ptr;
  }
  *p++ = '\n';
  s.append(b, (size_t)(p - b));
}

// The arc lines of a CSR, in arc order, formatted by every host thread into
// its own buffer (2M arcs each per batch, so memory stays bounded) and
// written in order.  fmt(s, u, i) appends the line of arc i (tail u), or
// nothing.
template <class Fmt>
bool write_arc_lines(FILE* f, const wbpr_csr* g, Fmt&& fmt) {
  const int64_t m = g->num_edges;
  const int32_t n = g->num_nodes;
  const int T = host_threads();
  constexpr int64_t kPer = 1 << 21;
  std::vector<std::string> out((size_t)T);
  for (int64_t a0 = 0; a0 < m; a0 += kPer * T) {
    auto work = [&](int k) {
      std::string& s = out[(size_t)k];
      s.clear();
      const int64_t a = a0 + kPer * k, b = std::min(m, a + kPer);
      if (a >= b) return;
      s.reserve((size_t)(b - a) * 24);
      int32_t u = (int32_t)(std::upper_bound(g->offsets, g->offsets + (size_t)n + 1, (int64_t)a,
                                             [](int64_t x, int32_t o) { return x < (int64_t)o; }) -
                            g->offsets) - 1;
      for (int64_t i = a; i < b; ++i) {
        while ((int64_t)g->offsets[u + 1] <= i) ++u;
        fmt(s, u, i);
      }
    };
    if (!run_pieces(T, work)) return false;
    for (const std::string& s : out)
      if (!s.empty() && std::fwrite(s.data(), 1, s.size(), f) != s.size()) return false;
  }
  return true;
}

}  // namespace

}  // namespace wbpr

// ===========================================================================
// C ABI
using namespace wbpr;

extern "C" {

const char* wbpr_status_str(wbpr_status s) {
  switch (s) {
    case WBPR_OK: return "ok";
    case WBPR_ERR_INVALID_ARG: return "invalid argument";
    case WBPR_ERR_CUDA: return "CUDA error";
    case WBPR_ERR_NO_CONVERGENCE: return "no convergence within the round/time budget";
    case WBPR_ERR_OVERFLOW: return "int32 overflow of excess or arc index";
    case WBPR_ERR_VERIFY: return "device verification failed";
    case WBPR_ERR_IO: return "file missing, truncated or malformed";
    case WBPR_ERR_NO_DEVICE: return "no CUDA device";
    case WBPR_ERR_TIMEOUT: return "bounded grid-wide wait timed out";
  }
  return "unknown status";
}

int32_t wbpr_abi_version(void) { return WBPR_ABI_VERSION; }

void wbpr_host_csr_free(wbpr_host_csr* g) {
  if (!g) return;
  std::free(g->offsets);
  std::free(g->destinations);
  std::free(g->capacities);
  std::free(g);
}

wbpr_status wbpr_host_csr_copy(const wbpr_csr* in, wbpr_host_csr** out) {
  wbpr_status st = check_csr(in);
  if (st) return st;
  Csr c;
  c.n = in->num_nodes;
  c.m = in->num_edges;
  c.m_declared = in->num_edges;
  c.off.assign(in->offsets, in->offsets + in->num_nodes + 1);
  c.dst.assign(in->destinations, in->destinations + in->num_edges);
  if (in->capacities) c.cap.assign(in->capacities, in->capacities + in->num_edges);
  else c.cap.assign((size_t)in->num_edges, 1);
  c.s = in->source;
  c.t = in->sink;
  return to_host_csr(std::move(c), out);
}

#define WBPR_READER(name, fn)                                 \
  wbpr_status name(const char* path, wbpr_host_csr** out) {   \
    if (!out) return WBPR_ERR_INVALID_ARG;                    \
    *out = nullptr;                                           \
    Csr c;                                                    \
    wbpr_status st;                                           \
    try {                                                     \
      st = fn(path, &c);                                      \
    } catch (const std::bad_alloc&) {                         \
      return WBPR_ERR_IO;                                     \
    }                                                         \
    if (st) return st;                                        \
    return to_host_csr(std::move(c), out);                    \
  }
WBPR_READER(wbpr_read_dimacs, read_dimacs)
WBPR_READER(wbpr_read_snap_txt, read_snap_txt)
WBPR_READER(wbpr_read_snap_bin, read_snap_bin)
WBPR_READER(wbpr_read_graph_cache, read_graph_cache)
#undef WBPR_READER

wbpr_status wbpr_write_graph_cache(const char* path, const wbpr_csr* g) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  FILE* f = path ? std::fopen(path, "wb") : nullptr;
  if (!f) return WBPR_ERR_IO;
  CacheHeader h;
  std::memcpy(h.magic, kCacheMagic, 8);
  h.version = 1;
  h.flags = g->capacities ? 1 : 0;
  h.n = g->num_nodes;
  h.m = g->num_edges;
  h.m_declared = g->num_edges;
  h.s = g->source;
  h.t = g->sink;
  const size_t n1 = (size_t)g->num_nodes + 1, m = (size_t)g->num_edges;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  ok = ok && std::fwrite(g->offsets, 4, n1, f) == n1;
  ok = ok && (m == 0 || std::fwrite(g->destinations, 4, m, f) == m);
  if (g->capacities) ok = ok && (m == 0 || std::fwrite(g->capacities, 4, m, f) == m);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? WBPR_OK : WBPR_ERR_IO;
}

wbpr_status wbpr_write_dimacs_flow(const char* path, const wbpr_csr* g, int64_t flow,
                                   const int32_t* arc_flow) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  if (g->num_edges > 0 && !arc_flow) return WBPR_ERR_INVALID_ARG;
  FILE* f = path ? std::fopen(path, "w") : nullptr;
  if (!f) return WBPR_ERR_IO;
  std::fprintf(f, "c maximum flow from %d to %d (1-based ids)\n", g->source + 1, g->sink + 1);
  std::fprintf(f, "s %lld\n", (long long)flow);
  const bool ok = write_arc_lines(f, g, [&](std::string& s, int32_t u, int64_t i) {
    if (arc_flow[i] > 0) append_line(s, 'f', u + 1, (int64_t)g->destinations[i] + 1, arc_flow[i]);
  });
  return (std::fclose(f) == 0 && ok) ? WBPR_OK : WBPR_ERR_IO;
}

// Bipartite matching as maximum flow (the paper's super-source /
// super-sink construction): left vertices 0..L-1, right vertices L..L+R-1,
// s = L+R, t = L+R+1; s->l and r->t for every vertex, l->r for every listed
// pair (duplicates kept once); all capacities 1.
wbpr_status wbpr_bipartite_network(int32_t L, int32_t R, int64_t num_pairs, const int32_t* left,
                                   const int32_t* right, wbpr_host_csr** out) {
  if (!out) return WBPR_ERR_INVALID_ARG;
  *out = nullptr;
  if (L < 1 || R < 1 || num_pairs < 0 || (num_pairs > 0 && (!left || !right))) return WBPR_ERR_INVALID_ARG;
  if ((int64_t)L + R + 2 > std::numeric_limits<int32_t>::max() ||
      (int64_t)L + R + num_pairs > std::numeric_limits<int32_t>::max() / 2)
    return WBPR_ERR_OVERFLOW;
  try {
    std::vector<uint64_t> key((size_t)num_pairs);
    for (int64_t k = 0; k < num_pairs; ++k) {
      if (left[k] < 0 || left[k] >= L || right[k] < 0 || right[k] >= R) return WBPR_ERR_INVALID_ARG;
      key[(size_t)k] = ((uint64_t)(uint32_t)left[k] << 32) | (uint32_t)right[k];
    }
    std::sort(key.begin(), key.end());
    key.erase(std::unique(key.begin(), key.end()), key.end());
    Csr c;
    c.n = L + R + 2;
    c.s = L + R;
    c.t = L + R + 1;
    c.off.assign((size_t)c.n + 1, 0);
    for (uint64_t k : key) c.off[(size_t)(k >> 32) + 1]++;
    for (int32_t r = 0; r < R; ++r) c.off[(size_t)L + r + 1] = 1;  // r -> t
    c.off[(size_t)c.s + 1] = L;                                     // s -> every l
    for (int32_t u = 0; u < c.n; ++u) c.off[u + 1] += c.off[u];
    c.m = c.off[c.n];
    c.m_declared = c.m;
    c.dst.resize((size_t)c.m);
    size_t at = 0;
    for (uint64_t k : key) c.dst[at++] = L + (int32_t)(k & 0xffffffffu);
    for (int32_t r = 0; r < R; ++r) c.dst[at++] = c.t;
    for (int32_t l = 0; l < L; ++l) c.dst[at++] = l;
    c.cap.assign((size_t)c.m, 1);
    return to_host_csr(std::move(c), out);
  } catch (const std::bad_alloc&) {
    return WBPR_ERR_OVERFLOW;
  }
}

wbpr_status wbpr_write_snap_bin(const char* path, const wbpr_csr* g) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  FILE* f = path ? std::fopen(path, "wb") : nullptr;
  if (!f) return WBPR_ERR_IO;
  int32_t hdr[3] = {g->num_nodes, (int32_t)g->num_edges, (int32_t)g->num_edges};
  bool ok = std::fwrite(hdr, 4, 3, f) == 3;
  ok = ok && std::fwrite(g->destinations, 4, (size_t)g->num_edges, f) == (size_t)g->num_edges;
  ok = ok && std::fwrite(g->offsets, 4, (size_t)g->num_nodes + 1, f) == (size_t)g->num_nodes + 1;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? WBPR_OK : WBPR_ERR_IO;
}

wbpr_status wbpr_write_dimacs(const char* path, const wbpr_csr* g) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  FILE* f = path ? std::fopen(path, "w") : nullptr;
  if (!f) return WBPR_ERR_IO;
  std::fprintf(f, "p max %d %lld\n", g->num_nodes, (long long)g->num_edges);
  if (g->source >= 0) std::fprintf(f, "n %d s\n", g->source + 1);
  if (g->sink >= 0) std::fprintf(f, "n %d t\n", g->sink + 1);
  const bool ok = write_arc_lines(f, g, [&](std::string& s, int32_t u, int64_t i) {
    append_line(s, 'a', u + 1, (int64_t)g->destinations[i] + 1, g->capacities ? g->capacities[i] : 1);
  });
  return (std::fclose(f) == 0 && ok) ? WBPR_OK : WBPR_ERR_IO;
}

#define WBPR_GEN(call)                            \
  if (!out) return WBPR_ERR_INVALID_ARG;          \
  *out = nullptr;                                 \
  Csr c;                                          \
  wbpr_status st;                                 \
  try {                                           \
    st = call;                                    \
  } catch (const std::bad_alloc&) {               \
    return WBPR_ERR_OVERFLOW;                     \
  }                                               \
  if (st) return st;                              \
  return to_host_csr(std::move(c), out);

wbpr_status wbpr_gen_genrmf(int32_t a, int32_t b, int32_t c1, int32_t c2, uint64_t seed,
                            wbpr_host_csr** out) {
  WBPR_GEN(gen_genrmf(a, b, c1, c2, seed, &c))
}
wbpr_status wbpr_gen_rmat(int32_t scale, int32_t ef, double a, double b, double cc, int32_t lo,
                          int32_t hi, uint64_t seed, wbpr_host_csr** out) {
  WBPR_GEN(gen_rmat(scale, ef, a, b, cc, lo, hi, seed, &c))
}
wbpr_status wbpr_gen_bipartite(int32_t L, int32_t R, double zs, int32_t dmax, uint64_t seed,
                               wbpr_host_csr** out) {
  WBPR_GEN(gen_bipartite(L, R, zs, dmax, seed, &c))
}
wbpr_status wbpr_gen_layered(int32_t layers, int32_t width, int32_t dlo, int32_t dhi,
                             int32_t clo, int32_t chi, uint64_t seed, wbpr_host_csr** out) {
  WBPR_GEN(gen_layered(layers, width, dlo, dhi, clo, chi, seed, &c))
}
wbpr_status wbpr_gen_grid(int32_t w, int32_t h, uint64_t seed, wbpr_host_csr** out) {
  WBPR_GEN(gen_grid(w, h, seed, &c))
}
#undef WBPR_GEN

wbpr_status wbpr_build_rcsr(const wbpr_csr* g, int32_t* roffsets, int32_t* rdestinations,
                            int32_t* flow_index) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  if (!roffsets || (g->num_edges && (!rdestinations || !flow_index))) return WBPR_ERR_INVALID_ARG;
  Rcsr r;
  st = build_rcsr_dev(g, &r);
  if (st) return st;
  std::memcpy(roffsets, r.rrow.data(), 4 * ((size_t)g->num_nodes + 1));
  for (int64_t j = 0; j < g->num_edges; ++j) {
    rdestinations[j] = r.rarc[2 * j];
    flow_index[j] = r.rarc[2 * j + 1];
  }
  return WBPR_OK;
}

wbpr_status wbpr_build_bcsr(const wbpr_csr* g, int32_t* offsets, int32_t* destinations,
                            int32_t* capacities, int32_t* backward_idx) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  if (!offsets || (g->num_edges && (!destinations || !capacities || !backward_idx)))
    return WBPR_ERR_INVALID_ARG;
  Bcsr16 b;
  st = build_bcsr16(g, &b);
  if (st) return st;
  std::memcpy(offsets, b.row.data(), 4 * ((size_t)g->num_nodes + 1));
  for (int64_t a = 0; a < 2 * g->num_edges; ++a) {
    destinations[a] = b.arc[2 * a];
    capacities[a] = b.arx[2 * a + 1];
    backward_idx[a] = b.arx[2 * a];
  }
  return WBPR_OK;
}

wbpr_status wbpr_build_bcsr2(const wbpr_csr* g, int32_t* offsets, int32_t* destinations,
                             int32_t* flows) {
  wbpr_status st = check_csr(g);
  if (st) return st;
  if (!offsets || (g->num_edges && (!destinations || !flows))) return WBPR_ERR_INVALID_ARG;
  Bcsr16 b;
  st = build_bcsr16(g, &b);
  if (st) return st;
  std::memcpy(offsets, b.row.data(), 4 * ((size_t)g->num_nodes + 1));
  for (int64_t a = 0; a < 2 * g->num_edges; ++a) {
    destinations[a] = b.arc[2 * a];
    flows[2 * a] = b.arc[2 * a + 1];
    flows[2 * a + 1] = b.arx[2 * a];
  }
  return WBPR_OK;
}

}  // extern "C"
