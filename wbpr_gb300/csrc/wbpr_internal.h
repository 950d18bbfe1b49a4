// Internal declarations shared by the host C++ files and the CUDA files of
// libwbpr.  Nothing here is part of the C ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "wbpr.h"

namespace wbpr {

// Owned CSR used inside the library.
struct Csr {
  int32_t n = 0;
  int64_t m = 0;
  int64_t m_declared = 0;
  std::vector<int32_t> off;  // n + 1
  std::vector<int32_t> dst;  // m
  std::vector<int32_t> cap;  // m
  int32_t s = -1;
  int32_t t = -1;
};

// Validate a caller CSR: monotone offsets, ids in range, capacities >= 0.
wbpr_status check_csr(const wbpr_csr* g);
// Only the O(1) part: pointers, sizes, offsets[0] == 0, offsets[n] == m (the
// device build checks the rest while it reads the arrays).
wbpr_status check_csr_shape(const wbpr_csr* g);

// Convert between the C view and the owned form.
wbpr_status to_host_csr(Csr&& c, wbpr_host_csr** out);

// Maximum, over vertices, of the summed capacity of arcs entering the vertex
// (an upper bound on any excess the solver can hold there).
int64_t max_in_capacity(const wbpr_csr* g);

// BCSR16 residual rows: row[n+1]; arc = {dst, residual}; arx = {rev, cap}.
// Forward arcs of u come first in input order, then the reverse twins of the
// arcs entering u, ordered by tail.  fwd_slot(i) = row[u] + (i - off[u]).
struct Bcsr16 {
  std::vector<int32_t> row;
  std::vector<int32_t> arc;  // 2 ints per residual arc
  std::vector<int32_t> arx;  // 2 ints per residual arc
};
wbpr_status build_bcsr16(const wbpr_csr* g, Bcsr16* out);

// RCSR residual form: forward {dst, residual}, reverse {tail, forward id}.
struct Rcsr {
  std::vector<int32_t> frow;  // n + 1
  std::vector<int32_t> farc;  // 2 ints per forward arc: dst, residual
  std::vector<int32_t> fcap;  // capacity per forward arc
  std::vector<int32_t> rrow;  // n + 1
  std::vector<int32_t> rarc;  // 2 ints per reverse entry: tail, forward id
};
wbpr_status build_rcsr_dev(const wbpr_csr* g, Rcsr* out);

// Hardware threads to use for host loops.
int host_threads();

// Record the text that wbpr_last_error() returns on this host thread.
void set_last_error(const std::string& msg);

}  // namespace wbpr
