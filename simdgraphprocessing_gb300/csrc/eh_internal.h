// Internal helpers shared by the host (.cpp) and device (.cu) translation units.
#pragma once

#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/eh_gb300.h"

namespace eh {

// Records a message for eh_last_error() and returns the status unchanged.
eh_status set_error(eh_status s, const char* fmt, ...);
void clear_error();

// Host graph behind eh_hgraph_t: CSR adjacency of a symmetric graph, or of
// the out-neighbourhoods of a directed one (then with a second, in-CSR).
struct HostGraph {
  uint64_t n = 0;
  std::vector<uint64_t> offsets;  // n+1
  std::vector<uint32_t> nbrs;     // offsets[n]
  std::vector<uint64_t> ext_ids;  // n
  uint64_t max_nbrhood_size = 0;  // as the reference reports it (pre-dedup for edge lists)
  bool directed = false;
  std::vector<uint64_t> in_offsets;  // directed only: n+1
  std::vector<uint32_t> in_nbrs;     // directed only: in_offsets[n]
};

// Builds a symmetric CSR from distinct undirected keys (lo << 32 | hi, lo < hi).
// `keys` is consumed.  Rows come out sorted ascending.
void csr_from_undirected_keys(uint64_t n, std::vector<uint64_t>& keys, HostGraph& g);

// Split of a host adjacency (n rows, m = offsets[n] entries) into `chunks`
// uploads of about m / chunks entries: chunk c holds rows [rows[c], rows[c+1])
// and is complete once entries [0, upto[c]) have been copied.  rows runs from
// 0 to n and upto from its first value to m, both non-decreasing whatever the
// offsets hold (a binary search of the offsets places the boundaries; rows
// with bad offsets are for the device pass to reject).
void plan_upload_chunks(uint64_t n, const uint64_t* offsets, uint64_t m, uint64_t chunks,
                        std::vector<uint64_t>& rows, std::vector<uint64_t>& upto);

}  // namespace eh

#define EH_CHECK_ARG(cond, ...)                                      \
  do {                                                               \
    if (!(cond)) return eh::set_error(EH_ERR_INVALID_ARGUMENT, __VA_ARGS__); \
  } while (0)
