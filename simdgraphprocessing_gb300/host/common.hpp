// Drop-in host API, common pieces: the names of the reference's src/common.hpp
// that application code uses (layout tags, timers, thread knobs), implemented
// over the GB300 engine's C ABI (include/eh_gb300.h).
#ifndef EH_DROPIN_COMMON_HPP
#define EH_DROPIN_COMMON_HPP

#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iostream>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/eh_gb300.h"

#define PADDING 300
#define MAX_THREADS 512
#define WRITE_TABLE 0
#define COMPRESSION 0
#define VECTORIZE 1

using namespace std;

namespace common {

// Layout tags, same values as the reference (src/common.hpp:171-181).
enum type : uint8_t {
  BITSET = 0,
  PSHORT = 1,
  UINTEGER = 2,
  BITPACKED = 3,
  VARIANT = 4,
  HYBRID = 5,
  KUNLE = 6,
  BITSET_NEW = 7,
  NEW_TYPE = 8
};

enum graph_type { DIRECTED, UNDIRECTED };

// Optimizer thresholds the reference exposes (src/common.hpp:70-73).  The device
// optimizer applies these defaults: bitset when |S| > 1 and |S|/(last-first) > 1/256.
static const size_t bitset_length = 0;
static const double bitset_req = (1.0 / 256.0);

static inline double startClock() { return omp_get_wtime(); }
static inline double stopClock(double t_in) { return omp_get_wtime() - t_in; }
static inline double stopClock(const string& in, double t_in) {
  const double t = omp_get_wtime() - t_in;
  std::cout << "Time[" + in + "]: " << t << " s" << std::endl;
  return t;
}

// The engine keeps per-thread state on the device; host scratch is not needed.
static inline void alloc_scratch_space(size_t, size_t) {}

// Throws with the engine's message when a C-ABI call fails.
static inline void check(eh_status s) {
  if (s != EH_OK) throw std::runtime_error(std::string(eh_status_string(s)) + ": " + eh_last_error());
}

static inline vector<uint32_t> range(uint32_t max) {
  vector<uint32_t> r(max);
  for (uint32_t i = 0; i < max; i++) r[i] = i;
  return r;
}

}  // namespace common

#endif
