// Checks eh::plan_upload_chunks (csrc/eh_host.cpp), the split of a host
// adjacency into the uploads that the build's first pass measures one by one:
// boundaries stay monotone and in range for any offsets, every entry is copied
// once, and with valid offsets each chunk's rows lie inside what has been
// copied when that chunk's upload completes.  Prints "ok".
#include <cstdio>
#include <random>
#include <vector>

#include "eh_internal.h"

#define REQUIRE(x)                                                     \
  do {                                                                 \
    if (!(x)) {                                                        \
      std::fprintf(stderr, "failed: %s (line %d)\n", #x, __LINE__);    \
      return 1;                                                        \
    }                                                                  \
  } while (0)

static int check(uint64_t n, const std::vector<uint64_t>& off, uint64_t chunks, bool valid) {
  const uint64_t m = off[n];
  std::vector<uint64_t> rows, upto;
  eh::plan_upload_chunks(n, off.data(), m, chunks, rows, upto);
  const uint64_t c_used = chunks < 1 ? 1 : chunks;
  REQUIRE(rows.size() == c_used + 1 && upto.size() == c_used);
  REQUIRE(rows.front() == 0 && rows.back() == n);
  for (size_t c = 0; c + 1 < rows.size(); c++) REQUIRE(rows[c] <= rows[c + 1]);
  REQUIRE(upto.back() == m);
  for (size_t c = 0; c < upto.size(); c++) {
    REQUIRE(upto[c] <= m);
    if (c) REQUIRE(upto[c - 1] <= upto[c]);
  }
  if (valid) {
    for (size_t c = 0; c < upto.size(); c++)
      for (uint64_t r = rows[c]; r < rows[c + 1]; r++) REQUIRE(off[r + 1] <= upto[c]);
  }
  return 0;
}

int main() {
  std::mt19937_64 rng(7);
  // n = 0 and empty graphs
  REQUIRE(check(0, {0}, 1, true) == 0);
  REQUIRE(check(0, {0}, 4, true) == 0);
  REQUIRE(check(5, {0, 0, 0, 0, 0, 0}, 3, true) == 0);
  for (int trial = 0; trial < 400; trial++) {
    const uint64_t n = rng() % 3000;
    std::vector<uint64_t> off(n + 1, 0);
    for (uint64_t i = 0; i < n; i++) {
      const uint64_t kind = rng() % 10;
      const uint64_t d = kind == 0 ? rng() % 5000 : kind < 4 ? 0 : rng() % 8;  // hubs, empty rows, short rows
      off[i + 1] = off[i] + d;
    }
    const uint64_t chunks = 1 + rng() % 20;
    REQUIRE(check(n, off, chunks, true) == 0);
    if (n > 2) {  // falling or out-of-range offsets: only the invariants hold
      std::vector<uint64_t> bad = off;
      for (int k = 0; k < 3; k++) bad[1 + rng() % (n - 1)] = rng() % (off[n] + 10);
      REQUIRE(check(n, bad, chunks, false) == 0);
    }
  }
  std::puts("ok");
  return 0;
}
