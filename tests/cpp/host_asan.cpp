// Drives the host half of the engine (csrc/eh_host.cpp: generators, binary and
// edge-list loaders, degree reordering, directed graphs) under AddressSanitizer
// and UndefinedBehaviorSanitizer.  Prints "ok" when every call behaves.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "eh_gb300.h"

#define REQUIRE(x)                                                              \
  do {                                                                          \
    if (!(x)) {                                                                 \
      std::fprintf(stderr, "failed: %s (%s)\n", #x, eh_last_error());           \
      return 1;                                                                 \
    }                                                                           \
  } while (0)

int main(int argc, char** argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  eh_hgraph_t g = nullptr, h = nullptr, d = nullptr, e = nullptr;
  REQUIRE(eh_generate_rmat(10, 6000, 0.57, 0.19, 0.19, 3, &g) == EH_OK);
  REQUIRE(eh_hgraph_reorder_by_degree(g) == EH_OK);
  const std::string bin = dir + "/g.bin";
  REQUIRE(eh_hgraph_write_binary(g, bin.c_str()) == EH_OK);
  REQUIRE(eh_hgraph_read_binary(bin.c_str(), &h) == EH_OK);
  uint64_t n1, m1, n2, m2;
  const uint64_t *o1, *o2;
  const uint32_t *b1, *b2;
  REQUIRE(eh_hgraph_view(g, &n1, &m1, &o1, &b1, nullptr, nullptr) == EH_OK);
  REQUIRE(eh_hgraph_view(h, &n2, &m2, &o2, &b2, nullptr, nullptr) == EH_OK);
  REQUIRE(n1 == n2 && m1 == m2);
  for (uint64_t k = 0; k < m1; k++) REQUIRE(b1[k] == b2[k]);
  // truncated file -> EH_ERR_IO, nothing leaked
  {
    FILE* f = std::fopen(bin.c_str(), "r+b");
    REQUIRE(f != nullptr);
    std::fclose(f);
    const std::string cut = dir + "/cut.bin";
    FILE* src = std::fopen(bin.c_str(), "rb");
    FILE* dst = std::fopen(cut.c_str(), "wb");
    char buf[100];
    size_t r = std::fread(buf, 1, sizeof(buf), src);
    std::fwrite(buf, 1, r, dst);
    std::fclose(src);
    std::fclose(dst);
    eh_hgraph_t bad = nullptr;
    REQUIRE(eh_hgraph_read_binary(cut.c_str(), &bad) == EH_ERR_IO);
    REQUIRE(eh_hgraph_read_directed_binary(cut.c_str(), &bad) == EH_ERR_IO);
  }
  // edge lists, directed graphs
  const std::string txt = dir + "/e.txt";
  {
    FILE* f = std::fopen(txt.c_str(), "w");
    std::fputs("1 2\n2 3\n3 1\n3 3\n7 1\n1 2\n", f);
    std::fclose(f);
  }
  REQUIRE(eh_hgraph_read_edge_list(txt.c_str(), &e) == EH_OK);
  eh_hgraph_free(e);
  REQUIRE(eh_hgraph_read_directed_edge_list(txt.c_str(), &e) == EH_OK);
  eh_hgraph_free(e);
  REQUIRE(eh_generate_directed_rmat(10, 5000, 0.57, 0.19, 0.19, 4, &d) == EH_OK);
  const std::string dbin = dir + "/d.bin";
  REQUIRE(eh_hgraph_write_directed_binary(d, dbin.c_str()) == EH_OK);
  REQUIRE(eh_hgraph_read_directed_binary(dbin.c_str(), &e) == EH_OK);
  int directed = 0;
  uint64_t mi = 0;
  REQUIRE(eh_hgraph_in_view(e, &directed, &mi, nullptr, nullptr) == EH_OK && directed == 1 && mi == 5000);
  REQUIRE(eh_hgraph_reorder_by_degree(e) == EH_ERR_UNSUPPORTED);
  eh_hgraph_free(e);
  eh_hgraph_t er = nullptr, ba = nullptr, pc = nullptr;
  REQUIRE(eh_generate_er(500, 3000, 5, &er) == EH_OK);
  REQUIRE(eh_generate_ba(500, 4, 6, &ba) == EH_OK);
  REQUIRE(eh_generate_planted_cliques(2000, 5000, 3, 10, 40, 7, &pc) == EH_OK);
  REQUIRE(eh_generate_rmat(2, 100, 0.57, 0.19, 0.19, 1, &e) == EH_ERR_INVALID_ARGUMENT);  // more edges than pairs
  eh_hgraph_free(er);
  eh_hgraph_free(ba);
  eh_hgraph_free(pc);
  eh_hgraph_free(d);
  eh_hgraph_free(h);
  eh_hgraph_free(g);
  std::puts("ok");
  return 0;
}
