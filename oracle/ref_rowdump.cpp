// Row dump of the reference's own SparseMatrix, for byte-format pinning.
// Compiled by oracle/build_ref.sh against the unmodified reference headers.
// Usage: ref_rowdump graph.bin <uint|bs|pshort|hybrid> <lower|all> out.bin
// out.bin: for each row, u8 type tag, u32 cardinality, u64 flattened byte
// count, then the flattened bytes exactly as SparseMatrix::build left them.
#include <cstdio>
#include <cstring>
#include <string>

#include "SparseMatrix.hpp"

template <class T>
static int dump(MutableGraph* g, bool lower, bool hybrid, const char* path) {
  auto node_sel = [](uint32_t, uint32_t) -> bool { return true; };
  auto lower_sel = [](uint32_t node, uint32_t nbr, uint32_t) -> bool { return nbr < node; };
  auto all_sel = [](uint32_t, uint32_t, uint32_t) -> bool { return true; };
  SparseMatrix<T, T>* m = lower ? SparseMatrix<T, T>::build(g, node_sel, lower_sel, 1)
                                : SparseMatrix<T, T>::build(g, node_sel, all_sel, 1);
  FILE* f = fopen(path, "wb");
  if (!f) return 1;
  for (size_t i = 0; i < m->matrix_size; i++) {
    Set<T> s = m->get_row((uint32_t)i);
    uint8_t type = (uint8_t)s.type;
    uint32_t card = (uint32_t)s.cardinality;
    // Flattened size: optional u64 tag, then uint payload or [u32 nbytes][payload].
    uint64_t inner = 0;
    if (s.type == common::UINTEGER) inner = 4ull * card;
    else if (card > 0) inner = 4 + s.number_of_bytes;
    uint64_t total = inner + (hybrid ? 8 : 0);
    fwrite(&type, 1, 1, f);
    fwrite(&card, 4, 1, f);
    fwrite(&total, 8, 1, f);
    fwrite(m->row_arrays[i], 1, total, f);
  }
  fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 5) {
    fprintf(stderr, "usage: %s graph.bin layout lower|all out.bin\n", argv[0]);
    return 2;
  }
  MutableGraph* g = MutableGraph::undirectedFromBinary(argv[1]);
  std::string layout = argv[2];
  bool lower = std::string(argv[3]) == "lower";
  ops::prepare_shuffling_dictionary16();
  if (layout == "uint") return dump<uinteger>(g, lower, false, argv[4]);
  if (layout == "bs") return dump<bitset>(g, lower, false, argv[4]);
  if (layout == "pshort") return dump<pshort>(g, lower, false, argv[4]);
  if (layout == "hybrid") return dump<hybrid>(g, lower, true, argv[4]);
  fprintf(stderr, "unknown layout %s\n", layout.c_str());
  return 2;
}
