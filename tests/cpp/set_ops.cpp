// Exercises the drop-in host-side ops::set_intersect / set_union /
// set_difference on hand-built sets in each layout and prints one line per
// case: "<name> <cardinality> <elements...>" (elements only for short results).
#include <cstdio>
#include <vector>

#include "set/Set.hpp"

static std::vector<uint8_t> pshort_bytes(const std::vector<uint32_t>& v) {
  std::vector<uint16_t> s;
  size_t i = 0;
  while (i < v.size()) {
    const uint32_t hi = v[i] >> 16;
    size_t j = i;
    while (j < v.size() && (v[j] >> 16) == hi) j++;
    s.push_back((uint16_t)hi);
    s.push_back((uint16_t)(j - i - 1));
    for (size_t k = i; k < j; k++) s.push_back((uint16_t)(v[k] & 0xffff));
    i = j;
  }
  std::vector<uint8_t> b(s.size() * 2);
  std::memcpy(b.data(), s.data(), b.size());
  return b;
}
static std::vector<uint8_t> bitset_bytes(const std::vector<uint32_t>& v, uint64_t first_word, uint64_t words) {
  std::vector<uint8_t> b(8 + 8 * words, 0);
  std::memcpy(b.data(), &first_word, 8);
  for (uint32_t x : v) {
    uint64_t w;
    std::memcpy(&w, b.data() + 8 + 8 * (x / 64 - first_word), 8);
    w |= 1ull << (x % 64);
    std::memcpy(b.data() + 8 + 8 * (x / 64 - first_word), &w, 8);
  }
  return b;
}
template <class R>
static void print(const char* name, const Set<R>& c) {
  std::printf("%s %zu", name, c.cardinality);
  if (c.cardinality <= 16) c.foreach([](uint32_t x) { std::printf(" %u", x); });
  std::printf("\n");
}

int main() {
  std::vector<uint32_t> a = {1, 5, 9, 64, 127, 70000, 70001};
  std::vector<uint32_t> b = {5, 6, 9, 127, 128, 70001, 90000};
  std::vector<uint8_t> ua(a.size() * 4), ub(b.size() * 4);
  std::memcpy(ua.data(), a.data(), ua.size());
  std::memcpy(ub.data(), b.data(), ub.size());
  std::vector<uint8_t> pa = pshort_bytes(a), pb = pshort_bytes(b);
  std::vector<uint8_t> ba = bitset_bytes(a, 0, 70001 / 64 + 1), bb = bitset_bytes(b, 0, 90000 / 64 + 1);
  Set<uinteger> UA(ua.data(), a.size(), ua.size(), common::UINTEGER), UB(ub.data(), b.size(), ub.size(), common::UINTEGER);
  Set<pshort> PA(pa.data(), a.size(), pa.size(), common::PSHORT), PB(pb.data(), b.size(), pb.size(), common::PSHORT);
  Set<bitset> BA(ba.data(), a.size(), ba.size(), common::BITSET), BB(bb.data(), b.size(), bb.size(), common::BITSET);
  std::vector<uint8_t> buf(1 << 20);
  Set<hybrid> C(buf.data());
  print("uu", *ops::set_intersect(&C, &UA, &UB));
  print("up", *ops::set_intersect(&C, &UA, &PB));
  print("pb", *ops::set_intersect(&C, &PA, &BB));
  print("bb", *ops::set_intersect(&C, &BA, &BB));
  print("pp", *ops::set_intersect(&C, &PA, &PB));
  // Two pshort sets sharing the full block 0 (plus 70000): the u16 count drops it.
  std::vector<uint32_t> full;
  for (uint32_t x = 0; x < 65536; x++) full.push_back(x);
  full.push_back(70000);
  std::vector<uint8_t> pf = pshort_bytes(full);
  Set<pshort> PF(pf.data(), full.size(), pf.size(), common::PSHORT);
  print("pp_full", *ops::set_intersect(&C, &PF, &PF));
  std::vector<uint8_t> uf(full.size() * 4);
  std::memcpy(uf.data(), full.data(), uf.size());
  Set<uinteger> UF(uf.data(), full.size(), uf.size(), common::UINTEGER);
  print("up_full", *ops::set_intersect(&C, &UF, &PF));
  // union / difference as n_path uses them
  Set<bitset> vis(8 + 8 * (90000 / 64 + 1));
  Set<bitset> old(8 + 8 * (90000 / 64 + 1));
  ops::set_union(&vis, &UA);
  old.copy_from(vis);
  ops::set_union(&vis, &PB);
  Set<uinteger> F(buf.data());
  print("diff", *ops::set_difference(&F, &vis, &old));
  return 0;
}
