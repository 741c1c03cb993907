// Host-side set operations of the reference's ops namespace
// (src/set/ops/intersection.hpp, union.hpp, difference.hpp), for code that
// combines rows read back with SparseMatrix::get_row / get_column.  The pattern
// counts never call these: they run as whole-graph launches on the device.
//
// set_intersect gives the reference's cardinality (including the pshort ∩
// pshort u16 partition count, intersection.hpp:857-865: a 2^16 block common to
// both sets adds 0 and none of its values reach the output) and writes the
// elements as a uinteger list into the caller's buffer C->data (the reference
// writes the layout of the kernel it dispatched to; the elements are the same).
#ifndef EH_DROPIN_OPS_HPP
#define EH_DROPIN_OPS_HPP

#include <vector>

namespace ops {

namespace detail {
template <class S>
inline std::vector<uint32_t> elements(const S* s) {
  std::vector<uint32_t> v;
  v.reserve(s->cardinality);
  if (s->cardinality) s->foreach([&](uint32_t x) { v.push_back(x); });
  return v;
}
inline uint64_t rd64(const uint8_t* p) {
  uint64_t v;
  std::memcpy(&v, p, 8);
  return v;
}
}  // namespace detail

// |A ∩ B| into C (C->data must hold min(|A|, |B|) u32 values).
template <class R, class TA, class TB>
inline Set<R>* set_intersect(Set<R>* C, const Set<TA>* A, const Set<TB>* B) {
  const std::vector<uint32_t> a = detail::elements(A), b = detail::elements(B);
  uint32_t* out = reinterpret_cast<uint32_t*>(C->data);
  size_t i = 0, j = 0, k = 0;
  while (i < a.size() && j < b.size()) {
    if (a[i] < b[j]) i++;
    else if (b[j] < a[i]) j++;
    else {
      out[k++] = a[i];
      i++;
      j++;
    }
  }
  if (A->type == common::PSHORT && B->type == common::PSHORT && k >= 65536) {
    // Drop every 2^16 block whose 65,536 values are all in the result.
    size_t w = 0;
    for (size_t r = 0; r < k;) {
      const uint32_t hi = out[r] >> 16;
      size_t e = r;
      while (e < k && (out[e] >> 16) == hi) e++;
      if (e - r != 65536)
        for (size_t q = r; q < e; q++) out[w++] = out[q];
      r = e;
    }
    k = w;
  }
  C->cardinality = k;
  C->number_of_bytes = k * sizeof(uint32_t);
  C->density = 0.0;
  C->type = common::UINTEGER;
  return C;
}

// A |= B for a bitset A laid out as [u64 first word][u64 words] (union.hpp:6-127).
template <class T>
inline void set_union(Set<bitset>* A, const Set<T>* B) {
  if (A->number_of_bytes < 8) return;
  const uint64_t first = detail::rd64(A->data);
  const uint64_t words = (A->number_of_bytes - 8) / 8;
  uint8_t* w = A->data + 8;
  if (B->cardinality)
    B->foreach([&](uint32_t x) {
      const uint64_t word = x / 64;
      if (word < first || word - first >= words) return;
      uint64_t v;
      std::memcpy(&v, w + 8 * (word - first), 8);
      v |= 1ull << (x % 64);
      std::memcpy(w + 8 * (word - first), &v, 8);
    });
}

// C = A \ B for two bitsets, as an ascending uinteger list (difference.hpp:5-84).
inline Set<uinteger>* set_difference(Set<uinteger>* C, const Set<bitset>* A, const Set<bitset>* B) {
  size_t k = 0;
  uint32_t* out = reinterpret_cast<uint32_t*>(C->data);
  if (A->number_of_bytes >= 8 && B->number_of_bytes >= 8) {
    const uint64_t fa = detail::rd64(A->data), fb = detail::rd64(B->data);
    const uint64_t na = (A->number_of_bytes - 8) / 8, nb = (B->number_of_bytes - 8) / 8;
    for (uint64_t i = 0; i < na; i++) {
      uint64_t x, y = 0;
      std::memcpy(&x, A->data + 8 + 8 * i, 8);
      const uint64_t word = fa + i;
      if (word >= fb && word - fb < nb) std::memcpy(&y, B->data + 8 + 8 * (word - fb), 8);
      for (uint64_t r = x & ~y; r; r &= r - 1) out[k++] = (uint32_t)(64 * word + __builtin_ctzll(r));
    }
  }
  C->cardinality = k;
  C->number_of_bytes = k * sizeof(uint32_t);
  C->density = 0.0;
  C->type = common::UINTEGER;
  return C;
}

}  // namespace ops

#endif
