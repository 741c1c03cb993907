// Drop-in layout tags (the reference's src/set/layouts/{uinteger,pshort,bitset,
// hybrid}.hpp).  Each names its engine layout and can walk a row that was
// copied back to the host in the reference's flattened format (debug / compat
// views; the counts themselves run on the device).
#ifndef EH_DROPIN_LAYOUTS_HPP
#define EH_DROPIN_LAYOUTS_HPP

#include "../../common.hpp"

namespace eh_layout_detail {
inline uint64_t rd64(const uint8_t* p) { uint64_t v; std::memcpy(&v, p, 8); return v; }
inline uint32_t rd32(const uint8_t* p) { uint32_t v; std::memcpy(&v, p, 4); return v; }
inline uint16_t rd16(const uint8_t* p) { uint16_t v; std::memcpy(&v, p, 2); return v; }

// Elements of a payload (data points past any u32 byte count) in ascending order.
template <typename F>
inline void walk(common::type t, const uint8_t* data, size_t card, size_t nbytes, F f) {
  if (t == common::UINTEGER) {
    for (size_t i = 0; i < card; i++) f(rd32(data + 4 * i));
  } else if (t == common::BITSET) {
    if (nbytes < 8) return;
    const uint64_t first = rd64(data);
    const size_t words = (nbytes - 8) / 8;
    for (size_t w = 0; w < words; w++) {
      uint64_t x = rd64(data + 8 + 8 * w);
      while (x) {
        f((uint32_t)(64 * (first + w) + __builtin_ctzll(x)));
        x &= x - 1;
      }
    }
  } else if (t == common::PSHORT) {
    size_t i = 0, seen = 0;
    while (seen < card) {
      const uint32_t hi = (uint32_t)rd16(data + 2 * i) << 16;
      const size_t cnt = (size_t)rd16(data + 2 * (i + 1)) + 1;
      for (size_t k = 0; k < cnt; k++) f(hi | rd16(data + 2 * (i + 2 + k)));
      seen += cnt;
      i += cnt + 2;
    }
  }
}
// (payload offset, payload bytes, type) of a flattened row without the hybrid tag.
inline std::tuple<size_t, size_t, common::type> inner(const uint8_t* p, size_t card, common::type t) {
  if (t == common::UINTEGER) return std::make_tuple((size_t)0, card * 4, t);
  if (card == 0) return std::make_tuple((size_t)0, (size_t)0, t);
  return std::make_tuple((size_t)4, (size_t)rd32(p), t);
}
}  // namespace eh_layout_detail

#define EH_LAYOUT_COMMON(TAG)                                                                       \
  template <typename F>                                                                             \
  static void foreach(F f, const uint8_t* data, size_t card, size_t nbytes, common::type t) {        \
    eh_layout_detail::walk(t, data, card, nbytes, f);                                               \
  }                                                                                                 \
  template <typename F>                                                                             \
  static void foreach_until(F f, const uint8_t* data, size_t card, size_t nbytes, common::type t) { \
    bool stop = false;                                                                              \
    eh_layout_detail::walk(t, data, card, nbytes, [&](uint32_t x) {                                 \
      if (!stop && f(x)) stop = true;                                                               \
    });                                                                                             \
  }

class uinteger {
 public:
  static common::type get_type() { return common::UINTEGER; }
  static eh_layout engine_layout() { return EH_LAYOUT_UINTEGER; }
  static std::tuple<size_t, size_t, common::type> get_flattened_data(const uint8_t* d, size_t card) {
    return eh_layout_detail::inner(d, card, common::UINTEGER);
  }
  EH_LAYOUT_COMMON(uinteger)
};

class pshort {
 public:
  static common::type get_type() { return common::PSHORT; }
  static eh_layout engine_layout() { return EH_LAYOUT_PSHORT; }
  static std::tuple<size_t, size_t, common::type> get_flattened_data(const uint8_t* d, size_t card) {
    return eh_layout_detail::inner(d, card, common::PSHORT);
  }
  EH_LAYOUT_COMMON(pshort)
};

class bitset {
 public:
  static common::type get_type() { return common::BITSET; }
  static eh_layout engine_layout() { return EH_LAYOUT_BITSET; }
  static std::tuple<size_t, size_t, common::type> get_flattened_data(const uint8_t* d, size_t card) {
    return eh_layout_detail::inner(d, card, common::BITSET);
  }
  EH_LAYOUT_COMMON(bitset)
};

// Per-set choice between uinteger and bitset (hybrid::get_type, hybrid.hpp:73-100),
// made on the device when the matrix is built.
class hybrid {
 public:
  static common::type get_type() { return common::HYBRID; }
  static eh_layout engine_layout() { return EH_LAYOUT_HYBRID; }
  static std::tuple<size_t, size_t, common::type> get_flattened_data(const uint8_t* d, size_t card) {
    const common::type t = (common::type)eh_layout_detail::rd64(d);
    auto r = eh_layout_detail::inner(d + 8, card, t);
    std::get<0>(r) += 8;
    return r;
  }
  EH_LAYOUT_COMMON(hybrid)
};

#undef EH_LAYOUT_COMMON

#endif
