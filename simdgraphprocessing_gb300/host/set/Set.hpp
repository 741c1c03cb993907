// Drop-in Set<T> (the reference's src/set/Set.hpp:14-132): a view of one set in
// a layout.  Rows handed out by SparseMatrix::get_row are host copies of the
// device rows in the reference's flattened format.
#ifndef EH_DROPIN_SET_HPP
#define EH_DROPIN_SET_HPP

#include "layouts/layouts.hpp"

template <class T>
class Set {
 public:
  uint8_t* data;
  size_t cardinality;
  size_t number_of_bytes;
  double density;
  common::type type;

  Set(uint8_t* data_in, size_t cardinality_in, size_t number_of_bytes_in, double density_in, common::type type_in)
      : data(data_in), cardinality(cardinality_in), number_of_bytes(number_of_bytes_in), density(density_in),
        type(type_in) {}
  Set(uint8_t* data_in, size_t cardinality_in, size_t number_of_bytes_in, common::type type_in)
      : data(data_in), cardinality(cardinality_in), number_of_bytes(number_of_bytes_in), density(0.0),
        type(type_in) {}
  explicit Set(uint8_t* data_in)
      : data(data_in), cardinality(0), number_of_bytes(0), density(0.0), type(T::get_type()) {}
  // A zeroed buffer of the given size (Set.hpp:47-56; like the reference, the
  // buffer belongs to the caller from here on).
  explicit Set(size_t number_of_bytes_in)
      : data(new uint8_t[number_of_bytes_in]()), cardinality(0), number_of_bytes(number_of_bytes_in),
        density(0.0), type(T::get_type()) {}
  Set(uint8_t* data_in, size_t number_of_bytes_in)
      : data(data_in), cardinality(0), number_of_bytes(number_of_bytes_in), density(0.0), type(T::get_type()) {}
  template <class U>
  Set(Set<U> in)
      : data(in.data), cardinality(in.cardinality), number_of_bytes(in.number_of_bytes), density(in.density),
        type(in.type) {}
  template <class U>
  Set(Set<U>* in)
      : data(in->data), cardinality(in->cardinality), number_of_bytes(in->number_of_bytes), density(in->density),
        type(in->type) {}

  // Copies another set's bytes and metadata (Set::copy_from, used by n_path).
  template <class U>
  void copy_from(const Set<U>& in) {
    std::memcpy(data, in.data, in.number_of_bytes);
    cardinality = in.cardinality;
    number_of_bytes = in.number_of_bytes;
    density = in.density;
    type = in.type;
  }

  template <typename F>
  void foreach(F f) const {
    T::foreach(f, data, cardinality, number_of_bytes, type);
  }
  template <typename F>
  void foreach_until(F f) const {
    T::foreach_until(f, data, cardinality, number_of_bytes, type);
  }

  // Set<T>::from_flattened (Set.hpp:172-176).
  static Set<T> from_flattened(uint8_t* set_data, size_t cardinality_in) {
    auto f = T::get_flattened_data(set_data, cardinality_in);
    return Set<T>(set_data + std::get<0>(f), cardinality_in, std::get<1>(f), std::get<2>(f));
  }
};

#include "ops.hpp"

#endif
