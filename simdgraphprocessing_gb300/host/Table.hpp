// Drop-in Table<T> / ParallelTable<T> (the reference's src/Table.hpp): column
// storage for result tuples.  The pattern apps only use the cardinality (tuple
// materialization is disabled in the reference, WRITE_TABLE == 0).
#ifndef EH_DROPIN_TABLE_HPP
#define EH_DROPIN_TABLE_HPP

#include <cstddef>
#include <fstream>
#include <string>

template <class T>
class Table {
 public:
  size_t num_columns;
  size_t column_size;
  size_t cardinality;
  T** data;
  T* tuple;
  Table(const size_t num_columns_in, const size_t column_size_in)
      : num_columns(num_columns_in), column_size(column_size_in), cardinality(0) {
    data = new T*[num_columns];
    tuple = new T[num_columns];
    for (size_t i = 0; i < num_columns; i++) data[i] = new T[column_size];
  }
  void print_data(std::ofstream& file) {
    for (size_t i = 0; i < cardinality; i++) {
      for (size_t j = 0; j < num_columns; j++) file << data[j][i] << "\t";
      file << std::endl;
    }
  }
};

template <class T>
class ParallelTable {
 public:
  Table<T>** table;
  size_t num_threads, num_columns, column_size, cardinality;
  ParallelTable(size_t num_threads_in, size_t num_columns_in, size_t column_size_in)
      : num_threads(num_threads_in), num_columns(num_columns_in), column_size(column_size_in), cardinality(0) {
    table = new Table<T>*[num_threads];
  }
  void allocate(size_t tid) { table[tid] = new Table<T>(num_columns, column_size); }
};

#endif
