// Drop-in ParallelBuffer<T> (the reference's src/ParallelBuffer.hpp): one host
// buffer per thread id.  The device kernels keep their per-thread state in
// registers and shared memory; this stays for host code that uses it.
#ifndef EH_DROPIN_PARALLELBUFFER_HPP
#define EH_DROPIN_PARALLELBUFFER_HPP

#include <cstddef>

template <class T>
class ParallelBuffer {
 public:
  size_t num_threads;
  size_t size;
  T** data;
  ParallelBuffer(size_t num_threads_in, size_t size_in) : num_threads(num_threads_in), size(size_in) {
    data = new T*[num_threads];
    for (size_t i = 0; i < num_threads; i++) data[i] = nullptr;
  }
  void allocate(size_t tid) { data[tid] = new T[size]; }
  void unallocate(size_t tid) {
    delete[] data[tid];
    data[tid] = nullptr;
  }
  ~ParallelBuffer() {}
};

#endif
