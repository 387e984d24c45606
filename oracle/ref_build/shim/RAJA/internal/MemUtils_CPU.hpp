// Stand-in for RAJA's aligned host allocation helpers.
#ifndef ORACLE_SHIM_RAJA_MEMUTILS_HPP
#define ORACLE_SHIM_RAJA_MEMUTILS_HPP
#include <cstdlib>
#include <cstddef>
#include "RAJA/util/types.hpp"
namespace RAJA {
template <typename T>
inline T* allocate_aligned_type(std::size_t align, std::size_t nbytes) {
  std::size_t rounded = (nbytes + align - 1) / align * align;
  if (rounded == 0) rounded = align;
  return static_cast<T*>(std::aligned_alloc(align, rounded));
}
inline void free_aligned(void* p) { std::free(p); }
}
#endif
