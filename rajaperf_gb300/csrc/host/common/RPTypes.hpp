// Basic data types of the suite's kernel interface (same names and meaning as
// the RAJA Performance Suite's common/RPTypes.hpp, so kernel code reads the
// same): FP64 reals, signed pointer-sized indices, long double checksums.
#pragma once

#include <cstddef>
#include <cstdint>

namespace rajaperf {

using RepIndex_type = volatile int;
using Index_type = std::ptrdiff_t;
using Index_ptr = Index_type*;
using Size_type = std::size_t;
using Int_type = int;
using Int_ptr = Int_type*;
using Checksum_type = long double;
using Real_type = double;
using Real_ptr = Real_type*;

}  // namespace rajaperf
