// Stand-in for RAJA/util/types.hpp: the suite's Index_type is RAJA::Index_type,
// a signed pointer-sized integer.
#ifndef ORACLE_SHIM_RAJA_TYPES_HPP
#define ORACLE_SHIM_RAJA_TYPES_HPP
#include <cstddef>
#include <utility>
namespace RAJA {
constexpr int DATA_ALIGN = 64;
using Index_type = std::ptrdiff_t;
using idx_t = std::ptrdiff_t;
}
#endif
