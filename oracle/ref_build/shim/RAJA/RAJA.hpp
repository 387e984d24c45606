// Umbrella stand-in for RAJA/RAJA.hpp. Only Base_Seq code paths are compiled
// against it (RUN_RAJA_SEQ, RUN_OPENMP and the GPU back ends stay undefined).
#ifndef ORACLE_SHIM_RAJA_HPP
#define ORACLE_SHIM_RAJA_HPP
#include "RAJA/config.hpp"
#include "RAJA/util/types.hpp"
#include "RAJA/util/macros.hpp"
#include "RAJA/util/Timer.hpp"
#include "RAJA/internal/MemUtils_CPU.hpp"
// RAJA's headers bring in the C string and algorithm headers that some
// kernels' Seq files use without including them (std::memcpy, std::sort).
#include <algorithm>
#include <cstring>
// Workgroup dispatch policy names that comm/HALO_base.hpp refers to in its
// RAJA-variant helpers (never instantiated by the Base_Seq code built here).
namespace RAJA {
template <typename... Ts> struct direct_dispatch {};
struct indirect_function_call_dispatch {};
struct indirect_virtual_function_dispatch {};
}  // namespace RAJA
#endif
