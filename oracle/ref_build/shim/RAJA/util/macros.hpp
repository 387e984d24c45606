#ifndef ORACLE_SHIM_RAJA_MACROS_HPP
#define ORACLE_SHIM_RAJA_MACROS_HPP
namespace RAJA { template <typename... T> inline void shim_unused(T&&...) {} }
#define RAJA_UNUSED_VAR(...) ::RAJA::shim_unused(__VA_ARGS__)
#define RAJA_UNUSED_ARG(x)
#define RAJA_INLINE inline
#define RAJA_HOST_DEVICE
#define RAJA_DEVICE
#endif
