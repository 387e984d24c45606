// Minimal stand-in for the RAJA configuration header, used only to compile
// the RAJA Performance Suite's own Base_Seq sources as a CPU oracle.
// The RAJA submodule is not vendored in the suite checkout; nothing here
// performs kernel arithmetic.
#ifndef ORACLE_SHIM_RAJA_CONFIG_HPP
#define ORACLE_SHIM_RAJA_CONFIG_HPP
#include <cstddef>
#endif
