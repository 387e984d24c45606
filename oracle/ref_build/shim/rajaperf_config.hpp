// Hand-written equivalent of the suite's CMake-generated rajaperf_config.hpp
// for a host-only, sequential build: no MPI, no Caliper, no GPU back end,
// default GPU tuning lists.
#ifndef RAJAPerf_config_HPP
#define RAJAPerf_config_HPP
#include "RAJA/config.hpp"
#include "camp/number.hpp"
#include "camp/list.hpp"
#include <type_traits>
#include <string>

template < typename ... Ts >
inline void RAJAPERF_UNUSED_VAR(Ts&&...) { }
#define RAJAPERF_UNUSED_ARG(...)

namespace rajaperf {
namespace integer {
template < size_t... Is >
using list_type = camp::list< camp::integral_constant<size_t, Is>... >;
}
struct configuration {
  using gpu_block_sizes = integer::list_type<>;
  using atomic_replications = integer::list_type<>;
  using gpu_items_per_thread = integer::list_type<>;
  std::string user_run;
  std::string date_run;
  std::string systype_run;
  std::string machine_run;
};
using std::conjunction;
template <typename Func, typename... Ts>
inline void seq_for(camp::list<Ts...> const&, Func&& func)
{
  int order[] = {0, (func(Ts{}), 0)...};
  RAJAPERF_UNUSED_VAR(order);
}
}
#endif
