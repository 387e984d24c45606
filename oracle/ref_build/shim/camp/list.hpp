#ifndef ORACLE_SHIM_CAMP_LIST_HPP
#define ORACLE_SHIM_CAMP_LIST_HPP
#include <cstddef>
#include <type_traits>
namespace camp {
template <typename... Ts> struct list {};
template <typename L> struct size;
template <typename... Ts>
struct size<list<Ts...>> : std::integral_constant<std::size_t, sizeof...(Ts)> {};
}
#endif
