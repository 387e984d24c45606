#ifndef ORACLE_SHIM_CAMP_NUMBER_HPP
#define ORACLE_SHIM_CAMP_NUMBER_HPP
#include <type_traits>
#include <cstddef>
namespace camp {
template <typename T, T v> using integral_constant = std::integral_constant<T, v>;
template <std::size_t v> using num = std::integral_constant<std::size_t, v>;
}
#endif
