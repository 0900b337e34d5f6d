// Minimal std-based stand-in for the one Boost.TypeTraits template the Dax
// hot-path headers use (dax/VectorTraits.h:21). Test infrastructure only.
#pragma once
#include <type_traits>
namespace boost {
template <class T> struct remove_const { typedef typename std::remove_const<T>::type type; };
}
