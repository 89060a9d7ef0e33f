// Kokkos_StdAlgorithms.hpp -- shim of Kokkos::Experimental::swap, the only
// std-algorithm the reference uses (GateFunctors.hpp:92,120,146).
#pragma once
#include "Kokkos_Core.hpp"

namespace Kokkos {
namespace Experimental {
template <class T> inline void swap(T &a, T &b) {
    T t = a;
    a = b;
    b = t;
}
} // namespace Experimental
} // namespace Kokkos
