// Kokkos-API shim: macros (test infrastructure only; see Kokkos_Core.hpp).
#ifndef EK_KOKKOS_SHIM_MACROS_HPP
#define EK_KOKKOS_SHIM_MACROS_HPP
#define KOKKOS_VERSION 50100
#define KOKKOS_VERSION_MAJOR 5
#define KOKKOS_VERSION_MINOR 1
#define KOKKOS_ENABLE_CXX17 1
#define KOKKOS_ENABLE_SERIAL 1
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]
#include <cassert>
#define KOKKOS_ASSERT(x) assert(x)
#endif
