// Kokkos-API shim (test infrastructure only).
#include <Kokkos_Core.hpp>
