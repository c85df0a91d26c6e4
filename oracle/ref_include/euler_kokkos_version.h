/* Stand-in for the CMake-generated euler_kokkos_version.h of the reference
 * (its version from CMakeLists.txt:52, no git information), used only to
 * compile the reference's own main.cpp against the Kokkos-API shim. */
#ifndef EULER_KOKKOS_VERSION_H_
#define EULER_KOKKOS_VERSION_H_
#define EULER_KOKKOS_VERSION "0.9.0"
#define EULER_KOKKOS_COMPILE_DATE ""
#define EULER_KOKKOS_COMPILE_TIME ""
#endif
