/* Stand-in for the CMake-generated euler_kokkos_config.h of the reference,
 * used only to compile the reference oracle (oracle/_ref): double precision,
 * no MPI, no HDF5. */
#ifndef EULER_KOKKOS_CONFIG_H
#define EULER_KOKKOS_CONFIG_H 1
#define EULER_KOKKOS_USE_DOUBLE 1
#define EULER_KOKKOS_BUILD_TYPE "Release"
#define EULER_KOKKOS_BUILD_COMPILER_ID "GNU"
#define EULER_KOKKOS_BUILD_COMPILER_VERSION ""
#define EULER_KOKKOS_SYSTEM_PROCESSOR ""
#define EULER_KOKKOS_SYSTEM_NAME "Linux"
#define EULER_KOKKOS_MPI_VENDOR ""
#endif
