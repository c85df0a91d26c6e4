// Kokkos-API shim: random pool (test infrastructure only).
// The stream is NOT Kokkos' stream; reference runs that use random initial
// conditions are always overwritten by an injected initial state.
#ifndef EK_KOKKOS_SHIM_RANDOM_HPP
#define EK_KOKKOS_SHIM_RANDOM_HPP
#include <Kokkos_Core.hpp>
namespace Kokkos
{
struct ShimXorShift64
{
  uint64_t s;
  double drand()
  {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  }
  double drand(double a, double b) { return a + (b - a) * drand(); }
  float  frand() { return (float)drand(); }
};
template <class Dev>
struct Random_XorShift64_Pool
{
  using generator_type = ShimXorShift64;
  uint64_t seed;
  Random_XorShift64_Pool() : seed(1) {}
  explicit Random_XorShift64_Pool(uint64_t s) : seed(s ? s : 1) {}
  generator_type get_state() const { return generator_type{ seed * 0x9E3779B97F4A7C15ull + 1 }; }
  void free_state(const generator_type &) const {}
};
} // namespace Kokkos
#endif
