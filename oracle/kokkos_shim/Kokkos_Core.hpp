// Minimal Kokkos-API-compatible host shim (test infrastructure only).
//
// The reference solver (pkestene/euler_kokkos) is written against Kokkos 5.x,
// which is not available offline.  This header provides the small subset of the
// public Kokkos API that the reference's solver sources use, so that those
// sources compile unmodified with g++ and run on the host (serial, or OpenMP
// when compiled with -fopenmp).  It is written from the public Kokkos API
// documentation, not from Kokkos sources, and is used only to build the
// reference oracle under oracle/_ref.  Nothing in the product links it.
#ifndef EK_KOKKOS_SHIM_CORE_HPP
#define EK_KOKKOS_SHIM_CORE_HPP

#include <Kokkos_Macros.hpp>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <iostream>
#include <limits>
#include <memory>
#include <sstream>
#include <fstream>
#include <iomanip>
#include <vector>
#include <map>
#include <string>
#include <type_traits>

namespace Kokkos
{

// ---------------------------------------------------------------- spaces
struct HostSpace
{
  using memory_space = HostSpace;
};
struct Serial
{
  using memory_space = HostSpace;
  using execution_space = Serial;
  static const char * name() { return "Serial(shim)"; }
  void fence() const {}
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

template <class ExecSpace, class MemSpace>
struct Device
{
  using execution_space = ExecSpace;
  using memory_space = MemSpace;
};

struct LayoutLeft
{};
struct LayoutRight
{};

inline void initialize(int &, char **&) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string &) {}
inline void print_configuration(std::ostream & os, bool = false)
{
  os << "Kokkos API shim (host, "
#ifdef _OPENMP
     << "OpenMP"
#else
     << "serial"
#endif
     << ")\n";
}

namespace hwloc
{
inline bool available() { return false; }
inline unsigned get_available_numa_count() { return 1; }
inline unsigned get_available_cores_per_numa() { return 1; }
inline unsigned get_available_threads_per_core() { return 1; }
} // namespace hwloc

// ---------------------------------------------------------------- math
using std::abs;
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::fmod;
using std::isnan;
using std::sqrt;
namespace Experimental
{
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::fmod;
using std::isnan;
using std::sqrt;
} // namespace Experimental

// ---------------------------------------------------------------- Array
template <class T, std::size_t N>
struct Array
{
  T m_data[N > 0 ? N : 1];
  KOKKOS_INLINE_FUNCTION T &       operator[](std::size_t i) { return m_data[i]; }
  KOKKOS_INLINE_FUNCTION const T & operator[](std::size_t i) const { return m_data[i]; }
  static constexpr std::size_t     size() { return N; }
  T *                              data() { return m_data; }
  const T *                        data() const { return m_data; }
};

// ---------------------------------------------------------------- View
namespace shim_detail
{
// Split a Kokkos data type such as double***[3] into value type, number of
// runtime extents and the trailing static extents.
template <class T>
struct DataTypeInfo
{
  using value_type = T;
  static constexpr int n_dyn = 0;
  static constexpr int n_static = 0;
  static void          static_extents(std::size_t *) {}
};
template <class T>
struct DataTypeInfo<T *>
{
  using value_type = typename DataTypeInfo<T>::value_type;
  static constexpr int n_dyn = DataTypeInfo<T>::n_dyn + 1;
  static constexpr int n_static = DataTypeInfo<T>::n_static;
  static void          static_extents(std::size_t * e) { DataTypeInfo<T>::static_extents(e); }
};
template <class T, std::size_t N>
struct DataTypeInfo<T[N]>
{
  using value_type = typename DataTypeInfo<T>::value_type;
  static constexpr int n_dyn = DataTypeInfo<T>::n_dyn;
  static constexpr int n_static = DataTypeInfo<T>::n_static + 1;
  // static extents are listed left to right after the dynamic ones
  static void static_extents(std::size_t * e)
  {
    e[0] = N;
    DataTypeInfo<T>::static_extents(e + 1);
  }
};

template <class... P>
struct LayoutOf
{
  using type = LayoutRight; // host default, as the OpenMP backend
};
template <class... P>
struct LayoutOf<LayoutLeft, P...>
{
  using type = LayoutLeft;
};
template <class... P>
struct LayoutOf<LayoutRight, P...>
{
  using type = LayoutRight;
};
template <class First, class... P>
struct LayoutOf<First, P...>
{
  using type = typename LayoutOf<P...>::type;
};
} // namespace shim_detail

template <class DataType, class... Props>
class View
{
public:
  using info = shim_detail::DataTypeInfo<DataType>;
  using value_type = typename info::value_type;
  using non_const_value_type = typename std::remove_const<value_type>::type;
  using layout_type = typename shim_detail::LayoutOf<Props...>::type;
  using array_layout = layout_type;
  static constexpr int rank = info::n_dyn + info::n_static;
  using host_mirror_type = View<DataType, layout_type, HostSpace>;
  using HostMirror = host_mirror_type;
  using memory_space = HostSpace;
  using execution_space = Serial;

  View() = default;

  template <class... Ints>
  explicit View(const std::string & label, Ints... n)
    : m_label(label)
  {
    static_assert(sizeof...(Ints) <= 8, "too many extents");
    std::size_t dyn[] = { static_cast<std::size_t>(n)..., 0 };
    for (int r = 0; r < 8; ++r)
      m_ext[r] = 1;
    for (int r = 0; r < info::n_dyn; ++r)
      m_ext[r] = r < (int)sizeof...(Ints) ? dyn[r] : 1;
    info::static_extents(m_ext + info::n_dyn);
    std::size_t total = 1;
    for (int r = 0; r < rank; ++r)
      total *= m_ext[r];
    m_size = total;
    m_data = std::shared_ptr<non_const_value_type>(new non_const_value_type[total ? total : 1](),
                                                   std::default_delete<non_const_value_type[]>());
    compute_strides();
  }

  // Conversion between views of equal element type and rank (the reference
  // passes a View<T****> where a View<T***[3]> is declared).
  template <class D2, class... P2>
  View(const View<D2, P2...> & o)
  {
    static_assert(View<D2, P2...>::rank == rank, "rank mismatch in shim view conversion");
    m_label = o.m_label;
    m_data = o.m_data;
    m_size = o.m_size;
    for (int r = 0; r < 8; ++r)
    {
      m_ext[r] = o.m_ext[r];
      m_stride[r] = o.m_stride[r];
    }
  }

  std::size_t extent(int r) const { return r < rank ? m_ext[r] : 1; }
  int         extent_int(int r) const { return (int)extent(r); }
  std::size_t size() const { return m_size; }
  std::size_t span() const { return m_size; }
  value_type * data() const { return m_data.get(); }
  const std::string & label() const { return m_label; }
  bool is_allocated() const { return (bool)m_data; }

  template <class... I>
  KOKKOS_INLINE_FUNCTION value_type & operator()(I... idx) const
  {
    std::size_t ii[] = { static_cast<std::size_t>(idx)..., 0 };
    std::size_t off = 0;
    for (int r = 0; r < (int)sizeof...(I); ++r)
    {
#ifdef EK_SHIM_BOUNDS_CHECK
      if (ii[r] >= m_ext[r])
      {
        std::fprintf(stderr, "shim View %s: index %zu out of bounds (%zu) in dim %d\n",
                     m_label.c_str(), ii[r], m_ext[r], r);
        std::abort();
      }
#endif
      off += ii[r] * m_stride[r];
    }
    return m_data.get()[off];
  }

  // public so that conversions can read them
  std::string                           m_label;
  std::shared_ptr<non_const_value_type> m_data;
  std::size_t                           m_ext[8] = { 1, 1, 1, 1, 1, 1, 1, 1 };
  std::size_t                           m_stride[8] = { 0, 0, 0, 0, 0, 0, 0, 0 };
  std::size_t                           m_size = 0;

private:
  void compute_strides()
  {
    if (std::is_same<layout_type, LayoutLeft>::value)
    {
      std::size_t s = 1;
      for (int r = 0; r < rank; ++r)
      {
        m_stride[r] = s;
        s *= m_ext[r];
      }
    }
    else
    {
      std::size_t s = 1;
      for (int r = rank - 1; r >= 0; --r)
      {
        m_stride[r] = s;
        s *= m_ext[r];
      }
    }
  }
};

template <class D, class... P>
typename View<D, P...>::host_mirror_type
create_mirror(const View<D, P...> & v)
{
  typename View<D, P...>::host_mirror_type m(
    v.label() + "_mirror", v.extent(0), v.extent(1), v.extent(2), v.extent(3), v.extent(4));
  return m;
}
template <class D, class... P>
typename View<D, P...>::host_mirror_type
create_mirror_view(const View<D, P...> & v)
{
  return v;
}

template <class D1, class... P1, class D2, class... P2>
void
deep_copy(const View<D1, P1...> & dst, const View<D2, P2...> & src)
{
  assert(dst.size() == src.size());
  if (dst.data() == src.data())
    return;
  std::memcpy((void *)dst.data(), (const void *)src.data(),
              sizeof(typename View<D1, P1...>::value_type) * dst.size());
}
template <class D1, class... P1>
void
deep_copy(const View<D1, P1...> & dst, const typename View<D1, P1...>::value_type & val)
{
  for (std::size_t i = 0; i < dst.size(); ++i)
    dst.data()[i] = val;
}

// ---------------------------------------------------------------- policies
template <unsigned N>
struct Rank
{
  static constexpr unsigned rank = N;
};

template <class... Args>
struct RangePolicy;
template <>
struct RangePolicy<>
{
  using tag = void;
  long begin, end;
  RangePolicy(long b, long e)
    : begin(b)
    , end(e)
  {}
};
template <class Tag>
struct RangePolicy<Tag>
{
  using tag = Tag;
  long begin, end;
  RangePolicy(long b, long e)
    : begin(b)
    , end(e)
  {}
};

template <class R, class Tag = void>
struct MDRangePolicy
{
  using tag = Tag;
  static constexpr unsigned rank = R::rank;
  long                      lo[3] = { 0, 0, 0 };
  long                      hi[3] = { 1, 1, 1 };
  MDRangePolicy(std::initializer_list<long> b, std::initializer_list<long> e)
  {
    int r = 0;
    for (long v : b)
      lo[r++] = v;
    r = 0;
    for (long v : e)
      hi[r++] = v;
  }
  template <class B, class E>
  MDRangePolicy(B, E, std::initializer_list<long>)
  {}
};

namespace shim_detail
{
template <class Tag, class F, class... I>
inline void
invoke(const F & f, I... i)
{
  if constexpr (std::is_void<Tag>::value)
    f(i...);
  else
    f(Tag(), i...);
}
template <class Tag, class F, class V, class... I>
inline void
invoke_reduce(const F & f, V & v, I... i)
{
  if constexpr (std::is_void<Tag>::value)
    f(i..., v);
  else
    f(Tag(), i..., v);
}
} // namespace shim_detail

template <class... A, class F>
void
parallel_for(const RangePolicy<A...> & p, const F & f)
{
  using Tag = typename RangePolicy<A...>::tag;
#pragma omp parallel for schedule(static)
  for (long i = p.begin; i < p.end; ++i)
    shim_detail::invoke<Tag>(f, (int)i);
}
template <class R, class T, class F>
void
parallel_for(const MDRangePolicy<R, T> & p, const F & f)
{
  using Tag = T;
  if constexpr (R::rank == 2)
  {
#pragma omp parallel for collapse(2) schedule(static)
    for (long i = p.lo[0]; i < p.hi[0]; ++i)
      for (long j = p.lo[1]; j < p.hi[1]; ++j)
        shim_detail::invoke<Tag>(f, (int)i, (int)j);
  }
  else
  {
#pragma omp parallel for collapse(3) schedule(static)
    for (long i = p.lo[0]; i < p.hi[0]; ++i)
      for (long j = p.lo[1]; j < p.hi[1]; ++j)
        for (long k = p.lo[2]; k < p.hi[2]; ++k)
          shim_detail::invoke<Tag>(f, (int)i, (int)j, (int)k);
  }
}
template <class P, class F>
void
parallel_for(const std::string &, const P & p, const F & f)
{
  parallel_for(p, f);
}
template <class P, class F>
void
parallel_for(const char * s, const P & p, const F & f)
{
  parallel_for(p, f);
}

// reducers
template <class T>
struct Max
{
  T & ref;
  explicit Max(T & r)
    : ref(r)
  {}
  static T identity() { return std::numeric_limits<T>::lowest(); }
  static void join(T & a, const T & b) { a = (b > a) ? b : a; }
};
template <class T>
struct Min
{
  T & ref;
  explicit Min(T & r)
    : ref(r)
  {}
  static T identity() { return std::numeric_limits<T>::max(); }
  static void join(T & a, const T & b) { a = (b < a) ? b : a; }
};
template <class T>
struct Sum
{
  T & ref;
  explicit Sum(T & r)
    : ref(r)
  {}
  static T identity() { return T(0); }
  static void join(T & a, const T & b) { a += b; }
};

template <class Red>
struct is_reducer : std::false_type
{};
template <class T>
struct is_reducer<Max<T>> : std::true_type
{};
template <class T>
struct is_reducer<Min<T>> : std::true_type
{};
template <class T>
struct is_reducer<Sum<T>> : std::true_type
{};

namespace shim_detail
{
template <class Red, class T, class F, class P>
void
reduce_impl(const P & p, const F & f, T & result)
{
  T total = Red::identity();
  if constexpr (std::is_same<P, RangePolicy<>>::value || std::is_same<P, RangePolicy<typename P::tag>>::value)
  {
#pragma omp parallel
    {
      T local = Red::identity();
#pragma omp for schedule(static)
      for (long i = p.begin; i < p.end; ++i)
        shim_detail::invoke_reduce<typename P::tag>(f, local, (int)i);
#pragma omp critical
      Red::join(total, local);
    }
  }
  else if constexpr (P::rank == 2)
  {
#pragma omp parallel
    {
      T local = Red::identity();
#pragma omp for collapse(2) schedule(static)
      for (long i = p.lo[0]; i < p.hi[0]; ++i)
        for (long j = p.lo[1]; j < p.hi[1]; ++j)
          shim_detail::invoke_reduce<typename P::tag>(f, local, (int)i, (int)j);
#pragma omp critical
      Red::join(total, local);
    }
  }
  else
  {
#pragma omp parallel
    {
      T local = Red::identity();
#pragma omp for collapse(3) schedule(static)
      for (long i = p.lo[0]; i < p.hi[0]; ++i)
        for (long j = p.lo[1]; j < p.hi[1]; ++j)
          for (long k = p.lo[2]; k < p.hi[2]; ++k)
            shim_detail::invoke_reduce<typename P::tag>(f, local, (int)i, (int)j, (int)k);
#pragma omp critical
      Red::join(total, local);
    }
  }
  result = total;
}
} // namespace shim_detail

template <class P, class F, class T>
void
parallel_reduce(const P & p, const F & f, Max<T> r)
{
  shim_detail::reduce_impl<Max<T>>(p, f, r.ref);
}
template <class P, class F, class T>
void
parallel_reduce(const P & p, const F & f, Min<T> r)
{
  shim_detail::reduce_impl<Min<T>>(p, f, r.ref);
}
template <class P, class F, class T>
void
parallel_reduce(const std::string &, const P & p, const F & f, T r)
{
  parallel_reduce(p, f, r);
}
template <class P, class F, class T>
void
parallel_reduce(const char *, const P & p, const F & f, T r)
{
  parallel_reduce(p, f, r);
}

// atomics (host: plain or omp atomic)
template <class T>
inline void
atomic_add(T * p, T v)
{
#pragma omp atomic
  *p += v;
}
template <class T>
inline void
atomic_sub(T * p, T v)
{
#pragma omp atomic
  *p -= v;
}

} // namespace Kokkos

#endif // EK_KOKKOS_SHIM_CORE_HPP
