// ek_opcount.cpp -- op-counting build of the C restatement (ek_oracle.c).
//
// TEST AND MEASUREMENT INFRASTRUCTURE ONLY: it counts the floating-point
// operations the reference algorithm performs (implementationVersion 0, in
// the reference's own expression order), to give the step's algorithmic FLOPs
// per cell-update.  The CUDA product never links it.
//
// The restatement is compiled unchanged as C++ with its scalar type `double`
// replaced by `cdouble`, a one-double struct whose operators and math
// functions count each operation by kind before computing it in FP64.
// cdouble has the size, alignment and calling convention of double (a
// one-member floating-point aggregate is passed and returned in an FP
// register on x86-64 and AArch64), so the library exports the oracle's C API
// unchanged (eko.py loads it in place of libek_oracle.so) plus
// eko_ops_reset / eko_ops_read.
//
// What counts: + - * / (add, mul, div), sqrt, fmin/fmax, fabs/copysign,
// unary minus, and comparisons, one each per scalar operation.  Conversions,
// copies and index arithmetic are not counted.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <cstdint>

namespace
{
enum
{
  OP_ADD,
  OP_MUL,
  OP_DIV,
  OP_SQRT,
  OP_MINMAX,
  OP_ABS,
  OP_NEG,
  OP_CMP,
  OP_KINDS
};
unsigned long long g_ops[OP_KINDS];
} // namespace

struct cdouble
{
  double v;
  cdouble() = default;
  constexpr cdouble(double x)
    : v(x)
  {}
  explicit operator double() const { return v; }
  explicit operator float() const { return (float)v; }
  explicit operator int() const { return (int)v; }
  explicit operator long() const { return (long)v; }
  explicit operator bool() const { return v != 0.0; }
  cdouble & operator+=(cdouble o)
  {
    ++g_ops[OP_ADD];
    v += o.v;
    return *this;
  }
  cdouble & operator-=(cdouble o)
  {
    ++g_ops[OP_ADD];
    v -= o.v;
    return *this;
  }
  cdouble & operator*=(cdouble o)
  {
    ++g_ops[OP_MUL];
    v *= o.v;
    return *this;
  }
  cdouble & operator/=(cdouble o)
  {
    ++g_ops[OP_DIV];
    v /= o.v;
    return *this;
  }
};
static_assert(sizeof(cdouble) == sizeof(double) && alignof(cdouble) == alignof(double), "cdouble layout");

static inline cdouble
operator+(cdouble a, cdouble b)
{
  ++g_ops[OP_ADD];
  return a.v + b.v;
}
static inline cdouble
operator-(cdouble a, cdouble b)
{
  ++g_ops[OP_ADD];
  return a.v - b.v;
}
static inline cdouble
operator*(cdouble a, cdouble b)
{
  ++g_ops[OP_MUL];
  return a.v * b.v;
}
static inline cdouble
operator/(cdouble a, cdouble b)
{
  ++g_ops[OP_DIV];
  return a.v / b.v;
}
static inline cdouble
operator-(cdouble a)
{
  ++g_ops[OP_NEG];
  return -a.v;
}
static inline cdouble
operator+(cdouble a)
{
  return a;
}
#define EKO_CMP(op)                                                                                                    \
  static inline bool operator op(cdouble a, cdouble b)                                                                 \
  {                                                                                                                    \
    ++g_ops[OP_CMP];                                                                                                   \
    return a.v op b.v;                                                                                                 \
  }
EKO_CMP(<)
EKO_CMP(<=)
EKO_CMP(>)
EKO_CMP(>=)
EKO_CMP(==)
EKO_CMP(!=)
#undef EKO_CMP

static inline cdouble
sqrt(cdouble a)
{
  ++g_ops[OP_SQRT];
  return std::sqrt(a.v);
}
static inline cdouble
fabs(cdouble a)
{
  ++g_ops[OP_ABS];
  return std::fabs(a.v);
}
static inline cdouble
copysign(cdouble a, cdouble b)
{
  ++g_ops[OP_ABS];
  return std::copysign(a.v, b.v);
}
static inline cdouble
fmax(cdouble a, cdouble b)
{
  ++g_ops[OP_MINMAX];
  return std::fmax(a.v, b.v);
}
static inline cdouble
fmin(cdouble a, cdouble b)
{
  ++g_ops[OP_MINMAX];
  return std::fmin(a.v, b.v);
}

// the restatement itself, with cdouble as its scalar
#define double cdouble
#include "ek_oracle.c"
#undef double

extern "C" void
eko_ops_reset(void)
{
  for (int k = 0; k < OP_KINDS; ++k)
    g_ops[k] = 0;
}

// out[8]: add/sub, mul, div, sqrt, fmin/fmax, fabs/copysign, negation, comparison
extern "C" int
eko_ops_read(unsigned long long * out, int n)
{
  for (int k = 0; k < n && k < OP_KINDS; ++k)
    out[k] = g_ops[k];
  return OP_KINDS;
}
