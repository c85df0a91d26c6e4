// Common device-side definitions for the fused MUSCL-Hancock kernels.
//
// Layout (identical to the reference's Kokkos::LayoutLeft device arrays,
// kokkos_shared.h:24-42): U[var][k][j][i], i fastest, ghost cells included.
// The step kernels never read the ghost cells stored in memory: a ghost
// coordinate is mapped to the interior cell the reference's boundary fill
// would copy from (BoundariesFunctors.h:17-1057), one dimension at a time.
// Because the reference fills the faces in the order x, y, z over the full
// transverse ranges (SolverBase.cpp:488-512), every edge/corner ghost ends up
// as the composition of the per-dimension maps, which is what this mapping
// computes.
#pragma once

#include <cstdint>
#include <cuda.h> // CUtensorMap (the type only; maps are encoded through the runtime's driver entry point)
#include <cuda_runtime.h>

#ifndef EK_NS
#define EK_NS ek_fast
#endif

namespace ekc
{

// variable indexes, enums.h:17-40
enum : int
{
  ID = 0,
  IP = 1,
  IU = 2,
  IV = 3,
  IW = 4,
  IA = 5,
  IB = 6,
  IC = 7
};

enum : int
{
  BC_DIRICHLET = 1, // reflecting
  BC_NEUMANN = 2,   // outflow / copy
  BC_PERIODIC = 3
};

struct KParams
{
  int       nx, ny, nz, gw;
  int       isize, jsize, ksize;
  int       mhd;
  long long plane;   // isize * jsize
  long long vstride; // isize * jsize * ksize: distance between variables
  int       bc[6];
  double    dx, dy, dz;
  double    gamma0, smallr, smallc, smallp, slope_type, cfl, tEnd, cIso;
  int       riemann;
  int       kchunk; // interior planes per CTA (3D kernels)
  // FP32 copies prepared on the host, so that mixed kernels do no per-thread
  // FP64 arithmetic (one FP64 instruction costs 64 FP32 ones on GB300)
  float     gamma0f, smallrf, smallcf, smallpf, slopef;
  float     idx, idy, idz; // 1/dx, 1/dy, 1/dz
  double    idxd, idyd, idzd; // 1/dx, 1/dy, 1/dz in FP64 (FP64 FMA build's CFL)
  int       mhd_stage;     // MHD update: stage the trace planes in shared memory
  double    gamma6, smallpp; // riemann_approx constants (HydroParams.cpp:353-356)
  float     gamma6f, smallppf;
  // static gravity (hydro; GravityParams.h:22-37): the field is gfield
  // (dim planes of the state's precision over the full grid) when set,
  // else the uniform vector g
  int          grav;         // source term + gravity CFL
  int          grav_hancock; // Hancock predictor of the face states
  double       g[3];
  float        gf[3];
  double       cfl_dxmin, dxmin; // cfl * min(dx, dy[, dz]) and min(dx, dy[, dz])
  float        cfl_dxminf, idxminf;
  const void * gfield;
};

// Per-step scalars kept on the device so that consecutive steps need no host
// round trip.  Slot s = step % 3 holds the max-reduced inverse time step
// (as an order-preserving integer key) and the time at the start of step.
// dt of a step and its FP64 ratios, computed once per step (step = -1: none)
struct StepConsts
{
  double t, dt, dtdx, dtdy, dtdz;
  int    step, active;
};
// Quotients by a shared denominator: the exact build divides each one, as the
// reference does; the FMA builds take one reciprocal and multiply (FP64: a
// division is a sequence of FMAs on GB300's 1/64-rate FP64 pipe).
#ifdef EK_EXACT_ONLY
constexpr bool kShareRecip = false;
#else
constexpr bool kShareRecip = true;
#endif

struct DevClock
{
  unsigned long long key[3];
  double             t[3];
  int                sid[3];    // step number the slot was written for
  int                iteration; // number of steps taken
  int                error;     // sticky device error flags
  double *           dtlog;     // dt of each step (capacity dtcap)
  int                dtcap;
  double             last_dt;   // dt of the last step taken (read with the clock)
  StepConsts         sc[3];     // per slot, by the last block of the CFL kernel
  unsigned int       fin[3];    // blocks of that kernel done (reset by the last)
};

enum : int
{
  EK_DEVERR_NONFINITE_DT = 1,
  EK_DEVERR_TMA_TIMEOUT = 2, // a tensor copy did not complete within its wait limit
};

// One instance of an ensemble of independent runs and one tile of work.
struct EnsInstance
{
  KParams    P;
  void *     U[2]; // ping-pong states
  DevClock * clk;
};
struct EnsTile
{
  int inst, bx, by;
};

// Mixed-precision MHD state: 5 FP32 hydro planes, then (256-byte aligned) the
// 3 FP64 face-field planes.
__host__ __device__ inline size_t
mixed_bfield_offset(long long vstride)
{
  return ((size_t)(5 * vstride * 4) + 255) / 256 * 256;
}
__host__ __device__ inline double *
mixed_bfield(void * U, const KParams & P)
{
  return (double *)((char *)U + mixed_bfield_offset(P.vstride));
}
__host__ __device__ inline const double *
mixed_bfield(const void * U, const KParams & P)
{
  return (const double *)((const char *)U + mixed_bfield_offset(P.vstride));
}

// order-preserving map double -> uint64 (total order on non-NaN values)
__host__ __device__ inline unsigned long long
dkey(double x)
{
  unsigned long long b;
#ifdef __CUDA_ARCH__
  b = (unsigned long long)__double_as_longlong(x);
#else
  memcpy(&b, &x, 8);
#endif
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__host__ __device__ inline double
dkey_inv(unsigned long long k)
{
  unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double x;
  memcpy(&x, &b, 8);
  return x;
#endif
}
// key of -DBL_MAX: the identity of the reference's Kokkos::Max reducer
#define EK_KEY_LOWEST 0x0010000000000000ull

} // namespace ekc

namespace EK_NS
{
using namespace ekc;
// Minimum resident CTAs per SM requested from the register allocator for the
// step kernels (FP32 / FP64 instantiations); overridable at build time.
#ifndef EK_H3_MINB_F32
#define EK_H3_MINB_F32 4
#endif
#ifndef EK_H3_MINB_F64
#define EK_H3_MINB_F64 2
#endif
#ifndef EK_MT_MINB_F32
#define EK_MT_MINB_F32 0
#endif
#ifndef EK_MT_MINB_F64
#define EK_MT_MINB_F64 0
#endif
#ifndef EK_MU_MINB_F32
#define EK_MU_MINB_F32 8
#endif
#ifndef EK_MU_MINB_F64
#define EK_MU_MINB_F64 1
#endif
#ifndef EK_M2_MINB_F32
#define EK_M2_MINB_F32 0
#endif
#ifndef EK_M2_MINB_F64
#define EK_M2_MINB_F64 0
#endif
#define EK_MINB(R, F32, F64) (sizeof(R) == 4 ? (F32) : (F64))
// Tile shapes (output cells per CTA in x, y) of the step kernels; the
// defaults are the measured best, euler_kokkos_gb300/tuning.py re-tunes them.
#ifndef EK_H2_TX
#define EK_H2_TX 32
#endif
#ifndef EK_H2_TY
#define EK_H2_TY 8
#endif
#ifndef EK_H3_TX
#define EK_H3_TX 32
#endif
#ifndef EK_H3_TY
#define EK_H3_TY 8
#endif
#ifndef EK_MT_TX
#define EK_MT_TX 32
#endif
#ifndef EK_MT_TY
#define EK_MT_TY 4
#endif
#ifndef EK_MU_TX
#define EK_MU_TX 16
#endif
#ifndef EK_MU_TY
#define EK_MU_TY 8
#endif
#ifndef EK_M2_TX
#define EK_M2_TX 16
#endif
#ifndef EK_M2_TY
#define EK_M2_TY 8
#endif


// FP64 <-> FP32 conversions on the integer pipes.  The hardware conversion
// instructions run on the FP64 unit, which issues at 1/64 of the FP32 rate on
// this GPU, so the mixed kernels convert the FP64 face fields this way.
// Normal results and zeros take the integer path and equal the hardware
// round-to-nearest-even conversion bit for bit; subnormal, overflowing,
// infinite and NaN values fall back to the hardware instruction.
__device__ __forceinline__ float
d2f_rn(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned           hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const unsigned           e = (hi >> 20) & 0x7ffu;
  if (e - 897u <= 253u)
  {
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;
    unsigned       f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(f);
  }
  if ((b << 1) == 0ull)
    return __uint_as_float(hi & 0x80000000u);
  return __double2float_rn(x);
}
__device__ __forceinline__ double
f2d(float x)
{
  const unsigned b = __float_as_uint(x);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u < 254u)
    return __hiloint2double((int)((b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3)),
                            (int)(b << 29));
  if ((b << 1) == 0u)
    return __hiloint2double((int)(b & 0x80000000u), 0);
  return (double)x;
}
// Approximate FP32 reciprocal, reciprocal square root and square root (one
// special-function-unit instruction each, about 1 ulp).  The mixed form uses
// them where the reference divides several numbers by one denominator or
// divides by a square root; the FP64 forms keep the reference's divisions.
__device__ __forceinline__ float
rcp_a(float x)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float
rsqrt_a(float x)
{
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float
sqrt_a(float x)
{
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Packed FP32 pairs: one instruction computes two lanes (sm_100 and later).
// The mixed form's solvers put the left and right states of a face in the two
// lanes; each lane rounds as the scalar operation does.
__device__ __forceinline__ float2
f2(float a, float b)
{
  return make_float2(a, b);
}
__device__ __forceinline__ float2
f2s(float a)
{
  return make_float2(a, a);
}
__device__ __forceinline__ float2
add2(float2 a, float2 b)
{
  return __fadd2_rn(a, b);
}
__device__ __forceinline__ float2
sub2(float2 a, float2 b)
{
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a); // b * -1 is exact: one rounding, as a - b
}
__device__ __forceinline__ float2
mul2(float2 a, float2 b)
{
  return __fmul2_rn(a, b);
}
__device__ __forceinline__ float2
fma2(float2 a, float2 b, float2 c)
{
  return __ffma2_rn(a, b, c);
}
__device__ __forceinline__ float2
neg2(float2 a)
{
  return make_float2(-a.x, -a.y);
}

// FP64 value in the working precision R
template <class R>
__device__ __forceinline__ R
to_r(double x)
{
  if constexpr (sizeof(R) == 4)
    return d2f_rn(x);
  else
    return x;
}

// Map a (possibly ghost) coordinate g in [0, n+2gw) of one dimension to the
// interior coordinate the boundary fill copies from; *flip is set when the
// reflecting wall flips the sign of the normal components.
__device__ __forceinline__ int
bc_map(int g, int n, int gw, int bc_lo, int bc_hi, bool * flip)
{
  // coordinates past the ghost layers only occur in the padding of partial
  // tiles; clamping keeps every read inside the array
  g = g < 0 ? 0 : (g > n + 2 * gw - 1 ? n + 2 * gw - 1 : g);
  if (g < gw)
  {
    if (bc_lo == BC_DIRICHLET)
    {
      *flip = !*flip;
      return 2 * gw - 1 - g;
    }
    if (bc_lo == BC_NEUMANN)
      return gw;
    return n + g;
  }
  if (g >= n + gw)
  {
    if (bc_hi == BC_DIRICHLET)
    {
      *flip = !*flip;
      return 2 * n + 2 * gw - 1 - g;
    }
    if (bc_hi == BC_NEUMANN)
      return n + gw - 1;
    return g - n;
  }
  return g;
}

// Source offset (in one variable plane) and per-dimension flips of a cell.
struct SrcCell
{
  long long off;
  bool      fx, fy, fz;
};

__device__ __forceinline__ SrcCell
src_cell(const KParams & P, int gi, int gj, int gk)
{
  SrcCell s;
  s.fx = s.fy = s.fz = false;
  int si = bc_map(gi, P.nx, P.gw, P.bc[0], P.bc[1], &s.fx);
  int sj = bc_map(gj, P.ny, P.gw, P.bc[2], P.bc[3], &s.fy);
  int sk = gk;
  if (P.ksize > 1)
    sk = bc_map(gk, P.nz, P.gw, P.bc[4], P.bc[5], &s.fz);
  s.off = (long long)sk * P.plane + (long long)sj * P.isize + si;
  return s;
}

// sign of variable v at a mapped cell: the reflecting fill multiplies the
// normal velocity (and, for MHD, the normal face field) by -1 per wall
__device__ __forceinline__ bool
flips(const SrcCell & s, int v, int mhd)
{
  bool f = false;
  if (v == IU || (mhd && v == IA))
    f ^= s.fx;
  if (v == IV || (mhd && v == IB))
    f ^= s.fy;
  if (v == IW || (mhd && v == IC))
    f ^= s.fz;
  return f;
}

// x or -x; the sign of a double is flipped with an integer XOR so that no
// FP64 instruction is issued (the result equals the FP64 negation bit for bit)
__device__ __forceinline__ double
neg_if(double x, bool f)
{
  return __longlong_as_double(__double_as_longlong(x) ^ (f ? (long long)0x8000000000000000ull : 0ll));
}
__device__ __forceinline__ float
neg_if(float x, bool f)
{
  return f ? -x : x;
}

template <class T>
__device__ __forceinline__ T
ldg(const T * p)
{
  return __ldg(p);
}

// dt at the start of a step, SolverBase::compute_dt (SolverBase.cpp:124-154).
// Returns false when the step must not run: the simulation is finished
// (SolverBase::finished, t >= tEnd - 1e-14, SolverBase.cpp:170-176) or an
// earlier launched step did not run (its slot was never committed).
__device__ __forceinline__ bool
step_dt(const KParams & P, const DevClock * clk, int step, double * t, double * dt)
{
  const int s = step % 3;
  if (clk->sid[s] != step)
    return false;
  const double invDt = dkey_inv(clk->key[s]);
  double       d = P.cfl / invDt;
  const double tt = clk->t[s];
  if (tt + d > P.tEnd)
    d = P.tEnd - tt;
  *t = tt;
  *dt = d;
  return !(tt >= P.tEnd - 1e-14);
}

// Step scalars computed once per CTA by thread 0 and shared: dt and the
// dt/dx ratios (the FP64 divisions would otherwise run in every thread).
template <class R>
struct StepScalars
{
  double t, dt;
  R      dtdx, dtdy, dtdz;
  int    active;
};
template <class R>
__device__ __forceinline__ bool
step_scalars(const KParams & P, const DevClock * clk, int step, StepScalars<R> * sh)
{
  if (threadIdx.x == 0)
  {
    double t, dt;
    sh->active = step_dt(P, clk, step, &t, &dt) ? 1 : 0;
    sh->t = t;
    sh->dt = dt;
    sh->dtdx = (R)(dt / P.dx);
    sh->dtdy = (R)(dt / P.dy);
    sh->dtdz = (R)(dt / P.dz);
  }
  __syncthreads();
  return sh->active != 0;
}

// Called by every block of the kernel that completes the CFL key of `step`
// (after its atomicMax): the last block to finish computes the step's dt and
// dt/dx ratios in FP64 once, for the step's kernels to read (step_consts), so
// that no block of those kernels runs the divisions behind a barrier.  The
// clock fields written by other blocks are read through volatile loads.
__device__ __forceinline__ void
finalize_step(DevClock * clk, const KParams & P, int step)
{
  __shared__ int last;
  __syncthreads();
  const int s = step % 3;
  if (threadIdx.x == 0)
  {
    __threadfence();
    const unsigned nb = gridDim.x * gridDim.y * gridDim.z;
    last = atomicAdd(&clk->fin[s], 1u) == nb - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0)
  {
    __threadfence();
    volatile DevClock * v = clk;
    StepConsts          c;
    c.step = step;
    c.active = 0;
    c.t = c.dt = c.dtdx = c.dtdy = c.dtdz = 0.0;
    if (v->sid[s] == step) // step_dt's arithmetic
    {
      const double invDt = dkey_inv(v->key[s]);
      double       d = P.cfl / invDt;
      const double tt = v->t[s];
      if (tt + d > P.tEnd)
        d = P.tEnd - tt;
      c.t = tt;
      c.dt = d;
      c.active = !(tt >= P.tEnd - 1e-14);
      c.dtdx = d / P.dx;
      c.dtdy = d / P.dy;
      c.dtdz = d / P.dz;
    }
    clk->sc[s] = c;
    clk->fin[s] = 0;
  }
}
// the constants of `step`; false when the step must not run (or they were
// not computed for it)
__device__ __forceinline__ bool
step_consts(const DevClock * clk, int step, StepConsts & c)
{
  c = clk->sc[step % 3];
  return c.step == step && c.active;
}

// Visit the interior cells of a state row by row: a block takes whole rows
// (j, k) with a grid stride and its threads take the cells of a row, so the
// index math needs one 32-bit division per row (a per-cell 64-bit division is
// a long software sequence).  f(i, j, k) gets ghost-inclusive indices.
template <class F>
__device__ __forceinline__ void
for_interior_rows(const KParams & P, F && f)
{
  const int nrows = P.ny * (P.ksize > 1 ? P.nz : 1);
  for (int row = blockIdx.x; row < nrows; row += gridDim.x)
  {
    const int j = row % P.ny + P.gw;
    const int k = P.ksize > 1 ? row / P.ny + P.gw : 0;
    for (int i = threadIdx.x + P.gw; i < P.nx + P.gw; i += blockDim.x)
      f(i, j, k);
  }
}
// blocks for a row-wise pass over the interior
__host__ __device__ inline int
row_blocks(const KParams & P)
{
  const long long nrows = (long long)P.ny * (P.ksize > 1 ? P.nz : 1);
  return (int)(nrows < 8192 ? nrows : 8192);
}

// bookkeeping done once per step by block 0, thread 0
__device__ __forceinline__ void
step_commit(DevClock * clk, int step, double t, double dt)
{
  clk->t[(step + 1) % 3] = t + dt;
  clk->sid[(step + 1) % 3] = step + 1;
  clk->key[(step + 2) % 3] = EK_KEY_LOWEST;
  if (step < clk->dtcap)
    clk->dtlog[step] = dt;
  clk->last_dt = dt;
  clk->iteration = step + 1;
}

// block-wide max of a thread-local key, then one atomicMax per block
template <int NT>
__device__ __forceinline__ void
block_max_commit(unsigned long long local, unsigned long long * dst)
{
  __shared__ unsigned long long red[NT / 32];
  for (int o = 16; o > 0; o >>= 1)
  {
    unsigned long long other = __shfl_xor_sync(0xffffffffu, local, o);
    local = other > local ? other : local;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    red[warp] = local;
  __syncthreads();
  if (warp == 0)
  {
    local = lane < NT / 32 ? red[lane] : 0ull;
    for (int o = 16; o > 0; o >>= 1)
    {
      unsigned long long other = __shfl_xor_sync(0xffffffffu, local, o);
      local = other > local ? other : local;
    }
    if (lane == 0)
      atomicMax(dst, local);
  }
}

// fmax semantics of the reference's reduction: a NaN candidate is ignored
__device__ __forceinline__ unsigned long long
cand_key(double v)
{
  return (v != v) ? 0ull : dkey(v);
}


// ---------------------------------------------------------------------------
// Tensor-memory-access (TMA) staging: one elected thread starts an
// asynchronous tiled copy global -> shared memory that completes on an
// mbarrier; the consumers wait on the barrier's phase.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned
smem_addr(const void * p)
{
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void
mbar_init(unsigned long long * bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
  // make the initialised barrier visible to the tensor-copy (async) proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// order this thread's earlier generic accesses of shared memory before the
// async-proxy writes of a tensor copy issued after it
__device__ __forceinline__ void
fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void
mbar_expect_tx(unsigned long long * bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// 4D tiled tensor copy of the box at (x, y, z, w) of *map into dst
__device__ __forceinline__ void
tma_load_4d(void * dst, const CUtensorMap * map, int x, int y, int z, int w, unsigned long long * bar)
{
  asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
               " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_addr(dst)),
               "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ unsigned long long
global_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// wait until phase `parity` of the barrier has completed; false when that
// has not happened within limit_ns (the caller reports the error and leaves)
__device__ __forceinline__ bool
mbar_wait(unsigned long long * bar, unsigned parity, unsigned long long limit_ns)
{
  const unsigned addr = smem_addr(bar);
  unsigned long long t0 = 0;
  for (int n = 0;; ++n)
  {
    unsigned done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(addr), "r"(parity)
                 : "memory");
    if (done)
      return true;
    const unsigned long long t = global_ns();
    if (n == 0)
      t0 = t;
    else if (t - t0 > limit_ns)
      return false;
  }
}


// Per-thread asynchronous copies global -> shared memory (element gathers
// whose source addresses follow the boundary mapping); completion is waited
// for by the issuing thread (cp.async.wait_all) before a block barrier.
template <int BYTES>
__device__ __forceinline__ void
cp_async(void * dst, const void * src)
{
  static_assert(BYTES == 4 || BYTES == 8, "cp.async element size");
  if constexpr (BYTES == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void
cp_async_commit()
{
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void
cp_async_wait_all()
{
  asm volatile("cp.async.wait_all;" ::: "memory");
}

} // namespace EK_NS
