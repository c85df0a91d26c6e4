// Kernel instantiations and launchers.  Compiled twice (see ek_launch.h):
//   -DEK_NS=ek_exact --fmad=false   FP64 only, bitwise parity build
//   -DEK_NS=ek_fast  --fmad=true    FP64 + mixed FP32
#include <cstring>

#include "ek_launch.h"
#include "ek_hydro_kernels.cuh"
#include "ek_mhd_kernels.cuh"
#include "ek_mhd2d_kernels.cuh"

namespace EK_NS
{

namespace
{
constexpr int H2_TX = EK_H2_TX, H2_TY = EK_H2_TY;
constexpr int H3_TX = EK_H3_TX, H3_TY = EK_H3_TY;

template <class R>
constexpr size_t
hydro2d_smem()
{
  constexpr int NV = 4, HX = H2_TX + 4, HY = H2_TY + 4;
  return sizeof(R) * (NV * HY * HX + 2 * NV * H2_TY * (H2_TX + 2) + 2 * NV * (H2_TY + 2) * H2_TX);
}
template <class R>
constexpr size_t
hydro3d_smem()
{
  // three padded ring slots and the face buffers
  constexpr int NV = 5;
  return sizeof(R) * (3 * hydro3d_slot_elems<R, H3_TX, H3_TY>() + 2 * NV * H3_TY * (H3_TX + 2) +
                      2 * NV * (H3_TY + 2) * H3_TX);
}

template <class S, class R, int RS, bool GRAV>
cudaError_t
hydro_step_rs(int dim, const void * Uin, void * Uout, const KParams & P, DevClock * clk, int step,
              const CUtensorMap * tmap, cudaStream_t st)
{
  if (dim == 2)
  {
    auto   k = hydro2d_step<S, R, H2_TX, H2_TY, RS, GRAV>;
    size_t sm = hydro2d_smem<R>();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess)
      return e;
    dim3 grid((P.nx + H2_TX - 1) / H2_TX, (P.ny + H2_TY - 1) / H2_TY, 1);
    k<<<grid, H2_TX * H2_TY, sm, st>>>((const S *)Uin, (S *)Uout, P, clk, step);
    return cudaGetLastError();
  }
  if constexpr (RS == 2)
  {
    // riemann_hydro for 3D states has no HLL branch (RiemannSolvers.h:608-640)
    return cudaErrorNotSupported;
  }
  else
  {
    // interior planes staged by tensor copies when Uin has a tensor map
    auto        k = tmap ? hydro3d_step<S, R, H3_TX, H3_TY, RS, GRAV, true>
                         : hydro3d_step<S, R, H3_TX, H3_TY, RS, GRAV, false>;
    size_t      sm = hydro3d_smem<R>();
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess)
      return e;
    dim3 grid((P.nx + H3_TX - 1) / H3_TX, (P.ny + H3_TY - 1) / H3_TY, (P.nz + P.kchunk - 1) / P.kchunk);
    CUtensorMap m;
    std::memset(&m, 0, sizeof m);
    if (tmap)
      m = *tmap;
    k<<<grid, H3_TX * H3_TY, sm, st>>>((const S *)Uin, (S *)Uout, P, clk, step, m);
    return cudaGetLastError();
  }
}

// the Riemann solver and static gravity are template parameters of the step
// kernels
template <class S, class R, bool GRAV>
cudaError_t
hydro_step_g(int dim, const void * Uin, void * Uout, const KParams & P, DevClock * clk, int step,
             const CUtensorMap * tmap, cudaStream_t st)
{
  switch (P.riemann)
  {
    case 0: return hydro_step_rs<S, R, 0, GRAV>(dim, Uin, Uout, P, clk, step, tmap, st);
    case 1: return hydro_step_rs<S, R, 1, GRAV>(dim, Uin, Uout, P, clk, step, tmap, st);
    case 2: return hydro_step_rs<S, R, 2, GRAV>(dim, Uin, Uout, P, clk, step, tmap, st);
    case 3: return hydro_step_rs<S, R, 3, GRAV>(dim, Uin, Uout, P, clk, step, tmap, st);
  }
  return cudaErrorNotSupported;
}

template <class S, class R>
cudaError_t
hydro_step_t(int dim, const void * Uin, void * Uout, const KParams & P, DevClock * clk, int step,
             const CUtensorMap * tmap, cudaStream_t st)
{
  return P.grav ? hydro_step_g<S, R, true>(dim, Uin, Uout, P, clk, step, tmap, st)
                : hydro_step_g<S, R, false>(dim, Uin, Uout, P, clk, step, tmap, st);
}

template <class S, class R>
cudaError_t
hydro_dt_t(int dim, const void * U, const KParams & P, unsigned long long * key, DevClock * fin, int fin_step,
           cudaStream_t st)
{
  const int blocks = row_blocks(P);
  if (dim == 2 && P.grav)
    hydro_dt_kernel<S, R, 4, true><<<blocks, 256, 0, st>>>((const S *)U, P, key, fin, fin_step);
  else if (dim == 2)
    hydro_dt_kernel<S, R, 4, false><<<blocks, 256, 0, st>>>((const S *)U, P, key, fin, fin_step);
  else if (P.grav)
    hydro_dt_kernel<S, R, 5, true><<<blocks, 256, 0, st>>>((const S *)U, P, key, fin, fin_step);
  else
    hydro_dt_kernel<S, R, 5, false><<<blocks, 256, 0, st>>>((const S *)U, P, key, fin, fin_step);
  return cudaGetLastError();
}
} // namespace

cudaError_t
hydro_step(int dim, int prec, const void * Uin, void * Uout, const KParams & P, DevClock * clk,
           int step, const CUtensorMap * tmap, cudaStream_t st)
{
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  return hydro_step_t<double, double>(dim, Uin, Uout, P, clk, step, tmap, st);
#else
  if (prec == 0)
    return hydro_step_t<double, double>(dim, Uin, Uout, P, clk, step, tmap, st);
  return hydro_step_t<float, float>(dim, Uin, Uout, P, clk, step, tmap, st);
#endif
}

cudaError_t
hydro_dt(int dim, int prec, const void * U, const KParams & P, unsigned long long * key, DevClock * fin,
         int fin_step, cudaStream_t st)
{
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  return hydro_dt_t<double, double>(dim, U, P, key, fin, fin_step, st);
#else
  if (prec == 0)
    return hydro_dt_t<double, double>(dim, U, P, key, fin, fin_step, st);
  return hydro_dt_t<float, float>(dim, U, P, key, fin, fin_step, st);
#endif
}

namespace
{
template <class S, class R>
cudaError_t
ensemble2d_t(const EnsInstance * insts, int n, const EnsTile * tiles, int ntiles, int * stepc, void * scal,
             int grid, cudaStream_t st)
{
  static_assert(sizeof(StepScalars<R>) <= 64, "per-instance step scalars are allocated 64 bytes each");
  StepScalars<R> * sc = static_cast<StepScalars<R> *>(scal);
  ensemble_scalars_kernel<R><<<(n + 127) / 128, 128, 0, st>>>(insts, n, stepc, sc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return e;
  auto   k = ensemble2d_step<S, R, H2_TX, H2_TY>;
  size_t sm = hydro2d_smem<R>() + ensemble_raw_bytes<S, R, H2_TX, H2_TY>();
  e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess)
    return e;
  k<<<grid, H2_TX * H2_TY, sm, st>>>(insts, tiles, ntiles, stepc, hydro2d_smem<R>(), sc);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return e;
  ensemble_advance<<<1, 1, 0, st>>>(stepc);
  return cudaGetLastError();
}
template <class S, class R>
int
ensemble2d_grid_t()
{
  auto   k = ensemble2d_step<S, R, H2_TX, H2_TY>;
  size_t sm = hydro2d_smem<R>() + ensemble_raw_bytes<S, R, H2_TX, H2_TY>();
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int per_sm = 0, dev = 0, nsm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, H2_TX * H2_TY, sm);
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  return (per_sm > 0 ? per_sm : 1) * (nsm > 0 ? nsm : 1);
}
} // namespace

cudaError_t
ensemble2d_step(int prec, const EnsInstance * insts, int n, const EnsTile * tiles, int ntiles, int * stepc,
                void * scal, int grid, cudaStream_t st)
{
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  return ensemble2d_t<double, double>(insts, n, tiles, ntiles, stepc, scal, grid, st);
#else
  if (prec == 0)
    return ensemble2d_t<double, double>(insts, n, tiles, ntiles, stepc, scal, grid, st);
  return ensemble2d_t<float, float>(insts, n, tiles, ntiles, stepc, scal, grid, st);
#endif
}

int
ensemble2d_grid(int prec)
{
#ifdef EK_EXACT_ONLY
  return ensemble2d_grid_t<double, double>();
#else
  return prec == 0 ? ensemble2d_grid_t<double, double>() : ensemble2d_grid_t<float, float>();
#endif
}

#ifndef EK_EXACT_ONLY
namespace
{
__global__ void
bounded_wait_kernel(unsigned long long limit_ns, unsigned long long * out)
{
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0)
    mbar_init(&bar, 1); // one arrival expected; none comes
  __syncthreads();
  const unsigned long long t0 = global_ns();
  const bool               ok = mbar_wait(&bar, 0u, limit_ns);
  const unsigned long long dt = global_ns() - t0;
  if (!ok)
    atomicAdd(out, 1ull);
  atomicMax(out + 1, dt);
}

// CUDA-core FMA throughput: every thread runs 8 independent FMA chains
// (x = x * a + b), 16 steps unrolled per loop trip, so the FMA pipe never
// waits on a dependency; the sum of the chains is stored so none is dead.
template <class T>
__global__ void __launch_bounds__(256)
fma_rate_kernel(T * out, int iters, T a, T b)
{
  T x[8];
#pragma unroll
  for (int c = 0; c < 8; ++c)
    x[c] = (T)(threadIdx.x + c);
  for (int i = 0; i < iters; ++i)
  {
#pragma unroll
    for (int u = 0; u < 16; ++u)
    {
#pragma unroll
      for (int c = 0; c < 8; ++c)
        x[c] = fma(x[c], a, b);
    }
  }
  T acc = x[0];
#pragma unroll
  for (int c = 1; c < 8; ++c)
    acc += x[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}
} // namespace

cudaError_t
fma_rate(int prec, int blocks, int iters, void * out, cudaStream_t st)
{
  if (prec == 0)
    fma_rate_kernel<double><<<blocks, 256, 0, st>>>((double *)out, iters, 0.999, 0.001);
  else
    fma_rate_kernel<float><<<blocks, 256, 0, st>>>((float *)out, iters, 0.999f, 0.001f);
  return cudaGetLastError();
}

cudaError_t
selftest_bounded_wait(unsigned long long limit_ns, unsigned long long * out, cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(unsigned long long), st);
  if (e != cudaSuccess)
    return e;
  bounded_wait_kernel<<<1, 128, 0, st>>>(limit_ns, out);
  return cudaGetLastError();
}

bool
hydro3d_tensor_map(int prec, const void * U, const KParams & P, CUtensorMap * out)
{
  // cuTensorMapEncodeTiled through the runtime's driver entry point (no
  // link-time dependency on the driver library)
  using Encode = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
  static Encode encode = [] {
    void *                          fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return (Encode)fn;
  }();
  const size_t es = prec == 0 ? sizeof(double) : sizeof(float);
  // global strides must be multiples of 16 bytes; the box's x origin
  // (gi0 - 2 = blockIdx.x * TX) is then 16-byte aligned since TX % 4 == 0
  if (!encode || P.ksize < 2 || ((size_t)P.isize * es) % 16 != 0 || (H3_TX % 4) != 0 ||
      (reinterpret_cast<uintptr_t>(U) % 16) != 0)
    return false;
  const cuuint64_t dims[4] = { (cuuint64_t)P.isize, (cuuint64_t)P.jsize, (cuuint64_t)P.ksize, 5 };
  const cuuint64_t strides[3] = { (cuuint64_t)P.isize * es, (cuuint64_t)P.plane * es, (cuuint64_t)P.vstride * es };
  const cuuint32_t box[4] = { H3_TX + 4, H3_TY + 4, 1, 5 };
  const cuuint32_t estr[4] = { 1, 1, 1, 1 };
  return encode(out, prec == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                const_cast<void *>(U), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

namespace
{
template <class S>
__global__ void
totals_kernel(const S * __restrict__ U, KParams P, double * acc)
{
  // FP64 mass and total energy over the interior; max |div B| for MHD
  double m = 0.0, e = 0.0, db = 0.0;
  for_interior_rows(P, [&](int i, int j, int k) {
    const long long off = (long long)k * P.plane + (long long)j * P.isize + i;
    m += (double)U[off];
    e += (double)U[P.vstride + off];
  });
  for (int o = 16; o > 0; o >>= 1)
  {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  if ((threadIdx.x & 31) == 0)
  {
    atomicAdd(acc + 0, m);
    atomicAdd(acc + 1, e);
  }
  (void)db;
}
} // namespace

cudaError_t
fill_ghosts(int prec, void * U, const KParams & P, int nbvar, cudaStream_t st)
{
  const long long n = P.vstride;
  const int       blocks = (int)((n + 255) / 256 < 8192 ? (n + 255) / 256 : 8192);
  if (prec == 0)
    fill_ghosts_kernel<double><<<blocks, 256, 0, st>>>((double *)U, P, nbvar, 0);
  else if (!P.mhd)
    fill_ghosts_kernel<float><<<blocks, 256, 0, st>>>((float *)U, P, nbvar, 0);
  else
  {
    // mixed MHD: 5 FP32 hydro planes followed by 3 FP64 face-field planes
    fill_ghosts_kernel<float><<<blocks, 256, 0, st>>>((float *)U, P, 5, 0);
    fill_ghosts_kernel<double><<<blocks, 256, 0, st>>>(mixed_bfield(U, P), P, 3, 5);
  }
  return cudaGetLastError();
}

namespace
{
// offset in the device state of element e of a host array (layout 0: LayoutLeft
// [var][k][j][i], 1: LayoutRight [i][j][k][var]); v receives the variable
__device__ __forceinline__ long long
host_elem_cell(long long e, int layout, const KParams & P, int nbvar, int & v)
{
  if (layout == 0)
  {
    v = (int)(e / P.vstride);
    return e - (long long)v * P.vstride;
  }
  v = (int)(e % nbvar);
  long long c = e / nbvar;
  const int k = (int)(c % P.ksize);
  c /= P.ksize;
  const int j = (int)(c % P.jsize);
  const int i = (int)(c / P.jsize);
  return (long long)k * P.plane + (long long)j * P.isize + i;
}

template <bool TO_STATE>
__global__ void
convert_stage_kernel(int prec, int layout, double * __restrict__ stage, void * __restrict__ U, KParams P, int nbvar,
                     long long first, long long count)
{
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < count;
       t += (long long)gridDim.x * blockDim.x)
  {
    int             v;
    const long long cell = host_elem_cell(first + t, layout, P, nbvar, v);
    if (prec == 0 || (P.mhd && v >= 5))
    {
      // FP64 state, or a face-field plane of the mixed MHD state
      double * D = prec == 0 ? (double *)U + (long long)v * P.vstride + cell
                             : mixed_bfield(U, P) + (long long)(v - 5) * P.vstride + cell;
      if (TO_STATE)
        *D = stage[t];
      else
        stage[t] = *D;
    }
    else
    {
      float * F = (float *)U + (long long)v * P.vstride + cell;
      if (TO_STATE)
        *F = __double2float_rn(stage[t]);
      else
        stage[t] = (double)*F;
    }
  }
}
} // namespace

cudaError_t
convert_stage(bool to_state, int prec, int layout, double * stage, void * U, const KParams & P, int nbvar,
              long long first, long long count, cudaStream_t st)
{
  const long long want = (count + 255) / 256;
  const int       blocks = (int)(want < 152 * 16 ? want : 152 * 16);
  if (blocks <= 0)
    return cudaSuccess;
  if (to_state)
    convert_stage_kernel<true><<<blocks, 256, 0, st>>>(prec, layout, stage, U, P, nbvar, first, count);
  else
    convert_stage_kernel<false><<<blocks, 256, 0, st>>>(prec, layout, stage, U, P, nbvar, first, count);
  return cudaGetLastError();
}

cudaError_t
ensemble_totals(int prec, const EnsInstance * insts, int n, const int * stepc, double * out,
                cudaStream_t st)
{
  cudaError_t e = cudaMemsetAsync(out, 0, 2 * sizeof(double) * n, st);
  if (e != cudaSuccess)
    return e;
  dim3 grid(16, n);
  if (prec == 0)
    ensemble_totals_kernel<double><<<grid, 256, 0, st>>>(insts, stepc, out);
  else
    ensemble_totals_kernel<float><<<grid, 256, 0, st>>>(insts, stepc, out);
  return cudaGetLastError();
}

cudaError_t
totals(int prec, const void * U, const KParams & P, int nbvar, double * out3, cudaStream_t st)
{
  (void)nbvar;
  cudaError_t e = cudaMemsetAsync(out3, 0, 3 * sizeof(double), st);
  if (e != cudaSuccess)
    return e;
  const int blocks = row_blocks(P);
  if (prec == 0)
    totals_kernel<double><<<blocks, 256, 0, st>>>((const double *)U, P, out3);
  else
    totals_kernel<float><<<blocks, 256, 0, st>>>((const float *)U, P, out3);
  e = cudaGetLastError();
  if (e != cudaSuccess || !P.mhd)
    return e;
  return mhd_divb_max(prec, U, P, out3 + 2, st);
}
#endif

} // namespace EK_NS
