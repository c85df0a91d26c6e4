// Host-callable launchers of the device kernels.  ek_kernels.cu is compiled
// twice: namespace ek_exact (FP64 only, no FMA contraction: bitwise parity
// with the reference's FP64 build) and ek_fast (FMA contraction; FP64 and the
// mixed FP32 form).
#pragma once

#include <cuda_runtime.h>

#include "ek_common.cuh"

#define EK_DECLARE_LAUNCHERS(NS)                                                                    \
  namespace NS                                                                                      \
  {                                                                                                 \
  using ekc::KParams;                                                                               \
  using ekc::DevClock;                                                                              \
  /* prec: 0 FP64, 1 mixed.  Uin/Uout device state arrays. */                                      \
  /* tmap: tensor map of Uin for the 3D kernel's staged planes, or null */                        \
  cudaError_t hydro_step(int dim, int prec, const void * Uin, void * Uout, const KParams & P,        \
                         DevClock * clk, int step, const CUtensorMap * tmap, cudaStream_t st);      \
  /* fin: also compute the step constants of step fin_step from key (the last block) */           \
  cudaError_t hydro_dt(int dim, int prec, const void * U, const KParams & P,                       \
                       unsigned long long * key, DevClock * fin, int fin_step, cudaStream_t st);    \
  cudaError_t mhd_dt(int prec, const void * U, const KParams & P, unsigned long long * key,         \
                     cudaStream_t st);                                                              \
  /* one MHD step = phase 0 (CFL), 1 (trace), 2 (fluxes, emfs, update; cfl_next: and the     */ \
  /* CFL of the updated state, the next step's dt, so its phase 0 is not needed), 3 (the      */ \
  /* repair pass of the mixed HLLD form, which then must follow phase 2) */                      \
  cudaError_t mhd_step(int prec, int phase, const void * Uin, void * Uout, void * work,             \
                       const KParams & P, DevClock * clk, int step, bool cfl_next, cudaStream_t st); \
  size_t      mhd_work_bytes(int prec, const KParams & P);                                          \
  /* one MHD 2D step = phase 0 (CFL), 1 (fused trace, fluxes, emf, update), 2 (the repair   */ \
  /* pass of the mixed HLLD form, which then must follow phase 1) */                               \
  cudaError_t mhd2d_step(int prec, int phase, const void * Uin, void * Uout, void * work,           \
                         const KParams & P, DevClock * clk, int step, cudaStream_t st);             \
  size_t      mhd2d_work_bytes(int prec, const KParams & P);                                        \
  cudaError_t mhd2d_dt(int prec, const void * U, const KParams & P, unsigned long long * key,       \
                       cudaStream_t st);                                                            \
  /* one step of every instance of a 2D hydro ensemble (persistent kernel) */                       \
  /* scal: per-instance step scalars (n entries of 64 bytes), written by the step */                \
  cudaError_t ensemble2d_step(int prec, const ekc::EnsInstance * insts, int n, const ekc::EnsTile * tiles, \
                              int ntiles, int * stepc, void * scal, int grid, cudaStream_t st);     \
  int         ensemble2d_grid(int prec);                                                            \
  }

EK_DECLARE_LAUNCHERS(ek_exact)
EK_DECLARE_LAUNCHERS(ek_fast)

namespace ek_fast
{
using ekc::KParams;
// precision-independent helpers (only built once)
cudaError_t fill_ghosts(int prec, void * U, const KParams & P, int nbvar, cudaStream_t st);
cudaError_t totals(int prec, const void * U, const KParams & P, int nbvar, double * out3,
                   cudaStream_t st);
cudaError_t ensemble_totals(int prec, const ekc::EnsInstance * insts, int n, const int * stepc,
                            double * out, cudaStream_t st);
// Host FP64 arrays <-> device state.  Elements [first, first + count) of a
// host array in the caller's layout (0 LayoutLeft, 1 LayoutRight; nbvar
// variables) sit in the device staging buffer stage; to_state: convert them
// into the state U (precision prec), else fill stage from U.
cudaError_t convert_stage(bool to_state, int prec, int layout, double * stage, void * U, const KParams & P,
                          int nbvar, long long first, long long count, cudaStream_t st);
// The bounded mbarrier wait on a barrier nothing completes (one block):
// out[0] = number of threads whose wait expired, out[1] = longest wait in ns.
cudaError_t selftest_bounded_wait(unsigned long long limit_ns, unsigned long long * out, cudaStream_t st);
// FMA chains for the CUDA-core FLOP rate: blocks x 256 threads x 8 chains x 16 x iters FMAs
cudaError_t fma_rate(int prec, int blocks, int iters, void * out, cudaStream_t st);
// Tensor map of a 3D hydro state U (box = the 3D kernel's tile plus halo, all
// five variables); false when the layout does not allow tensor copies.
bool hydro3d_tensor_map(int prec, const void * U, const KParams & P, CUtensorMap * out);
} // namespace ek_fast
