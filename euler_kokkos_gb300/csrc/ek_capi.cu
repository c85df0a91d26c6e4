// C ABI implementation: solver handle, device buffers, step sequencing.
//
// Host-side equivalent of SolverBase + SolverHydroMuscl/SolverMHDMuscl
// (SolverBase.cpp:124-195, SolverHydroMuscl.h:164-307, 635-700,
// SolverMHDMuscl.h:384-397, 741-801) with the kernels of ek_kernels.cu.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/ek_gb300.h"
#include "ek_internal.h"
#include "ek_launch.h"

namespace ek_internal
{
static thread_local std::string g_last_error;

ek_status
fail(ek_status s, const std::string & msg)
{
  g_last_error = msg;
  return s;
}
} // namespace ek_internal

// planes per CTA column of the 3D kernels when the parameters leave it at 0
#ifndef EK_KCHUNK_DEFAULT
#define EK_KCHUNK_DEFAULT 32
#endif

using ek_internal::fail;
using KParams = ekc::KParams;
using DevClock = ekc::DevClock;

struct ek_solver
{
  ek_params     p;
  KParams       kp;
  int           prec;
  bool          exact;
  void *        U[2] = { nullptr, nullptr }; // ping-pong device states
  size_t        state_bytes = 0;
  void *        work = nullptr; // MHD intermediates (if any)
  size_t        work_bytes = 0;
  DevClock *    clk = nullptr;  // device
  double *      dtlog = nullptr;
  int           dtcap = 0;
  double *      scratch3 = nullptr; // device totals
  void *        gfield = nullptr;   // static gravity field (state precision), if set
  // tensor maps of U[0] / U[1] for the 3D hydro kernel's staged planes
  alignas(64) CUtensorMap tmap[2];
  bool          has_tmap = false;
  cudaStream_t  stream = nullptr;
  int           device = 0;
  // host mirror of SolverBase state
  double        t = 0.0, dt = 0.0;
  int           iteration = 0;
  bool          has_state = false;
  long long     launches = 0;
  double *      stage = nullptr; // device staging of host FP64 arrays (set/get state)
  long long     stage_elems = 0;
  // kernel timing (ek_solver_set_profiling)
  bool                     profiling = false;
  std::vector<cudaEvent_t> ev_pool;            // recycled events
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev_pending;
  double                   kernel_ms[4] = { 0, 0, 0, 0 };
  long long                kernel_n[4] = { 0, 0, 0, 0 };
  bool                     owns = true; // false: a view into an ensemble's buffers
  // 3D MHD: the step whose CFL the last update kernel computed (-1: none)
  int                      cfl_step = -1;
};

// The mixed MHD form with the HLLD solver: each step ends with the repair pass
// (the tiles whose FP32 star states were ill-conditioned, recomputed with
// those faces in FP64); its tile list heads the work buffer.
static bool
has_repair(const ek_solver * s)
{
  return s->p.mhd && s->prec != 0 && s->kp.riemann == 4;
}

static cudaEvent_t
take_event(ek_solver * s)
{
  if (!s->ev_pool.empty())
  {
    cudaEvent_t e = s->ev_pool.back();
    s->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// fold the finished event pairs into the per-kernel totals
static void
drain_events(ek_solver * s)
{
  for (auto & pe : s->ev_pending)
  {
    float ms = 0.f;
    if (cudaEventSynchronize(pe.second.second) == cudaSuccess &&
        cudaEventElapsedTime(&ms, pe.second.first, pe.second.second) == cudaSuccess)
    {
      s->kernel_ms[pe.first] += ms;
      s->kernel_n[pe.first] += 1;
    }
    s->ev_pool.push_back(pe.second.first);
    s->ev_pool.push_back(pe.second.second);
  }
  s->ev_pending.clear();
}

static ek_status
cuda_fail(cudaError_t e, const char * what)
{
  return fail(e == cudaErrorMemoryAllocation ? EK_ERR_NO_MEMORY : EK_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}
#define EK_CUDA(call, what)                                                                         \
  do                                                                                                \
  {                                                                                                 \
    cudaError_t e__ = (call);                                                                       \
    if (e__ != cudaSuccess)                                                                         \
      return cuda_fail(e__, what);                                                                  \
  } while (0)

extern "C" int
ek_abi_version(void)
{
  return EK_ABI_VERSION;
}

extern "C" const char *
ek_status_string(ek_status s)
{
  switch (s)
  {
    case EK_OK: return "ok";
    case EK_ERR_INVALID: return "invalid argument";
    case EK_ERR_UNSUPPORTED: return "unsupported configuration";
    case EK_ERR_CUDA: return "CUDA error";
    case EK_ERR_NO_MEMORY: return "out of memory";
    case EK_ERR_NONFINITE: return "non-finite time step";
    case EK_ERR_PARSE: return "ini parse error";
    case EK_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

extern "C" const char *
ek_last_error(void)
{
  return ek_internal::g_last_error.c_str();
}

namespace ek_internal
{
ek_status
validate(const ek_params & p)
{
  if (p.dim != 2 && p.dim != 3)
    return fail(EK_ERR_INVALID, "dim must be 2 or 3");
  if (p.nx < 1 || p.ny < 1 || (p.dim == 3 && p.nz < 1))
    return fail(EK_ERR_INVALID, "grid sizes must be positive");
  const int gw = p.mhd ? 3 : 2;
  if (p.ghost_width != gw || p.nbvar != (p.mhd ? 8 : (p.dim == 2 ? 4 : 5)))
    return fail(EK_ERR_INVALID, "ghost_width/nbvar inconsistent with the solver kind");
  if (p.isize != p.nx + 2 * gw || p.jsize != p.ny + 2 * gw || (p.dim == 3 && p.ksize != p.nz + 2 * gw))
    return fail(EK_ERR_INVALID, "isize/jsize/ksize inconsistent with nx/ny/nz");
  if (p.nx < gw || p.ny < gw || (p.dim == 3 && p.nz < gw))
    return fail(EK_ERR_INVALID, "each dimension needs at least ghost_width interior cells");
  for (int f = 0; f < 2 * p.dim; ++f)
    if (p.bc[f] < 1 || p.bc[f] > 3)
      return fail(EK_ERR_INVALID, "boundary types must be 1 (reflect), 2 (outflow) or 3 (periodic)");
  // riemann_hydro / riemann_mhd dispatch (RiemannSolvers.h:573-640,
  // RiemannSolvers_MHD.h:368-389): for other values the reference leaves the
  // flux unset, so they are refused here
  if (!p.mhd && (p.riemann < 0 || p.riemann > 3))
    return fail(EK_ERR_UNSUPPORTED, "hydro: riemann must be approx, llf, hll or hllc");
  if (!p.mhd && p.dim == 3 && p.riemann == 2)
    return fail(EK_ERR_UNSUPPORTED, "Hydro_Muscl_3D: the reference's 3D solver dispatch has no hll branch");
  if (p.mhd && p.riemann != 1 && p.riemann != 2 && p.riemann != 4)
    return fail(EK_ERR_UNSUPPORTED, "MHD: riemann must be llf, hll or hlld");
  // slope_unsplit_hydro_{2d,3d} (HydroBaseFunctor2D.h:488-516,
  // HydroBaseFunctor3D.h:498-576) zero the slopes for slope_type 0 and limit
  // them for 1 and 2; the MHD slope routines (MHDBaseFunctor3D.h:379,
  // MHDBaseFunctor2D.h:369-420) only handle 1 and 2.  For other values the
  // reference leaves the slopes unwritten, so they are refused here.
  if (p.slope_type != 1.0 && p.slope_type != 2.0 && (p.mhd || p.slope_type != 0.0))
    return fail(EK_ERR_UNSUPPORTED, p.mhd ? "MHD: slope_type must be 1 (minmod) or 2 (MC)"
                                          : "hydro: slope_type must be 0 (first order), 1 (minmod) or 2 (MC)");
  // implementationVersion (SolverHydroMuscl.cpp:234-293, SolverMHDMuscl.cpp:397-445,
  // 490-560): hydro 1 is version 0's arithmetic split into more kernels (the
  // same bits); hydro 2 adds the face fluxes to the cells with atomics
  // (version 0's results up to the summation order).  Both run the fused
  // version-0 step.  The MHD versions 1 and 2 compute other numbers.
  if (p.implementation_version < 0 || p.implementation_version > 2)
    return fail(EK_ERR_INVALID, "implementationVersion must be 0, 1 or 2");
  if (p.mhd && p.implementation_version != 0)
    return fail(EK_ERR_UNSUPPORTED, "MHD: implementationVersion 1 and 2 compute another scheme; use 0");
  if (p.cIso > 0 || p.Omega0 > 0)
    return fail(EK_ERR_UNSUPPORTED, "isothermal and shearing-box terms are not implemented");
  if (p.exact_fp && p.precision != EK_PREC_FP64)
    return fail(EK_ERR_INVALID, "exact_fp requires precision fp64");
  if (p.precision != EK_PREC_FP64 && p.precision != EK_PREC_MIXED)
    return fail(EK_ERR_INVALID, "precision must be EK_PREC_FP64 or EK_PREC_MIXED");
  return EK_OK;
}

ekc::KParams
make_kparams(const ek_params & p)
{
  ekc::KParams k;
  std::memset(&k, 0, sizeof k);
  const int gw = p.mhd ? 3 : 2;
  k.nx = p.nx;
  k.ny = p.ny;
  k.nz = p.dim == 3 ? p.nz : 1;
  k.gw = gw;
  k.isize = p.isize;
  k.jsize = p.jsize;
  k.ksize = p.dim == 3 ? p.ksize : 1;
  k.mhd = p.mhd;
  k.plane = (long long)k.isize * k.jsize;
  k.vstride = k.plane * k.ksize;
  for (int f = 0; f < 6; ++f)
    k.bc[f] = p.bc[f];
  k.dx = p.dx;
  k.dy = p.dy;
  k.dz = p.dz;
  k.gamma0 = p.gamma0;
  k.smallr = p.smallr;
  k.smallc = p.smallc;
  k.smallp = p.smallp;
  k.slope_type = p.slope_type;
  k.cfl = p.cfl;
  k.tEnd = p.tEnd;
  k.cIso = p.cIso;
  k.riemann = p.riemann;
  k.kchunk = p.kchunk > 0 ? p.kchunk : (k.nz <= EK_KCHUNK_DEFAULT ? k.nz : EK_KCHUNK_DEFAULT);
  k.gamma0f = (float)p.gamma0;
  k.smallrf = (float)p.smallr;
  k.smallcf = (float)p.smallc;
  k.smallpf = (float)p.smallp;
  k.slopef = (float)p.slope_type;
  k.idx = (float)(1.0 / p.dx);
  k.idy = (float)(1.0 / p.dy);
  k.idz = (float)(1.0 / (p.dim == 3 ? p.dz : 1.0));
  k.idxd = 1.0 / p.dx;
  k.idyd = 1.0 / p.dy;
  k.idzd = 1.0 / (p.dim == 3 ? p.dz : 1.0);
  k.mhd_stage = p.mhd_stage;
  k.gamma6 = p.gamma6;
  k.smallpp = p.smallpp;
  k.gamma6f = (float)p.gamma6;
  k.smallppf = (float)p.smallpp;
  // static gravity: hydro only (SolverMHDMuscl has no gravity terms)
  k.grav = (!p.mhd && p.gravity_enabled) ? 1 : 0;
  k.grav_hancock = k.grav && p.gravity_hancock ? 1 : 0;
  for (int e = 0; e < 3; ++e)
  {
    k.g[e] = (e < p.dim) ? p.gravity[e] : 0.0;
    k.gf[e] = (float)k.g[e];
  }
  // ComputeDtGravityFunctor: dx = fmin(dx, dy) [, fmin(dx, dz)]
  k.dxmin = std::fmin(p.dx, p.dy);
  if (p.dim == 3)
    k.dxmin = std::fmin(k.dxmin, p.dz);
  k.cfl_dxmin = p.cfl * k.dxmin;
  k.cfl_dxminf = (float)k.cfl_dxmin;
  k.idxminf = (float)(1.0 / k.dxmin);
  k.gfield = nullptr;
  return k;
}

size_t
state_bytes(const ek_params & p, const ekc::KParams & kp)
{
  if (p.precision == EK_PREC_FP64)
    return sizeof(double) * (size_t)kp.vstride * p.nbvar;
  if (!p.mhd)
    return sizeof(float) * (size_t)kp.vstride * p.nbvar;
  return ekc::mixed_bfield_offset(kp.vstride) + sizeof(double) * 3 * (size_t)kp.vstride;
}
} // namespace ek_internal

extern "C" ek_status
ek_solver_create(const ek_params * params, ek_solver ** out)
{
  if (!params || !out)
    return fail(EK_ERR_INVALID, "ek_solver_create: null argument");
  *out = nullptr;
  const ek_params & p = *params;
  {
    ek_status v = ek_internal::validate(p);
    if (v != EK_OK)
      return v;
  }

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(EK_ERR_NO_DEVICE, "no CUDA device available");

  ek_solver * s = new ek_solver();
  s->p = p;
  s->prec = p.precision;
  s->exact = p.exact_fp != 0;
  cudaGetDevice(&s->device);
  s->kp = ek_internal::make_kparams(p);
  const KParams & k = s->kp;
  s->state_bytes = ek_internal::state_bytes(p, k);
  cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaMalloc(&s->U[0], s->state_bytes);
  if (e == cudaSuccess)
    e = cudaMalloc(&s->U[1], s->state_bytes);
  if (e == cudaSuccess)
    e = cudaMalloc((void **)&s->clk, sizeof(DevClock));
  s->dtcap = p.nStepmax > 0 ? (p.nStepmax < (1 << 22) ? p.nStepmax + 1 : (1 << 22)) : 1;
  if (e == cudaSuccess)
    e = cudaMalloc((void **)&s->dtlog, sizeof(double) * s->dtcap);
  if (e == cudaSuccess)
    e = cudaMalloc((void **)&s->scratch3, 3 * sizeof(double));
  if (e == cudaSuccess && p.mhd)
  {
    if (p.dim == 3)
      s->work_bytes = s->exact ? ek_exact::mhd_work_bytes(s->prec, k) : ek_fast::mhd_work_bytes(s->prec, k);
    else
      s->work_bytes = s->exact ? ek_exact::mhd2d_work_bytes(s->prec, k) : ek_fast::mhd2d_work_bytes(s->prec, k);
    if (s->work_bytes)
      e = cudaMalloc(&s->work, s->work_bytes);
  }
  // on the solver's stream: a legacy-stream memset is not ordered before the
  // uploads of the (non-blocking) solver stream
  if (e == cudaSuccess)
    e = cudaMemsetAsync(s->U[0], 0, s->state_bytes, s->stream);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(s->U[1], 0, s->state_bytes, s->stream);
  if (e == cudaSuccess && !p.mhd && p.dim == 3 && !p.no_tma)
    s->has_tmap = ek_fast::hydro3d_tensor_map(s->prec, s->U[0], k, &s->tmap[0]) &&
                  ek_fast::hydro3d_tensor_map(s->prec, s->U[1], k, &s->tmap[1]);
  if (e != cudaSuccess)
  {
    ek_status st = cuda_fail(e, "ek_solver_create");
    ek_solver_destroy(s);
    return st;
  }
  *out = s;
  return EK_OK;
}

extern "C" ek_status
ek_solver_destroy(ek_solver * s)
{
  if (!s)
    return EK_OK;
  if (!s->owns)
  {
    drain_events(s);
    cudaFree(s->stage);
    delete s;
    return EK_OK;
  }
  if (s->stream)
    cudaStreamSynchronize(s->stream);
  cudaFree(s->U[0]);
  cudaFree(s->U[1]);
  cudaFree(s->work);
  cudaFree(s->clk);
  cudaFree(s->dtlog);
  cudaFree(s->scratch3);
  cudaFree(s->gfield);
  cudaFree(s->stage);
  drain_events(s);
  for (auto e : s->ev_pool)
    cudaEventDestroy(e);
  if (s->stream)
    cudaStreamDestroy(s->stream);
  delete s;
  return EK_OK;
}

// Host FP64 arrays (either layout) <-> device state.  The FP64 LayoutLeft
// state is copied as is; every other combination goes through a bounded
// device staging buffer: one cudaMemcpyAsync per chunk of the host array and
// a kernel that converts (FP32 state) and/or transposes (LayoutRight) it on
// the device, so the host does no per-element work.
static const long long kStageElems = 1LL << 25; // 32 Mi doubles (256 MB)

static ek_status
ensure_stage(ek_solver * s, long long total)
{
  const long long want = total < kStageElems ? total : kStageElems;
  if (s->stage_elems >= want)
    return EK_OK;
  cudaFree(s->stage);
  s->stage = nullptr;
  s->stage_elems = 0;
  EK_CUDA(cudaMalloc((void **)&s->stage, sizeof(double) * (size_t)want), "staging buffer");
  s->stage_elems = want;
  return EK_OK;
}

// views into an ensemble keep no staging buffer between calls
static void
release_stage(ek_solver * s)
{
  if (s->owns)
    return;
  cudaFree(s->stage);
  s->stage = nullptr;
  s->stage_elems = 0;
}

static ek_status
host_to_state(ek_solver * s, const double * U, int layout, void * dev)
{
  const long long total = s->kp.vstride * s->p.nbvar;
  if (s->prec == EK_PREC_FP64 && layout == EK_LAYOUT_LEFT)
  {
    EK_CUDA(cudaMemcpyAsync(dev, U, sizeof(double) * (size_t)total, cudaMemcpyHostToDevice, s->stream), "upload");
    EK_CUDA(cudaStreamSynchronize(s->stream), "upload");
    return EK_OK;
  }
  ek_status st = ensure_stage(s, total);
  if (st != EK_OK)
    return st;
  for (long long first = 0; first < total; first += s->stage_elems)
  {
    const long long cnt = total - first < s->stage_elems ? total - first : s->stage_elems;
    EK_CUDA(cudaMemcpyAsync(s->stage, U + first, sizeof(double) * (size_t)cnt, cudaMemcpyHostToDevice, s->stream),
            "upload");
    EK_CUDA(ek_fast::convert_stage(true, s->prec, layout, s->stage, dev, s->kp, s->p.nbvar, first, cnt, s->stream),
            "upload");
    s->launches += 1;
  }
  EK_CUDA(cudaStreamSynchronize(s->stream), "upload");
  release_stage(s);
  return EK_OK;
}

static ek_status
state_to_host(ek_solver * s, const void * dev, double * U, int layout)
{
  const long long total = s->kp.vstride * s->p.nbvar;
  if (s->prec == EK_PREC_FP64 && layout == EK_LAYOUT_LEFT)
  {
    EK_CUDA(cudaMemcpyAsync(U, dev, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost, s->stream), "download");
    EK_CUDA(cudaStreamSynchronize(s->stream), "download");
    return EK_OK;
  }
  ek_status st = ensure_stage(s, total);
  if (st != EK_OK)
    return st;
  for (long long first = 0; first < total; first += s->stage_elems)
  {
    const long long cnt = total - first < s->stage_elems ? total - first : s->stage_elems;
    EK_CUDA(ek_fast::convert_stage(false, s->prec, layout, s->stage, const_cast<void *>(dev), s->kp, s->p.nbvar,
                                   first, cnt, s->stream),
            "download");
    s->launches += 1;
    EK_CUDA(cudaMemcpyAsync(U + first, s->stage, sizeof(double) * (size_t)cnt, cudaMemcpyDeviceToHost, s->stream),
            "download");
  }
  EK_CUDA(cudaStreamSynchronize(s->stream), "download");
  release_stage(s);
  return EK_OK;
}

// fin_step >= 0 (hydro): key is the clock's slot of that step; its step
// constants are computed too
static ek_status
launch_dt(ek_solver * s, const void * U, unsigned long long * key, int fin_step = -1)
{
  cudaError_t e;
  if (s->p.mhd && s->p.dim == 2)
    e = s->exact ? ek_exact::mhd2d_dt(s->prec, U, s->kp, key, s->stream)
                 : ek_fast::mhd2d_dt(s->prec, U, s->kp, key, s->stream);
  else if (s->p.mhd)
    e = s->exact ? ek_exact::mhd_dt(s->prec, U, s->kp, key, s->stream)
                 : ek_fast::mhd_dt(s->prec, U, s->kp, key, s->stream);
  else
  {
    DevClock * fin = fin_step >= 0 ? s->clk : nullptr;
    e = s->exact ? ek_exact::hydro_dt(s->p.dim, s->prec, U, s->kp, key, fin, fin_step, s->stream)
                 : ek_fast::hydro_dt(s->p.dim, s->prec, U, s->kp, key, fin, fin_step, s->stream);
  }
  if (e == cudaErrorNotSupported)
    return fail(EK_ERR_UNSUPPORTED, "kernel not available for this configuration");
  EK_CUDA(e, "dt kernel");
  s->launches += 1;
  return EK_OK;
}

// reset the device clock with t0 and the CFL reduction of the state
static ek_status
reset_clock(ek_solver * s, double t0)
{
  DevClock h;
  std::memset(&h, 0, sizeof h);
  for (int i = 0; i < 3; ++i)
  {
    h.key[i] = EK_KEY_LOWEST;
    h.t[i] = 0.0;
    h.sid[i] = -1;
    h.sc[i].step = -1;
    h.fin[i] = 0;
  }
  h.sid[0] = 0;
  h.t[0] = t0;
  h.iteration = 0;
  h.error = 0;
  h.dtlog = s->dtlog;
  h.dtcap = s->dtcap;
  s->cfl_step = -1;
  EK_CUDA(cudaMemcpyAsync(s->clk, &h, sizeof h, cudaMemcpyHostToDevice, s->stream), "clock reset");
  // an empty repair list and its tile counter
  if (has_repair(s))
    EK_CUDA(cudaMemsetAsync(s->work, 0, 4 * sizeof(int), s->stream), "clock reset");
  // hydro: slot 0 holds the CFL of the initial state (the constructor's
  // compute_dt()); MHD recomputes dt inside every step
  if (!s->p.mhd)
    return launch_dt(s, s->U[0], &s->clk->key[0], 0);
  return EK_OK;
}

static ek_status
read_clock(ek_solver * s, DevClock * h)
{
  EK_CUDA(cudaMemcpyAsync(h, s->clk, sizeof *h, cudaMemcpyDeviceToHost, s->stream), "clock read");
  EK_CUDA(cudaStreamSynchronize(s->stream), "clock read");
  return EK_OK;
}

static double
clock_dt(const ek_solver * s, const DevClock & h, int step)
{
  const double invDt = ekc::dkey_inv(h.key[step % 3]);
  double       d = s->p.cfl / invDt;
  const double tt = h.t[step % 3];
  if (tt + d > s->p.tEnd)
    d = s->p.tEnd - tt;
  return d;
}

static ek_status set_state_at(ek_solver * s, const double * U, int layout, double t0);

extern "C" ek_status
ek_solver_set_state(ek_solver * s, const double * U, int layout)
{
  if (!s || !U || (layout != EK_LAYOUT_LEFT && layout != EK_LAYOUT_RIGHT))
    return fail(EK_ERR_INVALID, "ek_solver_set_state: bad argument");
  return set_state_at(s, U, layout, s->p.tCurrent);
}

// the state injection of the constructor tail, starting at time t0 and
// iteration 0 (a restarted run also starts at iteration 0, SolverHydroMuscl.h:512-580)
static ek_status
set_state_at(ek_solver * s, const double * U, int layout, double t0)
{
  EK_CUDA(cudaSetDevice(s->device), "cudaSetDevice");
  ek_status st = host_to_state(s, U, layout, s->U[0]);
  if (st != EK_OK)
    return st;
  // U2 = U (deep_copy), ghosts of both follow the boundary conditions
  ek_status st2 = EK_OK;
  EK_CUDA(ek_fast::fill_ghosts(s->prec, s->U[0], s->kp, s->p.mhd ? 8 : s->p.nbvar, s->stream), "ghosts");
  EK_CUDA(cudaMemcpyAsync(s->U[1], s->U[0], s->state_bytes, cudaMemcpyDeviceToDevice, s->stream), "copy");
  s->launches += 1;
  s->t = t0;
  s->iteration = 0;
  st2 = reset_clock(s, s->t);
  if (st2 != EK_OK)
    return st2;
  s->has_state = true;
  // m_dt after the constructor
  double dt = 0.0;
  return ek_solver_compute_dt(s, &dt);
}

extern "C" ek_status
ek_selftest_bounded_wait(int limit_us, int * expired, double * elapsed_us)
{
  if (limit_us < 1 || limit_us > 1000000 || !expired || !elapsed_us)
    return fail(EK_ERR_INVALID, "ek_selftest_bounded_wait: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(EK_ERR_NO_DEVICE, "no CUDA device available");
  unsigned long long * d = nullptr;
  unsigned long long   h[2] = { 0, 0 };
  EK_CUDA(cudaMalloc((void **)&d, sizeof h), "selftest");
  cudaError_t e = ek_fast::selftest_bounded_wait((unsigned long long)limit_us * 1000ull, d, 0);
  if (e == cudaSuccess)
    e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  EK_CUDA(e, "selftest");
  *expired = h[0] == 128 ? 1 : 0;
  *elapsed_us = (double)h[1] / 1000.0;
  return EK_OK;
}

extern "C" ek_status
ek_measure_fma_rate(int precision, double * tflops)
{
  if (!tflops)
    return fail(EK_ERR_INVALID, "ek_measure_fma_rate: bad argument");
  int ndev = 0, dev = 0, sms = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(EK_ERR_NO_DEVICE, "no CUDA device available");
  EK_CUDA(cudaGetDevice(&dev), "fma rate");
  EK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "fma rate");
  const bool   f64 = precision == EK_PREC_FP64;
  const int    blocks = sms * 8;           // 8 resident 256-thread CTAs per SM
  const int    iters = f64 ? 200 : 4000;   // a few milliseconds at GB300's rates
  const size_t bytes = (size_t)blocks * 256 * (f64 ? sizeof(double) : sizeof(float));
  void *       out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t  e0 = nullptr, e1 = nullptr;
  cudaError_t  e = cudaMalloc(&out, bytes);
  if (e == cudaSuccess)
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess)
    e = cudaEventCreate(&e0);
  if (e == cudaSuccess)
    e = cudaEventCreate(&e1);
  if (e == cudaSuccess)
    e = ek_fast::fma_rate(f64 ? 0 : 1, blocks, 10, out, st); // warm-up
  double best = 0.0;
  for (int r = 0; r < 3 && e == cudaSuccess; ++r)
  {
    e = cudaEventRecord(e0, st);
    if (e == cudaSuccess)
      e = ek_fast::fma_rate(f64 ? 0 : 1, blocks, iters, out, st);
    if (e == cudaSuccess)
      e = cudaEventRecord(e1, st);
    if (e == cudaSuccess)
      e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess)
      e = cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * 8 * 16 * (double)iters * blocks * 256;
    if (e == cudaSuccess && ms > 0.f && flops / (ms * 1e9) > best)
      best = flops / (ms * 1e9);
  }
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  if (st)
    cudaStreamDestroy(st);
  cudaFree(out);
  EK_CUDA(e, "fma rate");
  *tflops = best;
  return EK_OK;
}

extern "C" ek_status
ek_solver_set_gravity_field(ek_solver * s, const double * G, int layout)
{
  if (!s || (layout != EK_LAYOUT_LEFT && layout != EK_LAYOUT_RIGHT))
    return fail(EK_ERR_INVALID, "ek_solver_set_gravity_field: bad argument");
  if (!s->kp.grav)
    return fail(EK_ERR_INVALID, "ek_solver_set_gravity_field: gravity is not enabled (hydro solvers, "
                                "[gravity] enabled)");
  EK_CUDA(cudaSetDevice(s->device), "cudaSetDevice");
  const int       dim = s->p.dim, is = s->kp.isize, js = s->kp.jsize, ks = s->kp.ksize;
  const long long n = s->kp.vstride;
  if (!G)
  {
    // back to the uniform field of the parameters
    EK_CUDA(cudaStreamSynchronize(s->stream), "gravity field");
    cudaFree(s->gfield);
    s->gfield = nullptr;
  }
  else
  {
    // device copy in the state's precision, LayoutLeft, one plane per component
    const size_t es = s->prec == EK_PREC_FP64 ? sizeof(double) : sizeof(float);
    if (!s->gfield)
      EK_CUDA(cudaMalloc(&s->gfield, es * (size_t)n * dim), "gravity field");
    std::vector<double> h((size_t)n * dim);
    if (layout == EK_LAYOUT_LEFT)
      std::memcpy(h.data(), G, sizeof(double) * h.size());
    else
      for (int i = 0; i < is; ++i)
        for (int j = 0; j < js; ++j)
          for (int k = 0; k < ks; ++k)
            for (int c = 0; c < dim; ++c)
              h[(size_t)c * n + ((size_t)k * js + j) * is + i] = G[(((size_t)i * js + j) * ks + k) * dim + c];
    if (s->prec == EK_PREC_FP64)
      EK_CUDA(cudaMemcpyAsync(s->gfield, h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, s->stream),
              "gravity field");
    else
    {
      std::vector<float> f(h.size());
      for (size_t i = 0; i < f.size(); ++i)
        f[i] = (float)h[i];
      EK_CUDA(cudaMemcpyAsync(s->gfield, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice, s->stream),
              "gravity field");
      EK_CUDA(cudaStreamSynchronize(s->stream), "gravity field");
    }
    EK_CUDA(cudaStreamSynchronize(s->stream), "gravity field");
  }
  s->kp.gfield = s->gfield;
  if (!s->has_state)
    return EK_OK;
  // the CFL candidate of the current step, with the new field
  const int          slot = s->iteration % 3;
  unsigned long long low = EK_KEY_LOWEST;
  EK_CUDA(cudaMemcpyAsync(&s->clk->key[slot], &low, sizeof low, cudaMemcpyHostToDevice, s->stream), "gravity dt");
  ek_status st = launch_dt(s, s->U[s->iteration % 2], &s->clk->key[slot], s->iteration);
  if (st != EK_OK)
    return st;
  EK_CUDA(cudaStreamSynchronize(s->stream), "gravity dt");
  return ek_solver_compute_dt(s, nullptr);
}

extern "C" ek_status
ek_solver_compute_dt(ek_solver * s, double * dt)
{
  if (!s || !s->has_state)
    return fail(EK_ERR_INVALID, "ek_solver_compute_dt: no state");
  DevClock h;
  if (s->p.mhd)
  {
    // dt from the primitive variables of the current (boundary-filled) state
    unsigned long long * tmp = reinterpret_cast<unsigned long long *>(s->scratch3);
    unsigned long long   low = EK_KEY_LOWEST, key = 0;
    EK_CUDA(cudaMemcpyAsync(tmp, &low, sizeof low, cudaMemcpyHostToDevice, s->stream), "dt");
    ek_status st = launch_dt(s, s->U[s->iteration % 2], tmp);
    if (st != EK_OK)
      return st;
    EK_CUDA(cudaMemcpyAsync(&key, tmp, sizeof key, cudaMemcpyDeviceToHost, s->stream), "dt");
    EK_CUDA(cudaStreamSynchronize(s->stream), "dt");
    double d = s->p.cfl / ekc::dkey_inv(key);
    if (s->t + d > s->p.tEnd)
      d = s->p.tEnd - s->t;
    s->dt = d;
  }
  else
  {
    ek_status st = read_clock(s, &h);
    if (st != EK_OK)
      return st;
    s->dt = clock_dt(s, h, s->iteration);
  }
  if (dt)
    *dt = s->dt;
  return EK_OK;
}

// one kernel of a step, bracketed by timing events when profiling
static ek_status
launch_one(ek_solver * s, int kernel_id, int phase, int step)
{
  const void * in = s->U[step % 2];
  void *       outp = s->U[(step + 1) % 2];
  cudaEvent_t  e0 = nullptr, e1 = nullptr;
  if (s->profiling)
  {
    e0 = take_event(s);
    e1 = take_event(s);
    cudaEventRecord(e0, s->stream);
  }
  cudaError_t e;
  if (s->p.mhd && s->p.dim == 2)
    e = s->exact ? ek_exact::mhd2d_step(s->prec, phase, in, outp, s->work, s->kp, s->clk, step, s->stream)
                 : ek_fast::mhd2d_step(s->prec, phase, in, outp, s->work, s->kp, s->clk, step, s->stream);
  else if (s->p.mhd)
    e = s->exact ? ek_exact::mhd_step(s->prec, phase, in, outp, s->work, s->kp, s->clk, step, true, s->stream)
                 : ek_fast::mhd_step(s->prec, phase, in, outp, s->work, s->kp, s->clk, step, true, s->stream);
  else
  {
    const CUtensorMap * tm = s->has_tmap ? &s->tmap[step % 2] : nullptr;
    e = s->exact ? ek_exact::hydro_step(s->p.dim, s->prec, in, outp, s->kp, s->clk, step, tm, s->stream)
                 : ek_fast::hydro_step(s->p.dim, s->prec, in, outp, s->kp, s->clk, step, tm, s->stream);
  }
  if (s->profiling)
  {
    cudaEventRecord(e1, s->stream);
    s->ev_pending.push_back({ kernel_id, { e0, e1 } });
  }
  if (e == cudaErrorNotSupported)
    return fail(EK_ERR_UNSUPPORTED, "kernel not available for this configuration");
  EK_CUDA(e, "step kernel");
  s->launches += 1;
  return EK_OK;
}

static ek_status
launch_step(ek_solver * s, int step)
{
  if (!s->p.mhd)
    return launch_one(s, 0, 0, step);
  if (s->p.dim == 2)
  {
    ek_status st = launch_one(s, 2, 0, step); // CFL of the step
    if (st == EK_OK)
      st = launch_one(s, 0, 1, step); // trace, fluxes, emf, update
    if (st == EK_OK && has_repair(s))
      st = launch_one(s, 3, 2, step); // the listed tiles with FP64 star states
    return st;
  }
  // CFL of the step: only when no update kernel computed it (the first step
  // after the state was set)
  ek_status st = EK_OK;
  if (s->cfl_step != step)
    st = launch_one(s, 2, 0, step);
  if (st == EK_OK)
    st = launch_one(s, 1, 1, step); // trace
  if (st == EK_OK)
    st = launch_one(s, 0, 2, step); // fluxes, emfs, update, and the next step's CFL
  if (st == EK_OK && has_repair(s))
    st = launch_one(s, 3, 3, step); // the listed tiles with FP64 star states; completes the CFL
  s->cfl_step = st == EK_OK ? step + 1 : -1;
  return st;
}

static int
host_finished(const ek_solver * s)
{
  return s->t >= (s->p.tEnd - 1e-14) || s->iteration >= s->p.nStepmax;
}

static ek_status
sync_from_clock(ek_solver * s)
{
  DevClock h;
  ek_status st = read_clock(s, &h);
  if (st != EK_OK)
    return st;
  if (h.error & ekc::EK_DEVERR_TMA_TIMEOUT)
    return fail(EK_ERR_CUDA, "a tensor copy of the step kernel did not complete within its 1 s wait limit");
  s->iteration = h.iteration;
  s->t = h.t[h.iteration % 3];
  if (h.iteration > 0)
    s->dt = h.last_dt; // the dt of the last step, in the same read (one host round trip per step)
  if (!(s->dt > 0.0) || !std::isfinite(s->dt))
    return fail(EK_ERR_NONFINITE, "time step is not finite and positive (dt = " + std::to_string(s->dt) + ")");
  return EK_OK;
}

extern "C" ek_status
ek_solver_next_iteration(ek_solver * s)
{
  if (!s || !s->has_state)
    return fail(EK_ERR_INVALID, "ek_solver_next_iteration: no state");
  ek_status st = launch_step(s, s->iteration);
  if (st != EK_OK)
    return st;
  return sync_from_clock(s);
}

extern "C" ek_status
ek_solver_run(ek_solver * s, int nsteps, int * done)
{
  if (!s || !s->has_state || nsteps < 0)
    return fail(EK_ERR_INVALID, "ek_solver_run: bad argument");
  const int start = s->iteration;
  int       issued = 0;
  // steps are launched back to back; the device skips steps once t >= tEnd,
  // so the host checks the clock only between batches
  const int batch = 256;
  while (issued < nsteps && !host_finished(s))
  {
    int n = nsteps - issued;
    n = n < batch ? n : batch;
    n = n < s->p.nStepmax - s->iteration ? n : s->p.nStepmax - s->iteration;
    for (int i = 0; i < n; ++i)
    {
      ek_status st = launch_step(s, s->iteration + i);
      if (st != EK_OK)
        return st;
    }
    issued += n;
    ek_status st = sync_from_clock(s);
    if (st != EK_OK)
      return st;
    if (s->iteration < start + issued)
      break; // tEnd reached on the device
  }
  if (done)
    *done = s->iteration - start;
  return EK_OK;
}

extern "C" ek_status
ek_solver_finished(ek_solver * s, int * finished)
{
  if (!s || !finished)
    return fail(EK_ERR_INVALID, "ek_solver_finished: bad argument");
  *finished = host_finished(s);
  return EK_OK;
}

extern "C" ek_status
ek_solver_time(ek_solver * s, double * t, double * dt, int * iteration)
{
  if (!s)
    return fail(EK_ERR_INVALID, "ek_solver_time: null solver");
  if (t)
    *t = s->t;
  if (dt)
    *dt = s->dt;
  if (iteration)
    *iteration = s->iteration;
  return EK_OK;
}

extern "C" ek_status
ek_solver_dt_history(ek_solver * s, double * dts, int n)
{
  if (!s || (!dts && n > 0) || n < 0 || n > s->iteration || n > s->dtcap)
    return fail(EK_ERR_INVALID, "ek_solver_dt_history: bad argument");
  if (n)
    EK_CUDA(cudaMemcpyAsync(dts, s->dtlog, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream), "dt history");
    EK_CUDA(cudaStreamSynchronize(s->stream), "dt history");
  return EK_OK;
}

extern "C" ek_status
ek_solver_get_state(ek_solver * s, double * U, int layout)
{
  if (!s || !U || !s->has_state || (layout != EK_LAYOUT_LEFT && layout != EK_LAYOUT_RIGHT))
    return fail(EK_ERR_INVALID, "ek_solver_get_state: bad argument");
  void * cur = s->U[s->iteration % 2];
  EK_CUDA(ek_fast::fill_ghosts(s->prec, cur, s->kp, s->p.mhd ? 8 : s->p.nbvar, s->stream), "ghosts");
  s->launches += 1;
  return state_to_host(s, cur, U, layout);
}

// restart file: a fixed header, then the FP64 LayoutLeft state, ghosts included
struct RestartHeader
{
  char    magic[8]; // "EKRSTRT1"
  int32_t dim, mhd, nbvar, isize, jsize, ksize;
  int32_t times_saved, iteration;
  double  t;
};

extern "C" ek_status
ek_solver_save_restart(ek_solver * s, const char * path, int times_saved)
{
  if (!s || !path || !s->has_state)
    return fail(EK_ERR_INVALID, "ek_solver_save_restart: bad argument");
  std::vector<double> h((size_t)s->kp.vstride * s->p.nbvar);
  ek_status           st = ek_solver_get_state(s, h.data(), EK_LAYOUT_LEFT);
  if (st != EK_OK)
    return st;
  RestartHeader hd;
  std::memset(&hd, 0, sizeof hd);
  std::memcpy(hd.magic, "EKRSTRT1", 8);
  hd.dim = s->p.dim, hd.mhd = s->p.mhd, hd.nbvar = s->p.nbvar;
  hd.isize = s->p.isize, hd.jsize = s->p.jsize, hd.ksize = s->p.dim == 3 ? s->p.ksize : 1;
  hd.times_saved = times_saved, hd.iteration = s->iteration;
  hd.t = s->t;
  FILE * f = std::fopen(path, "wb");
  if (!f)
    return fail(EK_ERR_INVALID, std::string("ek_solver_save_restart: cannot open ") + path);
  const bool ok = std::fwrite(&hd, sizeof hd, 1, f) == 1 && std::fwrite(h.data(), sizeof(double), h.size(), f) == h.size();
  if (std::fclose(f) != 0 || !ok)
    return fail(EK_ERR_INVALID, std::string("ek_solver_save_restart: write failed for ") + path);
  return EK_OK;
}

extern "C" ek_status
ek_solver_load_restart(ek_solver * s, const char * path, int reset_time, int * times_saved)
{
  if (!s || !path)
    return fail(EK_ERR_INVALID, "ek_solver_load_restart: bad argument");
  FILE * f = std::fopen(path, "rb");
  if (!f)
    return fail(EK_ERR_INVALID, std::string("ek_solver_load_restart: cannot open ") + path);
  RestartHeader hd;
  std::vector<double> h((size_t)s->kp.vstride * s->p.nbvar);
  bool ok = std::fread(&hd, sizeof hd, 1, f) == 1 && std::memcmp(hd.magic, "EKRSTRT1", 8) == 0;
  ok = ok && hd.dim == s->p.dim && hd.mhd == s->p.mhd && hd.nbvar == s->p.nbvar && hd.isize == s->p.isize &&
       hd.jsize == s->p.jsize && hd.ksize == (s->p.dim == 3 ? s->p.ksize : 1);
  ok = ok && std::fread(h.data(), sizeof(double), h.size(), f) == h.size();
  std::fclose(f);
  if (!ok)
    return fail(EK_ERR_INVALID, std::string("ek_solver_load_restart: not a restart file of this grid: ") + path);
  if (times_saved)
    *times_saved = hd.times_saved;
  return set_state_at(s, h.data(), EK_LAYOUT_LEFT, reset_time ? 0.0 : hd.t);
}

extern "C" ek_status
ek_solver_save_vtk(ek_solver * s, int step, const char * debug_name)
{
  if (!s || !s->has_state)
    return fail(EK_ERR_INVALID, "ek_solver_save_vtk: no state");
  std::vector<double> h((size_t)s->kp.vstride * s->p.nbvar);
  ek_status           st = ek_solver_get_state(s, h.data(), EK_LAYOUT_LEFT);
  if (st != EK_OK)
    return st;
  return ek_write_vtk(&s->p, h.data(), EK_LAYOUT_LEFT, step, debug_name);
}

extern "C" ek_status
ek_solver_totals(ek_solver * s, double out[3])
{
  if (!s || !out || !s->has_state)
    return fail(EK_ERR_INVALID, "ek_solver_totals: bad argument");
  cudaError_t e = ek_fast::totals(s->prec, s->U[s->iteration % 2], s->kp, s->p.nbvar, s->scratch3, s->stream);
  if (e == cudaErrorNotSupported)
    return fail(EK_ERR_UNSUPPORTED, "totals not available for this configuration");
  EK_CUDA(e, "totals");
  s->launches += s->p.mhd ? 2 : 1;
  EK_CUDA(cudaMemcpyAsync(out, s->scratch3, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream), "totals");
  EK_CUDA(cudaStreamSynchronize(s->stream), "totals");
  if (s->p.mhd)
  {
    // the device wrote an order-preserving key of max |div B|
    unsigned long long key;
    std::memcpy(&key, &out[2], sizeof key);
    out[2] = ekc::dkey_inv(key);
  }
  else
    out[2] = 0.0;
  const double cell = s->p.dx * s->p.dy * (s->p.dim == 3 ? s->p.dz : 1.0);
  out[0] *= cell;
  out[1] *= cell;
  return EK_OK;
}

extern "C" ek_status
ek_solver_device_state(ek_solver * s, void ** ptr, size_t * bytes)
{
  if (!s || !ptr)
    return fail(EK_ERR_INVALID, "ek_solver_device_state: bad argument");
  *ptr = s->U[s->iteration % 2];
  if (bytes)
    *bytes = s->state_bytes;
  return EK_OK;
}

extern "C" ek_status
ek_solver_synchronize(ek_solver * s)
{
  if (!s)
    return fail(EK_ERR_INVALID, "ek_solver_synchronize: null solver");
  EK_CUDA(cudaStreamSynchronize(s->stream), "synchronize");
  return EK_OK;
}

extern "C" ek_status
ek_solver_launch_count(ek_solver * s, long long * n)
{
  if (!s || !n)
    return fail(EK_ERR_INVALID, "ek_solver_launch_count: bad argument");
  *n = s->launches;
  return EK_OK;
}

extern "C" ek_status
ek_solver_stream(ek_solver * s, void ** stream)
{
  if (!s || !stream)
    return fail(EK_ERR_INVALID, "ek_solver_stream: bad argument");
  *stream = (void *)s->stream;
  return EK_OK;
}

extern "C" ek_status
ek_solver_set_profiling(ek_solver * s, int enable)
{
  if (!s)
    return fail(EK_ERR_INVALID, "ek_solver_set_profiling: null solver");
  drain_events(s);
  s->profiling = enable != 0;
  for (int i = 0; i < 4; ++i)
  {
    s->kernel_ms[i] = 0.0;
    s->kernel_n[i] = 0;
  }
  return EK_OK;
}

extern "C" ek_status
ek_solver_kernel_time(ek_solver * s, int kernel, double * total_ms, long long * launches)
{
  if (!s || kernel < 0 || kernel > 3)
    return fail(EK_ERR_INVALID, "ek_solver_kernel_time: bad argument");
  drain_events(s);
  if (total_ms)
    *total_ms = s->kernel_ms[kernel];
  if (launches)
    *launches = s->kernel_n[kernel];
  return EK_OK;
}

extern "C" ek_status
ek_solver_hlld_repairs(ek_solver * s, long long * tiles)
{
  if (!s || !tiles)
    return fail(EK_ERR_INVALID, "ek_solver_hlld_repairs: bad argument");
  *tiles = 0;
  if (!has_repair(s))
    return EK_OK;
  unsigned long long n = 0;
  EK_CUDA(cudaMemcpyAsync(&n, static_cast<char *>(s->work) + 2 * sizeof(int), sizeof n, cudaMemcpyDeviceToHost,
                          s->stream),
          "hlld repairs");
  EK_CUDA(cudaStreamSynchronize(s->stream), "hlld repairs");
  *tiles = (long long)n;
  return EK_OK;
}

// ===========================================================================
// Ensemble of independent 2D hydro runs
// ===========================================================================
struct ek_ensemble
{
  int                      n = 0;
  int                      prec = 0;
  bool                     exact = false;
  cudaStream_t             stream = nullptr;
  std::vector<ek_solver *> views; // per-instance views (no own device memory)
  void *                   states = nullptr; // all ping-pong states
  DevClock *               clocks = nullptr;
  double *                 dtlogs = nullptr;
  ekc::EnsInstance *       d_insts = nullptr;
  ekc::EnsTile *           d_tiles = nullptr;
  int *                    d_step = nullptr;
  double *                 d_totals = nullptr;
  void *                   d_scalars = nullptr; // per-instance step scalars (64 B each)
  int                      ntiles = 0;
  int                      grid = 0;
  int                      step = 0; // host copy of the device step counter
  long long                cells = 0;
  long long                launches = 0;
  cudaGraph_t              graph = nullptr;
  cudaGraphExec_t          graph_exec = nullptr;
  int                      graph_steps = 0;
};

extern "C" ek_status ek_ensemble_time(ek_ensemble * e, int i, double * t, double * dt, int * iteration);

extern "C" ek_status
ek_ensemble_destroy(ek_ensemble * e)
{
  if (!e)
    return EK_OK;
  if (e->stream)
    cudaStreamSynchronize(e->stream);
  for (auto v : e->views)
    ek_solver_destroy(v);
  if (e->graph_exec)
    cudaGraphExecDestroy(e->graph_exec);
  if (e->graph)
    cudaGraphDestroy(e->graph);
  cudaFree(e->states);
  cudaFree(e->clocks);
  cudaFree(e->dtlogs);
  cudaFree(e->d_insts);
  cudaFree(e->d_tiles);
  cudaFree(e->d_step);
  cudaFree(e->d_totals);
  cudaFree(e->d_scalars);
  if (e->stream)
    cudaStreamDestroy(e->stream);
  delete e;
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_create(const ek_params * params, int n, ek_ensemble ** out)
{
  if (!params || n < 1 || !out)
    return fail(EK_ERR_INVALID, "ek_ensemble_create: bad argument");
  *out = nullptr;
  for (int i = 0; i < n; ++i)
  {
    const ek_params & p = params[i];
    ek_status v = ek_internal::validate(p);
    if (v != EK_OK)
      return fail(v, "instance " + std::to_string(i) + ": " + ek_last_error());
    if (p.dim != 2 || p.mhd)
      return fail(EK_ERR_UNSUPPORTED, "ensembles hold Hydro_Muscl_2D runs");
    if (p.riemann != 3)
      return fail(EK_ERR_UNSUPPORTED, "ensembles use riemann=hllc");
    if (p.gravity_enabled)
      return fail(EK_ERR_UNSUPPORTED, "ensembles run without gravity");
    if (p.precision != params[0].precision || p.exact_fp != params[0].exact_fp)
      return fail(EK_ERR_INVALID, "all instances of an ensemble share precision and exact_fp");
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(EK_ERR_NO_DEVICE, "no CUDA device available");

  ek_ensemble * e = new ek_ensemble();
  e->n = n;
  e->prec = params[0].precision;
  e->exact = params[0].exact_fp != 0;
  int dev = 0;
  cudaGetDevice(&dev);
  // layout: instance i owns two states at offsets off[i], off[i] + bytes[i]
  std::vector<size_t> off(n), bytes(n);
  size_t              total = 0;
  int                 dtcap = 1;
  for (int i = 0; i < n; ++i)
  {
    ekc::KParams k = ek_internal::make_kparams(params[i]);
    bytes[i] = (ek_internal::state_bytes(params[i], k) + 255) / 256 * 256;
    off[i] = total;
    total += 2 * bytes[i];
    const int cap = params[i].nStepmax > 0 ? (params[i].nStepmax < (1 << 20) ? params[i].nStepmax + 1 : (1 << 20)) : 1;
    dtcap = cap > dtcap ? cap : dtcap;
    e->cells += (long long)params[i].nx * params[i].ny;
  }
  cudaError_t err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (err == cudaSuccess)
    err = cudaMalloc(&e->states, total);
  if (err == cudaSuccess)
    err = cudaMemsetAsync(e->states, 0, total, e->stream);
  if (err == cudaSuccess)
    err = cudaMalloc((void **)&e->clocks, sizeof(DevClock) * n);
  if (err == cudaSuccess)
    err = cudaMalloc((void **)&e->dtlogs, sizeof(double) * (size_t)dtcap * n);
  if (err == cudaSuccess)
    err = cudaMalloc((void **)&e->d_insts, sizeof(ekc::EnsInstance) * n);
  if (err == cudaSuccess)
    err = cudaMalloc((void **)&e->d_step, sizeof(int));
  if (err == cudaSuccess)
    err = cudaMemsetAsync(e->d_step, 0, sizeof(int), e->stream);
  if (err == cudaSuccess)
    err = cudaMalloc((void **)&e->d_totals, 2 * sizeof(double) * n);
  std::vector<ekc::EnsInstance> h_insts(n);
  std::vector<ekc::EnsTile>     tiles;
  if (err == cudaSuccess)
  {
    for (int i = 0; i < n; ++i)
    {
      ek_solver * v = new ek_solver();
      v->owns = false;
      v->p = params[i];
      v->kp = ek_internal::make_kparams(params[i]);
      v->prec = e->prec;
      v->exact = e->exact;
      v->device = dev;
      v->stream = e->stream;
      v->state_bytes = ek_internal::state_bytes(params[i], v->kp);
      v->U[0] = (char *)e->states + off[i];
      v->U[1] = (char *)e->states + off[i] + bytes[i];
      v->clk = e->clocks + i;
      v->dtlog = e->dtlogs + (size_t)i * dtcap;
      v->dtcap = dtcap;
      v->scratch3 = nullptr;
      e->views.push_back(v);
      h_insts[i].P = v->kp;
      h_insts[i].U[0] = v->U[0];
      h_insts[i].U[1] = v->U[1];
      h_insts[i].clk = v->clk;
      // tiles of the 2D step kernel, instance-major
      const int tx = (params[i].nx + EK_H2_TX - 1) / EK_H2_TX, ty = (params[i].ny + EK_H2_TY - 1) / EK_H2_TY;
      for (int by = 0; by < ty; ++by)
        for (int bx = 0; bx < tx; ++bx)
          tiles.push_back({ i, bx, by });
    }
    e->ntiles = (int)tiles.size();
    err = cudaMalloc((void **)&e->d_tiles, sizeof(ekc::EnsTile) * tiles.size());
    if (err == cudaSuccess)
      err = cudaMalloc(&e->d_scalars, 64 * (size_t)n);
  }
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(e->d_insts, h_insts.data(), sizeof(ekc::EnsInstance) * n, cudaMemcpyHostToDevice,
                          e->stream);
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(e->d_tiles, tiles.data(), sizeof(ekc::EnsTile) * tiles.size(),
                          cudaMemcpyHostToDevice, e->stream);
  if (err == cudaSuccess)
    err = cudaStreamSynchronize(e->stream);
  if (err != cudaSuccess)
  {
    ek_status st = cuda_fail(err, "ek_ensemble_create");
    ek_ensemble_destroy(e);
    return st;
  }
  e->grid = e->exact ? ek_exact::ensemble2d_grid(e->prec) : ek_fast::ensemble2d_grid(e->prec);
  *out = e;
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_set_state(ek_ensemble * e, int i, const double * U, int layout)
{
  if (!e || i < 0 || i >= e->n)
    return fail(EK_ERR_INVALID, "ek_ensemble_set_state: bad instance");
  if (e->step != 0)
    return fail(EK_ERR_INVALID, "ek_ensemble_set_state: states are set before the first step");
  return ek_solver_set_state(e->views[i], U, layout);
}

extern "C" ek_status
ek_ensemble_get_state(ek_ensemble * e, int i, double * U, int layout)
{
  if (!e || i < 0 || i >= e->n)
    return fail(EK_ERR_INVALID, "ek_ensemble_get_state: bad instance");
  double    t, dt;
  int       it;
  ek_status st = ek_ensemble_time(e, i, &t, &dt, &it); // current buffer follows the device clock
  if (st != EK_OK)
    return st;
  return ek_solver_get_state(e->views[i], U, layout);
}

static ek_status
ensemble_launch_steps(ek_ensemble * e, int nsteps)
{
  for (int k = 0; k < nsteps; ++k)
  {
    cudaError_t err = e->exact ? ek_exact::ensemble2d_step(e->prec, e->d_insts, e->n, e->d_tiles, e->ntiles,
                                                           e->d_step, e->d_scalars, e->grid, e->stream)
                               : ek_fast::ensemble2d_step(e->prec, e->d_insts, e->n, e->d_tiles, e->ntiles,
                                                          e->d_step, e->d_scalars, e->grid, e->stream);
    if (err != cudaSuccess)
      return cuda_fail(err, "ensemble step");
  }
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_run(ek_ensemble * e, int nsteps, int use_graph)
{
  if (!e || nsteps < 0)
    return fail(EK_ERR_INVALID, "ek_ensemble_run: bad argument");
  for (auto v : e->views)
    if (!v->has_state)
      return fail(EK_ERR_INVALID, "ek_ensemble_run: every instance needs a state");
  if (nsteps == 0)
    return EK_OK;
  if (!use_graph)
  {
    ek_status st = ensemble_launch_steps(e, nsteps);
    if (st != EK_OK)
      return st;
  }
  else
  {
    if (!e->graph_exec || e->graph_steps != nsteps)
    {
      if (e->graph_exec)
        cudaGraphExecDestroy(e->graph_exec);
      if (e->graph)
        cudaGraphDestroy(e->graph);
      e->graph_exec = nullptr;
      e->graph = nullptr;
      EK_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
      ek_status st = ensemble_launch_steps(e, nsteps);
      cudaGraph_t g = nullptr;
      cudaError_t ce = cudaStreamEndCapture(e->stream, &g);
      if (st != EK_OK)
        return st;
      EK_CUDA(ce, "graph capture");
      e->graph = g;
      EK_CUDA(cudaGraphInstantiate(&e->graph_exec, e->graph, 0), "graph instantiate");
      e->graph_steps = nsteps;
    }
    EK_CUDA(cudaGraphLaunch(e->graph_exec, e->stream), "graph launch");
  }
  e->launches += 3LL * nsteps;
  e->step += nsteps;
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_synchronize(ek_ensemble * e)
{
  if (!e)
    return fail(EK_ERR_INVALID, "ek_ensemble_synchronize: null ensemble");
  EK_CUDA(cudaStreamSynchronize(e->stream), "synchronize");
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_time(ek_ensemble * e, int i, double * t, double * dt, int * iteration)
{
  if (!e || i < 0 || i >= e->n)
    return fail(EK_ERR_INVALID, "ek_ensemble_time: bad instance");
  ek_solver * v = e->views[i];
  DevClock    h;
  ek_status   st = read_clock(v, &h);
  if (st != EK_OK)
    return st;
  v->iteration = h.iteration;
  v->t = h.t[h.iteration % 3];
  if (h.iteration > 0)
    v->dt = h.last_dt;
  return ek_solver_time(v, t, dt, iteration);
}

extern "C" ek_status
ek_ensemble_dt_history(ek_ensemble * e, int i, double * dts, int n)
{
  if (!e || i < 0 || i >= e->n)
    return fail(EK_ERR_INVALID, "ek_ensemble_dt_history: bad instance");
  double t, dt;
  int    it;
  ek_status st = ek_ensemble_time(e, i, &t, &dt, &it);
  if (st != EK_OK)
    return st;
  return ek_solver_dt_history(e->views[i], dts, n);
}

extern "C" ek_status
ek_ensemble_totals(ek_ensemble * e, double * out)
{
  if (!e || !out)
    return fail(EK_ERR_INVALID, "ek_ensemble_totals: bad argument");
  EK_CUDA(ek_fast::ensemble_totals(e->prec, e->d_insts, e->n, e->d_step, e->d_totals, e->stream), "totals");
  EK_CUDA(cudaMemcpyAsync(out, e->d_totals, 2 * sizeof(double) * e->n, cudaMemcpyDeviceToHost, e->stream),
          "totals");
  EK_CUDA(cudaStreamSynchronize(e->stream), "totals");
  for (int i = 0; i < e->n; ++i)
  {
    const double cell = e->views[i]->p.dx * e->views[i]->p.dy;
    out[2 * i] *= cell;
    out[2 * i + 1] *= cell;
  }
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_info(ek_ensemble * e, long long * interior_cells, int * tiles, int * grid, long long * launches)
{
  if (!e)
    return fail(EK_ERR_INVALID, "ek_ensemble_info: null ensemble");
  if (interior_cells)
    *interior_cells = e->cells;
  if (tiles)
    *tiles = e->ntiles;
  if (grid)
    *grid = e->grid;
  if (launches)
    *launches = e->launches;
  return EK_OK;
}

extern "C" ek_status
ek_ensemble_stream(ek_ensemble * e, void ** stream)
{
  if (!e || !stream)
    return fail(EK_ERR_INVALID, "ek_ensemble_stream: bad argument");
  *stream = (void *)e->stream;
  return EK_OK;
}
