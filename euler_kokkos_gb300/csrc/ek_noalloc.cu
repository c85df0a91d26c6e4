// ek_mhd3d_step_noalloc: one MHD_Muscl_3D FP64 time step on caller-owned
// device arrays that allocates no device memory.
//
// The step: boundaries of U_in (by index mapping), the CFL dt of that state,
// the trace, fluxes, emfs and update into U_out -- the same kernels as a step
// of ek_solver_next_iteration.
//
// Which callers cannot allocate, and why: a host code that hands the library
// only the two state arrays of the step and keeps every other byte of device
// memory in its own pool (a Kokkos memory space, an embedding code that
// budgets the whole HBM).  Such a caller cannot give the library a trace
// buffer, and a cudaMalloc / cudaFree pair per step would synchronise the
// device twice per step.  The step's only temporary, the 47-value compact
// trace of the z-marching trace kernel, therefore lives in a fixed file-scope
// device array.
//
// Limits and rules:
//   * the array is EK_NOALLOC_SCRATCH_BYTES (64 MiB); every GPU context that
//     loads this library holds it until the process exits;
//   * FP64 trace = 48 * 8 bytes per trace cell (47 values and one spare), the trace cells being
//     32 ceil((nx+2)/32) x (ny+2) x (nz+2) (blocks of 32 along x): grids whose
//     trace exceeds 64 MiB - 512 bytes (a 50^3 interior is the largest cube)
//     are rejected with EK_ERR_INVALID;
//   * the first call in each device context resolves the array's address with
//     cudaGetSymbolAddress (that device current); make that first call before
//     any stream capture.  The address is cached per device together with the
//     context's unique id, so a call after cudaDeviceReset (a new context)
//     resolves it again instead of using the old context's address;
//   * calls on one device share the array: two calls in flight at once
//     (different streams or host threads) race on it and must be serialised
//     by the caller, e.g. by issuing them on one stream;
//   * nothing in the array has to start at zero: each call writes the clock
//     slots itself (a one-thread kernel, before the step's kernels) and the
//     trace kernel writes every trace value the update kernel reads;
//   * a call with dt_out = NULL does not wait for its step, so it cannot
//     report a non-finite dt itself: the next call's set-up kernel records
//     it (sticky flag in the array) and the next call with dt_out reports it
//     as EK_ERR_NONFINITE (its own step is still taken), then clears the flag;
//     a call with dt_out reports its own step's outcome itself.
#include <cmath>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/ek_gb300.h"
#include "ek_internal.h"
#include "ek_launch.h"

// the scratch: file scope, fixed size, one copy per device context
static __device__ __align__(256) unsigned char g_noalloc_scratch[EK_NOALLOC_SCRATCH_BYTES];

namespace
{

// [0, 256): the step's device clock; [256, 264): the dt of the step;
// [264, 272): StepFlags; [512, EK_NOALLOC_SCRATCH_BYTES): the compact trace
constexpr size_t kClockOffset = 0;
constexpr size_t kDtOffset = 256;
constexpr size_t kFlagsOffset = 264;
constexpr size_t kTraceOffset = 512;
static_assert(sizeof(ekc::DevClock) <= kDtOffset - kClockOffset, "clock region too small");

// sticky: an earlier call's step ended with a non-finite dt (1) or a device
// error flag (2) that no call has reported yet; armed: a call has set up a
// step whose outcome the next set-up inspects
struct StepFlags
{
  unsigned int sticky, armed;
};
static_assert(kFlagsOffset + sizeof(StepFlags) <= kTraceOffset, "flag region too small");

constexpr int kMaxDevices = 64;
std::mutex    g_setup_mutex;
struct ScratchAddr
{
  void *             ptr;
  unsigned long long ctx_id;
};
ScratchAddr g_scratch_addr[kMaxDevices] = {};

// unique id of the calling thread's current context (cuCtxGetId, reached
// through the runtime's driver entry points so the library does not link
// libcuda); 0 when the driver does not provide it
unsigned long long
current_context_id()
{
  using GetCurrent = int (*)(void **);
  using GetId = int (*)(void *, unsigned long long *);
  static GetCurrent get_current = nullptr;
  static GetId      get_id = nullptr;
  static bool       looked = false;
  if (!looked)
  {
    void *                          f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    looked = true;
  }
  void *             ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0)
    return 0;
  return id;
}

// once per device context, with that device current
ek_status
scratch_address(int dev, unsigned char ** out)
{
  if (dev < 0 || dev >= kMaxDevices)
    return ek_internal::fail(EK_ERR_UNSUPPORTED, "ek_mhd3d_step_noalloc: device ordinal " + std::to_string(dev) +
                                                     " beyond the " + std::to_string(kMaxDevices) + " supported");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  const unsigned long long    id = current_context_id();
  ScratchAddr &               a = g_scratch_addr[dev];
  // resolve again when the context changed (id 0: unknown, resolve every time)
  if (!a.ptr || id == 0 || a.ctx_id != id)
  {
    void *      ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
    if (e != cudaSuccess)
      return ek_internal::fail(EK_ERR_CUDA, std::string("ek_mhd3d_step_noalloc: cudaGetSymbolAddress: ") +
                                                cudaGetErrorString(e));
    a.ptr = ptr;
    a.ctx_id = id;
  }
  *out = static_cast<unsigned char *>(a.ptr);
  return EK_OK;
}

// the clock of a single step starting at t0 (slot 0 committed, CFL slot at
// the lowest key, dt slot NaN until the update kernel writes it)
// Before the reset, the outcome of the previous call's step (when one was set
// up) goes into the sticky flags, so an asynchronous call's non-finite dt or
// device error is reported by the next call that waits for its step.
__global__ void
noalloc_clock_init(ekc::DevClock * clk, double t0, double * dt_slot, StepFlags * fl)
{
  if (fl->armed)
  {
    const double d = *dt_slot;
    if (!(d > 0.0) || !isfinite(d))
      fl->sticky |= 1u;
    if (clk->error != 0)
      fl->sticky |= 2u;
  }
  fl->armed = 1u;
  for (int s = 0; s < 3; ++s)
  {
    clk->key[s] = EK_KEY_LOWEST;
    clk->t[s] = 0.0;
    clk->sid[s] = -1;
    clk->sc[s].step = -1;
    clk->sc[s].active = 0;
    clk->fin[s] = 0;
  }
  clk->sid[0] = 0;
  clk->t[0] = t0;
  clk->iteration = 0;
  clk->error = 0;
  clk->dtlog = dt_slot;
  clk->dtcap = 1;
  clk->last_dt = 0.0;
  *dt_slot = __longlong_as_double(0x7ff8000000000000ll);
}

} // namespace

extern "C" ek_status
ek_mhd3d_step_noalloc(const ek_params * params, const double * U_in, double * U_out, double t,
                      double * dt_out, void * stream)
{
  using ek_internal::fail;
  if (!params || !U_in || !U_out)
    return fail(EK_ERR_INVALID, "ek_mhd3d_step_noalloc: null argument");
  const ek_params & p = *params;
  {
    ek_status v = ek_internal::validate(p);
    if (v != EK_OK)
      return v;
  }
  if (!p.mhd || p.dim != 3)
    return fail(EK_ERR_UNSUPPORTED, "ek_mhd3d_step_noalloc: MHD_Muscl_3D only");
  if (p.precision != EK_PREC_FP64)
    return fail(EK_ERR_UNSUPPORTED, "ek_mhd3d_step_noalloc: the state arrays are FP64 (precision must be fp64)");
  const ekc::KParams kp = ek_internal::make_kparams(p);
  const size_t       trace_bytes = ek_exact::mhd_work_bytes(0, kp);
  if (trace_bytes > EK_NOALLOC_SCRATCH_BYTES - kTraceOffset)
    return fail(EK_ERR_INVALID,
                "ek_mhd3d_step_noalloc: grid too large for the static scratch: the trace needs " +
                    std::to_string(trace_bytes) + " bytes (384 per trace cell, 32 ceil((nx+2)/32) x (ny+2) x "
                    "(nz+2) cells), the scratch holds " +
                    std::to_string(EK_NOALLOC_SCRATCH_BYTES - kTraceOffset));
  const size_t state = ek_internal::state_bytes(p, kp);
  const char * a = reinterpret_cast<const char *>(U_in);
  const char * b = reinterpret_cast<const char *>(U_out);
  if (a < b + state && b < a + state)
    return fail(EK_ERR_INVALID, "ek_mhd3d_step_noalloc: U_in and U_out overlap");
  if (!(t < p.tEnd - 1e-14))
    return fail(EK_ERR_INVALID, "ek_mhd3d_step_noalloc: t >= tEnd, the run is finished");

  int dev = 0;
  {
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
      return fail(EK_ERR_NO_DEVICE, std::string("ek_mhd3d_step_noalloc: ") + cudaGetErrorString(e));
  }
  unsigned char * scratch = nullptr;
  {
    ek_status s = scratch_address(dev, &scratch);
    if (s != EK_OK)
      return s;
  }
  ekc::DevClock * clk = reinterpret_cast<ekc::DevClock *>(scratch + kClockOffset);
  double *        dt_slot = reinterpret_cast<double *>(scratch + kDtOffset);
  StepFlags *     flags = reinterpret_cast<StepFlags *>(scratch + kFlagsOffset);
  void *          trace = scratch + kTraceOffset;
  cudaStream_t    st = static_cast<cudaStream_t>(stream);

  noalloc_clock_init<<<1, 1, 0, st>>>(clk, t, dt_slot, flags);
  cudaError_t e = cudaGetLastError();
  for (int phase = 0; phase < 3 && e == cudaSuccess; ++phase)
    e = p.exact_fp ? ek_exact::mhd_step(0, phase, U_in, U_out, trace, kp, clk, 0, false, st)
                   : ek_fast::mhd_step(0, phase, U_in, U_out, trace, kp, clk, 0, false, st);
  if (e != cudaSuccess)
    return fail(EK_ERR_CUDA, std::string("ek_mhd3d_step_noalloc: launch: ") + cudaGetErrorString(e));
  if (!dt_out)
    return EK_OK;
  // this step's dt and device flags, and what earlier asynchronous calls left
  StepFlags fl{};
  int       dev_error = 0;
  e = cudaMemcpyAsync(dt_out, dt_slot, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&fl, flags, sizeof fl, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&dev_error, &clk->error, sizeof dev_error, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(st);
  if (e != cudaSuccess)
    return fail(EK_ERR_CUDA, std::string("ek_mhd3d_step_noalloc: dt read: ") + cudaGetErrorString(e));
  // this call reports its own outcome and what the flags hold: disarm and
  // clear them (ordered before the next call on this stream)
  e = cudaMemsetAsync(flags, 0, sizeof(StepFlags), st);
  if (e != cudaSuccess)
    return fail(EK_ERR_CUDA, std::string("ek_mhd3d_step_noalloc: flag reset: ") + cudaGetErrorString(e));
  if (fl.sticky != 0)
  {
    return fail(EK_ERR_NONFINITE, std::string("ek_mhd3d_step_noalloc: an earlier call without dt_out ended ") +
                                      ((fl.sticky & 1u) ? "with a non-finite or non-positive dt"
                                                        : "with a device error flag set") +
                                      " (this call's step was taken)");
  }
  if (dev_error & ekc::EK_DEVERR_TMA_TIMEOUT)
    return fail(EK_ERR_CUDA, "ek_mhd3d_step_noalloc: a bounded wait of the step expired");
  if (!(*dt_out > 0.0) || !std::isfinite(*dt_out))
    return fail(EK_ERR_NONFINITE, "ek_mhd3d_step_noalloc: time step is not finite and positive (dt = " +
                                      std::to_string(*dt_out) + ")");
  return EK_OK;
}
