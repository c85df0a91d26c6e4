/*
 * ek_gb300.h -- C ABI of the GB300-native unsplit MUSCL-Hancock step.
 *
 * This is the drop-in boundary for the reference's solver path
 * (pkestene/euler_kokkos, implementationVersion=0 of SolverHydroMuscl and
 * SolverMHDMuscl).  Plain pointers and sizes only.  Every function returns an
 * ek_status; no function aborts or exits the process (the reference aborts
 * on an unknown solver name, SolverFactory.h:105-113, and exits on invalid
 * parameters, HydroParams.cpp:352-358; here those are EK_ERR_INVALID).
 *
 * State arrays exchanged with the caller hold the FULL ghost-inclusive
 * conserved state (isize x jsize [x ksize] x nbvar, FP64) in one of the two
 * Kokkos layouts of the reference (kokkos_shared.h:24-42):
 *   EK_LAYOUT_LEFT  -- U[((var*ksize + k)*jsize + j)*isize + i] (Kokkos CUDA)
 *   EK_LAYOUT_RIGHT -- U[((i*jsize + j)*ksize + k)*nbvar + var] (Kokkos OpenMP)
 * Variable order ID=0, IP=1 (total energy), IU, IV, IW, IA, IB, IC
 * (enums.h:17-40); MHD face-centred B: U(i,j,k,IA) is Bx on the left x-face.
 */
#ifndef EK_GB300_H
#define EK_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EK_ABI_VERSION 1

typedef enum ek_status
{
  EK_OK = 0,
  EK_ERR_INVALID = 1,     /* bad argument, bad parameter, unknown solver name */
  EK_ERR_UNSUPPORTED = 2, /* a configuration this library does not implement */
  EK_ERR_CUDA = 3,        /* a CUDA runtime error (see ek_last_error) */
  EK_ERR_NO_MEMORY = 4,   /* device or pinned-host allocation failed */
  EK_ERR_NONFINITE = 5,   /* the time step became non-finite or non-positive */
  EK_ERR_PARSE = 6,       /* malformed .ini text */
  EK_ERR_NO_DEVICE = 7    /* no CUDA device */
} ek_status;

typedef enum ek_layout
{
  EK_LAYOUT_LEFT = 0,
  EK_LAYOUT_RIGHT = 1
} ek_layout;

typedef enum ek_precision
{
  EK_PREC_FP64 = 0, /* the drop-in: FP64 state and arithmetic */
  EK_PREC_MIXED = 1 /* FP32 state/arithmetic with FP64 islands (dt, CT face B, cancellation,
                       ill-conditioned HLLD star states: ek_solver_hlld_repairs) */
} ek_precision;

/* Run parameters.  Field meanings and defaults follow HydroParams
 * (HydroParams.h:32-197, HydroParams.cpp:37-180, 327-359) and SolverBase
 * (SolverBase.cpp:21-40).  ek_params_from_ini fills every field exactly as
 * the reference's ConfigMap + HydroParams do, including the float rounding
 * of every real read through strtof (ConfigMap.cpp:37-46). */
typedef struct ek_params
{
  int    dim;   /* 2 or 3 */
  int    mhd;   /* 0 hydro (SolverHydroMuscl), 1 MHD (SolverMHDMuscl) */
  int    nx, ny, nz;
  int    ghost_width; /* 2 hydro, 3 MHD */
  int    nbvar;       /* 4 hydro 2D, 5 hydro 3D, 8 MHD */
  int    isize, jsize, ksize;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double dx, dy, dz;
  int    bc[6]; /* boundary_type_{xmin,xmax,ymin,ymax,zmin,zmax}: 1 reflect, 2 outflow, 3 periodic */
  double gamma0, gamma6, cfl, slope_type, smallr, smallc, smallp, smallpp, cIso, Omega0;
  int    riemann; /* 0 approx, 1 llf, 2 hll, 3 hllc, 4 hlld (enums.h:175-182) */
  int    implementation_version;
  int    nStepmax;
  double tEnd;
  double tCurrent; /* [run] tCurrent: initial m_t */
  int    nOutput;
  int    nlog;
  int    precision; /* ek_precision; [gb300] precision = fp64 | mixed */
  int    exact_fp;  /* 1: FP64 kernels with the reference's arithmetic, no FMA contraction and
                       every division, bitwise equal to it ([gb300] exact = 1) */
  int    kchunk;    /* 3D planes per CTA column (0: automatic; [gb300] kchunk) */
  int    mhd_stage; /* MHD update kernel stages the trace planes in shared memory ([gb300] mhd_stage) */
  char   solver_name[32];
  char   problem[32];
  char   output_dir[256];    /* [output] outputDir ("./") */
  char   output_prefix[128]; /* [output] outputPrefix ("output") */
  int    vtk_enabled;        /* [output] vtk_enabled (1) */
  int    vtk_ascii;          /* [output] outputVtkAscii (0) */
  /* static gravity, GravityParams (GravityParams.h:22-37, SolverBase.cpp:38-39);
   * used by the hydro solvers only, as in the reference */
  int    gravity_enabled;       /* [gravity] enabled (0) */
  int    gravity_static;        /* [gravity] static (0): read, no effect (as in the reference) */
  int    gravity_hancock;       /* [gravity] hancock_predictor_enabled (0) */
  int    gravity_well_balanced; /* [gravity] well_balanced_reconstruction_enabled (0): read, no effect */
  double gravity[3];            /* uniform field the solver starts with: [rayleigh_taylor] gx, gy, gz
                                   (0, -0.1, 0) when problem = rayleigh_taylor, the field the
                                   reference's init writes (HydroInitFunctors2D.h:735-771); else 0 */
  int    no_tma;                /* 1: the 3D hydro kernel loads every plane with plain loads instead of
                                   staging interior planes by tensor copies ([gb300] tma = 0) */
} ek_params;

typedef struct ek_solver ek_solver;

/* Library identification (does not touch the GPU). */
int          ek_abi_version(void);
const char * ek_status_string(ek_status s);
/* Message of the last error raised on the calling thread ("" if none). */
const char * ek_last_error(void);

/* Parse .ini text (ConfigMap semantics) and derive the run parameters
 * (HydroParams::HydroParams + init).  Replaces ConfigMap(filename) and
 * HydroParams(configMap, par_env) of main.cpp:100-110.  CPU only. */
ek_status ek_params_from_ini(const char * text, size_t len, ek_params * out);

/* Create a solver on the current CUDA device.  Replaces
 * SolverFactory::Instance().create(name, params, configMap)
 * (SolverFactory.h:83-116) for the names Hydro_Muscl_2D/3D, MHD_Muscl_2D/3D;
 * the initial condition is not computed here but injected with
 * ek_solver_set_state (the reference's init(U) becomes the caller's). */
ek_status ek_solver_create(const ek_params * params, ek_solver ** out);
ek_status ek_solver_destroy(ek_solver * s);

/* Inject a full state (host memory) and replay the reference constructor
 * tail: make_boundaries(U), deep_copy(U2,U), [MHD: convertToPrimitives(U)],
 * compute_dt() (SolverHydroMuscl.h:276-286, SolverMHDMuscl.h:384-397).
 * Sets m_t = params.tCurrent and m_iteration = 0. */
ek_status ek_solver_set_state(ek_solver * s, const double * U, int layout);
/* Copy the current state (U if m_iteration is even, else U2) to host memory,
 * ghost cells filled by the boundary conditions (save_solution path,
 * SolverHydroMuscl.h:749-762). */
ek_status ek_solver_get_state(ek_solver * s, double * U, int layout);

/* Static gravity field of a hydro solver with params->gravity_enabled:
 * replaces SolverHydroMuscl::gravity_field (SolverHydroMuscl.h:86-87, a
 * VectorField of dim components over the full grid, ghosts included, filled
 * by the problem's init).  G holds dim components per cell in the given
 * layout (LayoutLeft: G[((comp*ksize + k)*jsize + j)*isize + i];
 * LayoutRight: G[((i*jsize + j)*ksize + k)*dim + comp]); NULL returns to the
 * uniform params->gravity.  The CFL of the current state is recomputed (as the
 * constructor's compute_dt() after init), so the next step uses the new
 * field.  EK_ERR_INVALID when gravity is not enabled or the solver is MHD. */
ek_status ek_solver_set_gravity_field(ek_solver * s, const double * G, int layout);

/* SolverBase::compute_dt (SolverBase.cpp:124-154): dt on the current state,
 * clamped so that t + dt <= tEnd.  Writes m_dt to *dt when dt != NULL. */
ek_status ek_solver_compute_dt(ek_solver * s, double * dt);
/* SolverBase::next_iteration (SolverBase.cpp:180-195): one fused step, then
 * ++m_iteration, m_t += m_dt.  Synchronises to read back m_dt, as the
 * reference's parallel_reduce does. */
ek_status ek_solver_next_iteration(ek_solver * s);
/* while (!finished() && n < nsteps) next_iteration(), without a host round
 * trip per step; *done receives the number of steps taken. */
ek_status ek_solver_run(ek_solver * s, int nsteps, int * done);
/* SolverBase::finished (SolverBase.cpp:170-176) */
ek_status ek_solver_finished(ek_solver * s, int * finished);
/* m_t, m_dt (the last step's dt) and m_iteration */
ek_status ek_solver_time(ek_solver * s, double * t, double * dt, int * iteration);
/* dt of steps 0..n-1 (the reference's printed dt sequence) */
ek_status ek_solver_dt_history(ek_solver * s, double * dts, int n);
/* FP64 totals over the interior: [mass, total energy, max |div B| (MHD, else 0)] */
ek_status ek_solver_totals(ek_solver * s, double out[3]);
/* Device pointer / byte size of the current state (zero-copy access; the
 * storage type is FP64, or FP32 hydro variables + FP64 face B in the mixed
 * form).  Valid until the next step. */
ek_status ek_solver_device_state(ek_solver * s, void ** ptr, size_t * bytes);
/* Block until all work of the solver is done; reports device-side errors. */
ek_status ek_solver_synchronize(ek_solver * s);
/* Number of kernel launches issued by this solver so far. */
ek_status ek_solver_launch_count(ek_solver * s, long long * n);

/* Diagnostic: run the bounded mbarrier wait that guards the step kernels'
 * tensor copies on a barrier nothing completes, with a limit of limit_us
 * microseconds, on the current device.  *expired = 1 when every thread's wait
 * gave up (the kernel then left normally), *elapsed_us = the longest wait.
 * Shows that a copy that never lands ends in an error status, not a hang. */
ek_status ek_selftest_bounded_wait(int limit_us, int * expired, double * elapsed_us);

/* Diagnostic: the device's CUDA-core FMA throughput in TFLOP/s (2 FLOPs per
 * FMA), FP64 (precision EK_PREC_FP64) or FP32 (otherwise), measured with
 * CUDA events over independent FMA chains on every SM (best of 3 launches of
 * a few milliseconds).  The denominator of the step's FLOP roofline. */
ek_status ek_measure_fma_rate(int precision, double * tflops);

/* The CUDA stream (cudaStream_t) all work of the solver is issued on. */
ek_status ek_solver_stream(ek_solver * s, void ** stream);

/* Kernel timing with CUDA events recorded on the solver's stream around
 * every launch of the step kernels (no counterpart in the reference, whose
 * timers wrap whole phases: SolverBase.h:35-45, CudaTimer.h).  Enabling
 * resets the accumulators.  kernel: 0 the fused step kernel (hydro) or the
 * flux/emf/update kernel (MHD), 1 the MHD trace kernel, 2 the MHD CFL kernel,
 * 3 the MHD repair kernel (mixed precision, HLLD). */
ek_status ek_solver_set_profiling(ek_solver * s, int enable);
ek_status ek_solver_kernel_time(ek_solver * s, int kernel, double * total_ms, long long * launches);

/* Mixed-precision MHD with the HLLD solver (no counterpart in the reference,
 * whose HLLD is FP64 throughout): a tile of a step in which a face's FP32
 * star-state denominator rho (S - u)(S - u*) - Bn^2 is ill-conditioned (below
 * 2^-14 Bn^2, or at the reference's degenerate-state test) is recomputed by
 * the step's repair kernel with those faces solved in FP64.  tiles: the tiles
 * recomputed since the state was set (0 for the other forms); synchronises
 * the solver's stream. */
ek_status ek_solver_hlld_repairs(ek_solver * s, long long * tiles);

/* VTK output in the reference's own format: save_VTK_2D / save_VTK_3D
 * (IO_VTK.cpp:24-400, non-MPI), reached by save_solution
 * (SolverBase.cpp:210-219 -> IO_ReadWrite.cpp:50-130).  Writes
 * <output_dir>/<output_prefix>_<step, 7 digits>.vti (or
 * ..._<debug_name>_<step>.vti): ImageData cell data of the interior cells in
 * FP64, raw appended binary or ASCII (params->vtk_ascii), variable names
 * rho, energy, rho_vx, rho_vy, rho_vz, bx, by, bz (SolverBase.cpp:60-67).
 * The file is byte for byte the reference's.  ek_write_vtk takes a host state
 * in either layout (CPU only); ek_solver_save_vtk writes the solver's current
 * state.  step is the caller's output counter (the reference's
 * m_times_saved). */
ek_status ek_write_vtk(const ek_params * params, const double * U, int layout, int step,
                       const char * debug_name);
ek_status ek_solver_save_vtk(ek_solver * s, int step, const char * debug_name);

/* Restart files.  The reference restarts from its HDF5 output
 * (init_restart: load_data -> m_times_saved, m_t; SolverHydroMuscl.h:512-580,
 * SolverMHDMuscl.h:611-639); HDF5 is not available here, so the file is raw
 * binary: a header (magic "EKRSTRT1", dim, mhd, nbvar, isize, jsize, ksize,
 * times_saved, iteration, t) and the FP64 LayoutLeft state with its ghosts.
 * Loading restores the state, m_t (0 when reset_time, the reference's
 * restart_reset_totaltime) and the output counter, and starts at
 * m_iteration 0 as the reference does; the grid must match. */
ek_status ek_solver_save_restart(ek_solver * s, const char * path, int times_saved);
ek_status ek_solver_load_restart(ek_solver * s, const char * path, int reset_time, int * times_saved);

/* ---------------------------------------------------------------------------
 * Ensembles of independent Hydro_Muscl_2D runs (no counterpart in the
 * reference, which runs one problem per process): every instance has its own
 * grid size, parameters, boundary conditions and time step.  One step of all
 * instances is one persistent kernel over a flat (instance, tile) work list;
 * ek_ensemble_run can capture the steps in a CUDA graph and replay it.
 * ------------------------------------------------------------------------- */
typedef struct ek_ensemble ek_ensemble;

/* n parameter sets (all 2D hydro, same precision and exact_fp) */
ek_status ek_ensemble_create(const ek_params * params, int n, ek_ensemble ** out);
ek_status ek_ensemble_destroy(ek_ensemble * e);
/* inject the state of instance i (before the first step), as ek_solver_set_state */
ek_status ek_ensemble_set_state(ek_ensemble * e, int i, const double * U, int layout);
ek_status ek_ensemble_get_state(ek_ensemble * e, int i, double * U, int layout);
/* nsteps steps of every instance (instances past their tEnd stay put);
 * use_graph = 1 captures the nsteps launches in one CUDA graph and replays it
 * on later calls with the same nsteps.  Asynchronous: see ek_ensemble_synchronize. */
ek_status ek_ensemble_run(ek_ensemble * e, int nsteps, int use_graph);
ek_status ek_ensemble_synchronize(ek_ensemble * e);
/* m_t, m_dt and m_iteration of instance i */
ek_status ek_ensemble_time(ek_ensemble * e, int i, double * t, double * dt, int * iteration);
ek_status ek_ensemble_dt_history(ek_ensemble * e, int i, double * dts, int n);
/* FP64 totals per instance: out[2i] mass, out[2i+1] total energy */
ek_status ek_ensemble_totals(ek_ensemble * e, double * out);
/* interior cells over all instances, work tiles per step, persistent grid size,
 * kernel launches issued */
ek_status ek_ensemble_info(ek_ensemble * e, long long * interior_cells, int * tiles, int * grid,
                           long long * launches);
ek_status ek_ensemble_stream(ek_ensemble * e, void ** stream);

/* ---------------------------------------------------------------------------
 * One MHD_Muscl_3D FP64 step on caller-owned device arrays that allocates no
 * device memory (no counterpart in the reference).  For callers that own
 * every byte of device memory in their own pool (a Kokkos memory space, an
 * embedding code that budgets the whole HBM) and hand the step only its two
 * state arrays, and for which a cudaMalloc / cudaFree pair per step (each
 * synchronising the device) is not acceptable.  It runs the same kernels as a
 * step of ek_solver_next_iteration.
 *
 * The step's temporary (the 47 x FP64 per-cell compact trace) lives in one
 * static device array of EK_NOALLOC_SCRATCH_BYTES, held by every GPU context
 * that loads this library until the process exits.  The trace takes 384 bytes
 * for each of 32 ceil((nx+2)/32) x (ny+2) x (nz+2) cells; grids whose trace
 * exceeds EK_NOALLOC_SCRATCH_BYTES - 512 (a 50^3 interior is the largest cube)
 * are rejected: EK_ERR_INVALID.
 *
 * U_in, U_out: device pointers, FP64 EK_LAYOUT_LEFT, ghost-inclusive, not
 * overlapping.  The step reads U_in's interior (ghost values follow the
 * boundary conditions by index mapping, so U_in's ghost cells are not read)
 * and writes U_out's interior cells only.  t: time at the start of the step.
 * dt is computed on the device from U_in as the solver's step does (CFL of the
 * state, clamped at tEnd); params->precision must be EK_PREC_FP64,
 * params->exact_fp selects the bitwise-parity build.
 * dt_out: NULL (the call is asynchronous on `stream`) or a host pointer that
 * receives the step's dt (the call then synchronises `stream`;
 * EK_ERR_NONFINITE if dt is not finite and positive).  An asynchronous call
 * cannot report its own non-finite dt: the next call records it on the
 * device and the next call with dt_out returns EK_ERR_NONFINITE for it (that
 * call's own step is still taken).
 * stream: a cudaStream_t, NULL for the default stream.
 *
 * The first call in each device context (that device current) resolves the
 * array's address with cudaGetSymbolAddress: make it before any stream
 * capture.  After cudaDeviceReset the next call resolves it again.
 * Calls on one device share the array, so calls in flight at the same time
 * (other streams, other host threads) race: serialise them (one stream). */
#define EK_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
ek_status ek_mhd3d_step_noalloc(const ek_params * params, const double * U_in, double * U_out, double t,
                                double * dt_out, void * stream);

#ifdef __cplusplus
}
#endif
#endif /* EK_GB300_H */
