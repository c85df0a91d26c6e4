/*
 * ek_oracle.h -- CPU restatement of the euler_kokkos unsplit MUSCL-Hancock
 * step (hydro 2D/3D, constrained-transport MHD 3D) in plain C.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it to check or time
 * the reference algorithm.  The product (the CUDA library) never links it.
 *
 * It restates the reference's implementationVersion=0 kernel sequence
 * (SolverHydroMuscl.cpp:304-390, SolverMHDMuscl.cpp:461-568) in the same
 * floating-point expression order, so that a build with
 * -ffp-contract=off reproduces the reference bit for bit.  It is pinned
 * against the reference's own sources compiled with a Kokkos-API shim
 * (oracle/_ref, tests/golden).
 *
 * State layout: U[((var*ksize + k)*jsize + j)*isize + i] (i fastest, the
 * variable index slowest), ghost cells included; the reference's
 * Kokkos::LayoutLeft device layout (kokkos_shared.h:24-42).
 */
#ifndef EK_ORACLE_H
#define EK_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* variable indexes, enums.h:17-40 */
enum { EKO_ID = 0, EKO_IP = 1, EKO_IU = 2, EKO_IV = 3, EKO_IW = 4, EKO_IA = 5, EKO_IB = 6, EKO_IC = 7 };
/* boundary types, enums.h:185-192 */
enum { EKO_BC_DIRICHLET = 1, EKO_BC_NEUMANN = 2, EKO_BC_PERIODIC = 3 };
/* riemann solver types, enums.h:175-182 */
enum { EKO_RIEMANN_APPROX = 0, EKO_RIEMANN_LLF = 1, EKO_RIEMANN_HLL = 2, EKO_RIEMANN_HLLC = 3, EKO_RIEMANN_HLLD = 4 };

typedef struct eko_params
{
  int    dim;  /* 2 or 3 */
  int    mhd;  /* 0 hydro, 1 MHD */
  int    nx, ny, nz;
  int    gw;    /* ghost width: 2 hydro, 3 MHD (HydroParams.cpp:95-116) */
  int    nbvar; /* 4, 5 or 8 */
  int    isize, jsize, ksize;
  double xmin, ymin, zmin, dx, dy, dz;
  int    bc[6]; /* xmin, xmax, ymin, ymax, zmin, zmax */
  double gamma0, cfl, slope_type, smallr, smallc, smallp, smallpp, cIso, Omega0;
  int    riemann;
  double tEnd;
  int    nStepmax;
  double gamma6; /* (gamma0 + 1) / (2 gamma0), HydroParams.cpp:356 */
  /* static gravity (hydro only; GravityParams.h:22-37) */
  int    grav_enabled;  /* [gravity] enabled */
  int    grav_hancock;  /* [gravity] hancock_predictor_enabled */
  double gravity[3];    /* uniform field of the Rayleigh-Taylor init
                           (HydroInitFunctors2D.h:735-771, HydroInitFunctors3D.h:806-842);
                           0 for other problems (a zero-initialised VectorField) */
} eko_params;

typedef struct eko_solver eko_solver;

/* Create a solver on an injected initial state U0 (full array, layout above)
 * and replay the reference constructor tail: make_boundaries(U),
 * deep_copy(U2,U), [MHD: convertToPrimitives(U)], compute_dt()
 * (SolverHydroMuscl.h:276-286, SolverMHDMuscl.h:384-397).  t0 is m_t. */
eko_solver * eko_create(const eko_params * p, const double * U0, double t0);
void         eko_destroy(eko_solver * s);
/* SolverBase::next_iteration (SolverBase.cpp:180-195); returns 0 on success */
int          eko_next_iteration(eko_solver * s);
/* Replace the gravity field (dim components over the full grid, layout
 * G[((comp*ksize + k)*jsize + j)*isize + i]) and recompute m_dt as the
 * constructor does; returns -1 when gravity is not enabled. */
int          eko_set_gravity_field(eko_solver * s, const double * G);
int          eko_finished(const eko_solver * s);
void         eko_get_state(const eko_solver * s, double * U);
double       eko_time(const eko_solver * s);
double       eko_dt(const eko_solver * s);
int          eko_iteration(const eko_solver * s);
long         eko_ncells(const eko_params * p);

/* number of OpenMP threads the oracle uses (1 when built without OpenMP) */
int eko_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
