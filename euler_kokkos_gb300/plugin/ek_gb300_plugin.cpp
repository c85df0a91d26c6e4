// ek_gb300_plugin.cpp -- the reference-side binding: one translation unit
// added to euler_kokkos' own build and linked with -lek_gb300.
//
// SolverFactory::registerSolver exists to "register a callback from a plugin
// code, at runtime" (SolverFactory.h:64-75).  This file registers, under the
// reference's own names (SolverFactory.cpp:18-22), solvers that derive from
// the reference's SolverHydroMuscl<dim> / SolverMHDMuscl<dim> and route the
// time step to libek_gb300.  The reference's initial conditions, output
// writers, restart reader and main.cpp stay unchanged:
//   * construction: the base class runs the reference's init (and
//     init_restart); the library solver is created with the same parameters
//     (ek_solver_create, the HydroParams fields, ConfigMap's [gb300] keys);
//   * the state goes to the device at the first compute_dt_local() or
//     next_iteration_impl() after construction, so a caller that rewrites U
//     after the constructor (an injected initial state) is honoured;
//   * next_iteration_impl(): the reference's log line and output schedule,
//     then one fused device step; m_dt becomes that step's dt and
//     SolverBase::next_iteration adds it to m_t, the same FP64 addition the
//     device does;
//   * save_solution_impl(): the device state is copied back into U / U2,
//     then the reference's own writers run.
// Errors of the library abort with its message, as the reference aborts on
// its own fatal errors (SolverFactory.h:105-113).
//
// Build (reference tree R, this repository E): compile this file with the
// reference's include paths and -I E/include, link with
// -L E/euler_kokkos_gb300/_build -lek_gb300.  oracle/Makefile.ref (target
// `plugin`) builds the reference's own main.cpp with it against the
// repository's Kokkos-API shim; tests/test_plugin.py runs that build.
#include "ek_gb300.h"
#include "muscl/SolverHydroMuscl.h"
#include "muscl/SolverMHDMuscl.h"
#include "shared/SolverFactory.h"

#include <cstdio>
#include <cstdlib>
#include <type_traits>

namespace euler_kokkos
{

namespace
{

ek_params
to_ek_params(const HydroParams & hp, int mhd)
{
  ek_params p = {};
  p.dim = hp.dimType == THREE_D ? 3 : 2;
  p.mhd = mhd;
  p.nx = hp.nx;
  p.ny = hp.ny;
  p.nz = hp.nz;
  p.ghost_width = hp.ghostWidth;
  p.nbvar = hp.nbvar;
  p.isize = hp.isize;
  p.jsize = hp.jsize;
  p.ksize = hp.ksize;
  p.xmin = hp.xmin;
  p.xmax = hp.xmax;
  p.ymin = hp.ymin;
  p.ymax = hp.ymax;
  p.zmin = hp.zmin;
  p.zmax = hp.zmax;
  p.dx = hp.dx;
  p.dy = hp.dy;
  p.dz = hp.dz;
  // BC_DIRICHLET = 1 (reflecting), BC_NEUMANN = 2 (outflow), BC_PERIODIC = 3
  const BoundaryConditionType bc[6] = { hp.boundary_type_xmin, hp.boundary_type_xmax, hp.boundary_type_ymin,
                                        hp.boundary_type_ymax, hp.boundary_type_zmin, hp.boundary_type_zmax };
  for (int f = 0; f < 6; ++f)
    p.bc[f] = (int)bc[f];
  const HydroSettings & s = hp.settings;
  p.gamma0 = s.gamma0;
  p.gamma6 = s.gamma6;
  p.cfl = s.cfl;
  p.slope_type = s.slope_type;
  p.smallr = s.smallr;
  p.smallc = s.smallc;
  p.smallp = s.smallp;
  p.smallpp = s.smallpp;
  p.cIso = s.cIso;
  p.Omega0 = s.Omega0;
  p.riemann = (int)hp.riemannSolverType;
  p.implementation_version = hp.implementationVersion;
  p.nStepmax = hp.nStepmax;
  p.tEnd = hp.tEnd;
  p.nOutput = hp.nOutput;
  p.nlog = hp.nlog;
  p.precision = EK_PREC_FP64;
  return p;
}

void
check(ek_status st)
{
  if (st != EK_OK)
  {
    std::fprintf(stderr, "libek_gb300: %s\n", ek_last_error());
    std::abort();
  }
}

} // namespace

// Base = muscl::SolverHydroMuscl<dim> or muscl::SolverMHDMuscl<dim>
template <class Base, int MHD>
class SolverGB300 : public Base
{
public:
  SolverGB300(HydroParams & hp, ConfigMap & cm)
    : Base(hp, cm)
  {
    ek_params p = to_ek_params(hp, MHD);
    p.tCurrent = this->m_t; // 0, or the time init_restart read
    p.exact_fp = cm.getInteger("gb300", "exact", 0);
    p.precision = cm.getString("gb300", "precision", "fp64") == "mixed" ? EK_PREC_MIXED : EK_PREC_FP64;
    p.gravity_enabled = this->m_gravity.enabled; // GravityParams (SolverBase.cpp:38-39)
    p.gravity_hancock = this->m_gravity.hancock_predictor_enabled;
    check(ek_solver_create(&p, &m_s));
  }
  ~SolverGB300() override { ek_solver_destroy(m_s); }

  static SolverBase *
  create(HydroParams & hp, ConfigMap & cm)
  {
    return new SolverGB300(hp, cm);
  }

  double
  compute_dt_local() override
  {
    upload();
    double dt = 0.0;
    check(ek_solver_compute_dt(m_s, &dt));
    return dt;
  }

  // SolverBase::next_iteration calls this, then ++m_iteration, m_t += m_dt
  void
  next_iteration_impl() override
  {
    upload();
    if (this->m_iteration % this->m_nlog == 0)
      std::printf("time step=%7d (dt=% 10.8f t=% 10.8f)\n", this->m_iteration, this->m_dt, this->m_t);
    if (this->params.enableOutput && this->should_save_solution())
      this->save_solution();
    const ek_status st = ek_solver_next_iteration(m_s);
    if (st != EK_ERR_NONFINITE) // the reference keeps stepping on a non-finite dt
      check(st);
    double t, dt;
    int    it;
    check(ek_solver_time(m_s, &t, &dt, &it));
    this->m_dt = dt;
  }

  void
  save_solution_impl() override
  {
    if (m_uploaded)
    {
      // the device state into U or U2 (the current one by iteration parity),
      // then the reference's writers
      check(ek_solver_get_state(m_s, this->Uhost.data(), layout()));
      Kokkos::deep_copy(this->m_iteration % 2 == 0 ? this->U : this->U2, this->Uhost);
    }
    Base::save_solution_impl();
  }

private:
  // the current state (U, as the constructor or the caller left it) to the
  // device: set_state runs the constructor tail there (boundaries, dt)
  void
  upload()
  {
    if (m_uploaded)
      return;
    Kokkos::deep_copy(this->Uhost, this->U);
    check(ek_solver_set_state(m_s, this->Uhost.data(), layout()));
    if constexpr (!MHD)
    {
      if (this->m_gravity.enabled)
      {
        // the static field the reference's init wrote (SolverHydroMuscl.h:86-87)
        auto g = Kokkos::create_mirror(this->gravity_field);
        Kokkos::deep_copy(g, this->gravity_field);
        check(ek_solver_set_gravity_field(m_s, g.data(), layout()));
      }
    }
    m_uploaded = true;
  }
  static int
  layout()
  {
    using L = typename std::remove_reference<decltype(std::declval<Base &>().U)>::type::array_layout;
    return std::is_same<L, Kokkos::LayoutLeft>::value ? EK_LAYOUT_LEFT : EK_LAYOUT_RIGHT;
  }

  ek_solver * m_s = nullptr;
  bool        m_uploaded = false;
};

// replaces the built-in entries (SolverFactory.cpp:18-22) before main()
// creates its solver
static const bool ek_gb300_registered = [] {
  SolverFactory & f = SolverFactory::Instance();
  f.registerSolver("Hydro_Muscl_2D", &SolverGB300<muscl::SolverHydroMuscl<2>, 0>::create);
  f.registerSolver("Hydro_Muscl_3D", &SolverGB300<muscl::SolverHydroMuscl<3>, 0>::create);
  f.registerSolver("MHD_Muscl_2D", &SolverGB300<muscl::SolverMHDMuscl<2>, 1>::create);
  f.registerSolver("MHD_Muscl_3D", &SolverGB300<muscl::SolverMHDMuscl<3>, 1>::create);
  return true;
}();

} // namespace euler_kokkos
