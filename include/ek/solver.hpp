/* ek/solver.hpp -- the reference's SolverBase interface over the C ABI,
 * without Kokkos (header only, C++17, host code).
 *
 * ek::Solver has the method set and public state of euler_kokkos'
 * SolverBase (src/shared/SolverBase.h:53-259) with the same sequencing:
 *   compute_dt()            SolverBase.cpp:124-154 (m_dt = compute_dt_local(),
 *                           clamped at m_tEnd)
 *   compute_dt_local()      the solver's CFL time step (SolverHydroMuscl.h:589-631,
 *                           SolverMHDMuscl.h:718-737), on the device
 *   finished()              SolverBase.cpp:170-176
 *   next_iteration()        SolverBase.cpp:180-195: next_iteration_impl(), then
 *                           ++m_iteration, m_t += m_dt
 *   next_iteration_impl()   the step log line every m_nlog steps
 *                           (SolverHydroMuscl.h:646-652), output when due, one
 *                           fused device step; m_dt becomes that step's dt
 *   should_save_solution()  SolverBase.cpp:241-268
 *   save_solution()         save_solution_impl(), then ++m_times_saved
 *   save_solution_impl()    the reference's VTK file (IO_VTK.cpp:24-400)
 *   read_restart_file()     init_restart from a file of save_restart()
 *   make_boundaries()       a no-op: every step maps ghost cells through the
 *                           boundary conditions; get_state() returns them filled
 * Solver names, .ini keys and the conserved-variable layout are the
 * reference's (include/ek_gb300.h).  Errors throw ek::Error (the reference
 * aborts; the C ABI returns a status).  Where the reference keeps stepping on
 * a non-finite dt, so does next_iteration(): the status is kept in
 * last_status(). */
#ifndef EK_SOLVER_HPP
#define EK_SOLVER_HPP

#include <cmath>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../ek_gb300.h"

namespace ek
{

class Error : public std::runtime_error
{
public:
  Error(ek_status s, const std::string & what)
    : std::runtime_error(what + ": " + ek_last_error())
    , status(s)
  {}
  ek_status status;
};

inline void
check(ek_status s, const char * what)
{
  if (s != EK_OK)
    throw Error(s, what);
}

class Solver
{
public:
  // SolverFactory::create(name, params, configMap) with the .ini text
  // (SolverFactory.h:83-116): the solver is the one [run] solver_name names
  explicit Solver(const std::string & ini_text)
  {
    check(ek_params_from_ini(ini_text.data(), ini_text.size(), &params), "ek_params_from_ini");
    create();
  }
  explicit Solver(const ek_params & p)
    : params(p)
  {
    create();
  }
  Solver(const Solver &) = delete;
  Solver & operator=(const Solver &) = delete;
  virtual ~Solver() { ek_solver_destroy(m_s); }

  // the initial condition: init(U) and the constructor tail (boundaries,
  // U2 = U, compute_dt; SolverHydroMuscl.h:276-286, SolverMHDMuscl.h:384-397).
  // U: FP64, ghost cells included, layout EK_LAYOUT_LEFT or EK_LAYOUT_RIGHT.
  void
  set_state(const double * U, int layout = EK_LAYOUT_LEFT)
  {
    check(ek_solver_set_state(m_s, U, layout), "ek_solver_set_state");
    pull_time();
  }
  // the current state with its ghost cells filled (save_solution's copy-out)
  void
  get_state(double * U, int layout = EK_LAYOUT_LEFT) const
  {
    check(ek_solver_get_state(m_s, U, layout), "ek_solver_get_state");
  }
  size_t
  state_size() const
  {
    return (size_t)params.isize * params.jsize * (params.dim == 3 ? params.ksize : 1) * params.nbvar;
  }

  virtual void
  compute_dt()
  {
    m_dt = compute_dt_local();
    if (m_t + m_dt > m_tEnd)
      m_dt = m_tEnd - m_t;
  }
  virtual double
  compute_dt_local()
  {
    double dt = 0.0;
    check(ek_solver_compute_dt(m_s, &dt), "ek_solver_compute_dt");
    return dt;
  }
  virtual int
  finished()
  {
    return m_t >= (m_tEnd - 1e-14) || m_iteration >= params.nStepmax;
  }
  virtual void
  next_iteration()
  {
    next_iteration_impl();
    ++m_iteration;
    m_t += m_dt;
  }
  virtual void
  next_iteration_impl()
  {
    if (m_nlog > 0 && m_iteration % m_nlog == 0 && log)
      std::printf("time step=%7d (dt=% 10.8f t=% 10.8f)\n", m_iteration, m_dt, m_t);
    if (params.nOutput != 0 && should_save_solution())
      save_solution();
    m_status = ek_solver_next_iteration(m_s);
    if (m_status != EK_OK && m_status != EK_ERR_NONFINITE)
      throw Error(m_status, "ek_solver_next_iteration");
    double t, dt;
    int    it;
    check(ek_solver_time(m_s, &t, &dt, &it), "ek_solver_time");
    m_dt = dt; // the step's dt; next_iteration adds it to m_t as the device did
  }
  virtual int
  should_save_solution()
  {
    const double interval = m_tEnd / params.nOutput;
    if (params.nOutput < 0)
      return 1;
    if ((m_t - (m_times_saved - 1) * interval) > interval)
      return 1;
    if (std::fabs(m_t - m_tEnd) < 1e-12) // ISFUZZYNULL (utils.h:20-22)
      return 1;
    return 0;
  }
  virtual void
  save_solution()
  {
    save_solution_impl();
    ++m_times_saved;
  }
  virtual void
  save_solution_impl()
  {
    if (params.vtk_enabled)
      check(ek_solver_save_vtk(m_s, m_times_saved, ""), "ek_solver_save_vtk");
  }
  // init_restart (SolverHydroMuscl.h:512-580) from a file of save_restart
  virtual void
  read_restart_file()
  {
    int saved = 0;
    check(ek_solver_load_restart(m_s, m_restart_run_filename.c_str(), m_restart_reset_totaltime ? 1 : 0, &saved),
          "ek_solver_load_restart");
    m_times_saved = saved;
    pull_time();
  }
  void
  save_restart(const std::string & path)
  {
    check(ek_solver_save_restart(m_s, path.c_str(), m_times_saved), "ek_solver_save_restart");
  }
  // ghost cells are mapped through the boundary conditions in every step
  virtual void
  make_boundaries()
  {}
  virtual void
  init_io()
  {}

  ek_status
  last_status() const
  {
    return m_status;
  }
  ek_solver *
  handle() const
  {
    return m_s;
  }

  ek_params params{};
  double    m_t = 0.0;
  double    m_dt = 0.0;
  int       m_iteration = 0;
  double    m_tEnd = 0.0;
  double    m_cfl = 0.0;
  int       m_nlog = 10;
  long long m_nCells = 0; // ghost cells included, as the reference counts them
  int       m_times_saved = 0;
  std::string m_restart_run_filename;
  bool      m_restart_reset_totaltime = false; // [run] restart_reset_totaltime
  std::map<int, std::string> m_variables_names;
  bool      log = true; // print the step log line

private:
  void
  create()
  {
    check(ek_solver_create(&params, &m_s), "ek_solver_create");
    m_tEnd = params.tEnd;
    m_cfl = params.cfl;
    m_nlog = params.nlog;
    m_t = params.tCurrent;
    m_nCells = (long long)params.isize * params.jsize * (params.dim == 3 ? params.ksize : 1);
    // the output variable names (SolverBase.cpp:60-67, indices of enums.h:17-40)
    const char * names[] = { "rho", "energy", "rho_vx", "rho_vy", "rho_vz", "bx", "by", "bz" };
    for (int v = 0; v < 8; ++v)
      m_variables_names[v] = names[v];
  }
  void
  pull_time()
  {
    double t, dt;
    int    it;
    check(ek_solver_time(m_s, &t, &dt, &it), "ek_solver_time");
    m_t = t;
    m_dt = dt;
    m_iteration = it;
  }

  ek_solver * m_s = nullptr;
  ek_status   m_status = EK_OK;
};

} // namespace ek

#endif /* EK_SOLVER_HPP */
