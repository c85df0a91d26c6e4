// ek_main: the reference's driver loop (src/main.cpp:53-159) over the C ABI,
// in C++, with an injected initial state (the reference's init functors are
// not part of this library): ConfigMap + HydroParams from the .ini
// (ek_params_from_ini), the solver from its name (ek_solver_create), the
// initial state, then while (!finished()) next_iteration(), and the final
// state.  It prints the reference's lines on stdout: "Start computation....",
// the step log every nlog steps (SolverHydroMuscl.h:646-652,
// SolverMHDMuscl.h:752-758), "final time is" (main.cpp:150-151) and the timer
// summary with the Perf line (solver_utils.h:15-55, ghost cells counted as in
// SolverHydroMuscl.h:182).  The step is one fused GPU pass, so the
// reference's per-phase timers (compute dt, boundaries, primitives, fluxes,
// update) are inside "godunov" and print 0.
//
// usage: ek_main <file.ini> <nsteps> <out.ekst> <U0.ekst>
//   nsteps  at most this many steps (the .ini's nStepmax and tEnd also stop
//           the run, as in the reference)
//   U0      the initial state: the caller's init(U), the full FP64 LayoutLeft
//           array with ghost cells
// State files use the EKST layout (little endian): char magic[8]="EKSTATE1";
// int64 dim, nbvar, isize, jsize, ksize, ghost, iteration, ndt; double t;
// double dt[ndt]; double U[isize*jsize*ksize*nbvar] with i fastest, then j,
// k, var.  With [output] vtk_enabled the final state is also written as the
// reference's VTK file (save_solution).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ek_gb300.h"

namespace
{

struct EkstHeader
{
  char    magic[8];
  int64_t dim, nbvar, isize, jsize, ksize, ghost, iteration, ndt;
  double  t;
};

int
fail(const char * what)
{
  std::fprintf(stderr, "ek_main: %s: %s\n", what, ek_last_error());
  return 1;
}

bool
read_file(const char * path, std::string & out)
{
  FILE * f = std::fopen(path, "rb");
  if (!f)
    return false;
  char   buf[65536];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0)
    out.append(buf, n);
  std::fclose(f);
  return true;
}

} // namespace

int
main(int argc, char ** argv)
{
  if (argc != 5)
  {
    std::fprintf(stderr, "usage: %s <file.ini> <nsteps> <out.ekst> <U0.ekst>\n", argv[0]);
    return 2;
  }
  std::string ini;
  if (!read_file(argv[1], ini))
  {
    std::fprintf(stderr, "ek_main: cannot read %s\n", argv[1]);
    return 2;
  }
  const long nsteps = std::strtol(argv[2], nullptr, 10);

  ek_params p;
  if (ek_params_from_ini(ini.data(), ini.size(), &p) != EK_OK)
    return fail("parameters");
  const int64_t ks = p.dim == 3 ? p.ksize : 1;
  const size_t  n = (size_t)p.isize * p.jsize * ks * p.nbvar;

  // initial state
  std::vector<double> U(n);
  {
    FILE *     f = std::fopen(argv[4], "rb");
    EkstHeader h;
    if (!f || std::fread(&h, sizeof h, 1, f) != 1 || std::memcmp(h.magic, "EKSTATE1", 8) != 0 ||
        h.nbvar != p.nbvar || h.isize != p.isize || h.jsize != p.jsize || h.ksize != ks)
    {
      std::fprintf(stderr, "ek_main: %s is not a state of this grid\n", argv[4]);
      return 2;
    }
    std::fseek(f, (long)(sizeof h + sizeof(double) * h.ndt), SEEK_SET);
    const bool ok = std::fread(U.data(), sizeof(double), n, f) == n;
    std::fclose(f);
    if (!ok)
    {
      std::fprintf(stderr, "ek_main: short state file %s\n", argv[4]);
      return 2;
    }
  }

  ek_solver * s = nullptr;
  if (ek_solver_create(&p, &s) != EK_OK)
    return fail("solver");
  if (ek_solver_set_state(s, U.data(), EK_LAYOUT_LEFT) != EK_OK)
    return fail("set_state");

  std::vector<double> dts;
  int                 finished = 0;
  const int           nlog = p.nlog > 0 ? p.nlog : 1;
  std::printf("Start computation....\n");
  const auto t_start = std::chrono::steady_clock::now();
  double     t_io = 0.0;
  for (long k = 0; k < nsteps; ++k)
  {
    if (ek_solver_finished(s, &finished) != EK_OK)
      return fail("finished");
    if (finished)
      break;
    {
      // next_iteration_impl's log line: iteration, dt and t before the step
      double t0, dt0;
      int    it0;
      if (ek_solver_time(s, &t0, &dt0, &it0) != EK_OK)
        return fail("time");
      if (it0 % nlog == 0)
        std::printf("time step=%7d (dt=% 10.8f t=% 10.8f)\n", it0, dt0, t0);
    }
    const ek_status st = ek_solver_next_iteration(s);
    double          t, dt;
    int             it;
    ek_solver_time(s, &t, &dt, &it);
    dts.push_back(dt);
    if (st == EK_ERR_NONFINITE)
      continue; // the reference keeps stepping on a non-finite dt
    if (st != EK_OK)
      return fail("next_iteration");
  }

  double t, dt;
  int    it;
  if (ek_solver_time(s, &t, &dt, &it) != EK_OK || ek_solver_get_state(s, U.data(), EK_LAYOUT_LEFT) != EK_OK)
    return fail("final state");
  if (p.vtk_enabled)
  {
    const auto t_io0 = std::chrono::steady_clock::now();
    if (ek_solver_save_vtk(s, 0, "") != EK_OK)
      return fail("save_vtk");
    t_io = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_io0).count();
  }
  ek_solver_destroy(s);
  const double t_tot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();

  // main.cpp:150-153 and print_solver_monitoring_info (solver_utils.h:15-55)
  std::printf("final time is %f\n", t);
  const double t_god = t_tot - t_io;
  const double ncells = (double)p.isize * p.jsize * (p.dim == 3 ? p.ksize : 1);
  std::printf("total        time : %5.3f secondes\n", t_tot);
  std::printf("godunov      time : %5.3f secondes %5.2f%%\n", t_god, 100 * t_god / t_tot);
  std::printf("compute dt   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
  std::printf("boundaries   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
  std::printf("comp. prim.  time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
  std::printf("comp. flux   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
  std::printf("hydro update time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
  std::printf("io           time : %5.3f secondes %5.2f%%\n", t_io, 100 * t_io / t_tot);
  std::printf("Perf              : %5.3f number of Mcell-updates/s\n", it * ncells / t_tot * 1e-6);

  FILE * f = std::fopen(argv[3], "wb");
  if (!f)
  {
    std::fprintf(stderr, "ek_main: cannot write %s\n", argv[3]);
    return 3;
  }
  EkstHeader h;
  std::memset(&h, 0, sizeof h);
  std::memcpy(h.magic, "EKSTATE1", 8);
  h.dim = p.dim, h.nbvar = p.nbvar, h.isize = p.isize, h.jsize = p.jsize, h.ksize = ks;
  h.ghost = p.ghost_width, h.iteration = it, h.ndt = (int64_t)dts.size(), h.t = t;
  bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
  ok = ok && (dts.empty() || std::fwrite(dts.data(), sizeof(double), dts.size(), f) == dts.size());
  ok = ok && std::fwrite(U.data(), sizeof(double), n, f) == n;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? 0 : 3;
}
