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
// k, var.  With [run] nOutput != 0 the solution is saved as main.cpp does
// (first and last state, and whenever should_save_solution() says so; VTK
// files of the reference's format when [output] vtk_enabled).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ek/solver.hpp"

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

  // the reference's loop through the SolverBase-shaped interface (ek/solver.hpp)
  std::vector<double> dts;
  double              t = 0.0, t_io = 0.0, t_tot = 0.0;
  int                 it = 0;
  try
  {
    ek::Solver s(p);
    s.set_state(U.data(), EK_LAYOUT_LEFT);
    if (p.nOutput != 0)
      s.save_solution(); // main.cpp:118-119
    std::printf("Start computation....\n");
    const auto t_start = std::chrono::steady_clock::now();
    for (long k = 0; k < nsteps && !s.finished(); ++k)
    {
      s.next_iteration(); // step log line, one fused step, ++m_iteration, m_t += m_dt
      dts.push_back(s.m_dt);
    }
    s.get_state(U.data(), EK_LAYOUT_LEFT);
    if (p.nOutput != 0)
    {
      // the last state (main.cpp:140-142)
      const auto t_io0 = std::chrono::steady_clock::now();
      s.save_solution();
      t_io = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_io0).count();
    }
    t_tot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    t = s.m_t;
    it = s.m_iteration;

    // main.cpp:150-153 and print_solver_monitoring_info (solver_utils.h:15-55)
    std::printf("final time is %f\n", t);
    const double t_god = t_tot - t_io;
    std::printf("total        time : %5.3f secondes\n", t_tot);
    std::printf("godunov      time : %5.3f secondes %5.2f%%\n", t_god, 100 * t_god / t_tot);
    std::printf("compute dt   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
    std::printf("boundaries   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
    std::printf("comp. prim.  time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
    std::printf("comp. flux   time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
    std::printf("hydro update time : %5.3f secondes %5.2f%%\n", 0.0, 0.0);
    std::printf("io           time : %5.3f secondes %5.2f%%\n", t_io, 100 * t_io / t_tot);
    std::printf("Perf              : %5.3f number of Mcell-updates/s\n", it * (double)s.m_nCells / t_tot * 1e-6);
  }
  catch (const ek::Error & e)
  {
    std::fprintf(stderr, "ek_main: %s\n", e.what());
    return 1;
  }

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
