// ek_main: the reference's driver loop (src/main.cpp:53-159) over the C ABI,
// in C++: ConfigMap + HydroParams from the .ini (ek_params_from_ini), the
// solver from its name (ek_solver_create), the initial state, then
// while (!finished()) next_iteration(), and the final state.
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
  for (long k = 0; k < nsteps; ++k)
  {
    if (ek_solver_finished(s, &finished) != EK_OK)
      return fail("finished");
    if (finished)
      break;
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
  if (p.vtk_enabled && ek_solver_save_vtk(s, 0, "") != EK_OK)
    return fail("save_vtk");
  ek_solver_destroy(s);

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
