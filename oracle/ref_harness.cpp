// Reference harness (test infrastructure only).
//
// Drives the reference's OWN solver classes, compiled from the reference
// sources against the Kokkos-API shim in oracle/kokkos_shim, exactly the way
// the reference's src/main.cpp:53-159 does (ConfigMap -> HydroParams ->
// SolverFactory::create -> while(!finished()) next_iteration()), with two
// additions needed for parity testing:
//   * an optional injected initial state U0 (overwrites solver->U after the
//     constructor, then replays the constructor tail: make_boundaries(U),
//     deep_copy(U2,U), [MHD: convertToPrimitives(U)], compute_dt();
//     SolverHydroMuscl.h:276-286, SolverMHDMuscl.h:384-397),
//   * a dump of the final state and of the dt sequence in the EKST format.
//
// usage: ref_run <file.ini> <nsteps> <out.ekst> [<U0.ekst>]
// (environment: EK_REF_SAVE, EK_REF_GRAVITY, EK_REF_DUMP0 -- see run())
//
// EKST format (little endian): char magic[8]="EKSTATE1"; int64 dim, nbvar,
// isize, jsize, ksize, ghost, iteration, ndt; double t; double dt[ndt];
// double U[isize*jsize*ksize*nbvar] with i fastest, then j, k, var.

#include "shared/HydroParams.h"
#include "shared/SolverBase.h"
#include "shared/SolverFactory.h"
#include "muscl/SolverHydroMuscl.h"
#include "muscl/SolverMHDMuscl.h"
#include "utils/config/ConfigMap.h"
#include "utils/mpi/ParallelEnv.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace ekh
{
using namespace euler_kokkos;

struct EkHeader
{
  char    magic[8];
  int64_t dim, nbvar, isize, jsize, ksize, ghost, iteration, ndt;
  double  t;
};

template <class View>
static void
copy_in(View & v, const std::vector<double> & buf, int dim, int nb, int is, int js, int ks)
{
  for (int var = 0; var < nb; ++var)
    for (int k = 0; k < ks; ++k)
      for (int j = 0; j < js; ++j)
        for (int i = 0; i < is; ++i)
        {
          double x = buf[(size_t)i + (size_t)is * (j + (size_t)js * (k + (size_t)ks * var))];
          if constexpr (View::rank == 3)
            v(i, j, var) = x;
          else
            v(i, j, k, var) = x;
        }
  (void)dim;
}

template <class View>
static void
copy_out(const View & v, std::vector<double> & buf, int nb, int is, int js, int ks)
{
  buf.assign((size_t)is * js * ks * nb, 0.0);
  for (int var = 0; var < nb; ++var)
    for (int k = 0; k < ks; ++k)
      for (int j = 0; j < js; ++j)
        for (int i = 0; i < is; ++i)
        {
          double x;
          if constexpr (View::rank == 3)
            x = v(i, j, var);
          else
            x = v(i, j, k, var);
          buf[(size_t)i + (size_t)is * (j + (size_t)js * (k + (size_t)ks * var))] = x;
        }
}

// one EKST file: header, dt sequence, state (copy_out layout)
static int
write_ekst(const char * path, int dim, int nb, int is, int js, int ks, int ghost, int iteration, double t,
           const std::vector<double> & dts, const std::vector<double> & buf)
{
  FILE * f = std::fopen(path, "wb");
  if (!f)
    return 3;
  EkHeader h{};
  std::memcpy(h.magic, "EKSTATE1", 8);
  h.dim = dim;
  h.nbvar = nb;
  h.isize = is;
  h.jsize = js;
  h.ksize = ks;
  h.ghost = ghost;
  h.iteration = iteration;
  h.ndt = (int64_t)dts.size();
  h.t = t;
  std::fwrite(&h, sizeof h, 1, f);
  if (!dts.empty())
    std::fwrite(dts.data(), sizeof(double), dts.size(), f);
  std::fwrite(buf.data(), sizeof(double), buf.size(), f);
  std::fclose(f);
  return 0;
}

template <class Solver>
static int
run(Solver * s, euler_kokkos::HydroParams & p, int nsteps, const char * out, const char * in, bool mhd)
{
  const int dim = p.dimType == TWO_D ? 2 : 3;
  const int is = p.isize, js = p.jsize, ks = dim == 2 ? 1 : p.ksize, nb = p.nbvar;
  if (in)
  {
    FILE * f = std::fopen(in, "rb");
    if (!f)
    {
      std::fprintf(stderr, "cannot open %s\n", in);
      return 2;
    }
    EkHeader h;
    if (std::fread(&h, sizeof h, 1, f) != 1 || h.isize != is || h.jsize != js || h.ksize != ks ||
        h.nbvar != nb)
    {
      std::fprintf(stderr, "bad initial state header in %s\n", in);
      return 2;
    }
    std::vector<double> dts(h.ndt);
    if (h.ndt && std::fread(dts.data(), sizeof(double), h.ndt, f) != (size_t)h.ndt)
      return 2;
    std::vector<double> buf((size_t)is * js * ks * nb);
    if (std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size())
      return 2;
    std::fclose(f);
    copy_in(s->U, buf, dim, nb, is, js, ks);
    // EK_REF_GRAVITY=<file.ekst> (nbvar = dim): replaces the static gravity
    // field the constructor's init left (SolverHydroMuscl.h:86-87, 228-231)
    if constexpr (std::is_same<Solver, muscl::SolverHydroMuscl<2>>::value ||
                  std::is_same<Solver, muscl::SolverHydroMuscl<3>>::value)
    {
      const char * gpath = std::getenv("EK_REF_GRAVITY");
      if (gpath && gpath[0])
      {
        FILE * g = std::fopen(gpath, "rb");
        EkHeader gh;
        if (!g || std::fread(&gh, sizeof gh, 1, g) != 1 || gh.nbvar != dim || gh.isize != is ||
            gh.jsize != js || gh.ksize != ks || s->gravity_field.size() == 0)
        {
          std::fprintf(stderr, "bad gravity field %s\n", gpath);
          return 2;
        }
        std::fseek(g, (long)(sizeof gh + sizeof(double) * gh.ndt), SEEK_SET);
        std::vector<double> gbuf((size_t)is * js * ks * dim);
        if (std::fread(gbuf.data(), sizeof(double), gbuf.size(), g) != gbuf.size())
          return 2;
        std::fclose(g);
        copy_in(s->gravity_field, gbuf, dim, dim, is, js, ks);
      }
    }
    // replay the constructor tail on the injected state
    s->make_boundaries(s->U);
    Kokkos::deep_copy(s->U2, s->U);
    if constexpr (std::is_same<Solver, muscl::SolverMHDMuscl<2>>::value ||
                  std::is_same<Solver, muscl::SolverMHDMuscl<3>>::value)
      s->convertToPrimitives(s->U);
    s->compute_dt();
  }
  (void)mhd;
  // EK_REF_DUMP0=<file>: the state the run starts from (the reference's own
  // init when no state is injected)
  const char * dump0 = std::getenv("EK_REF_DUMP0");
  if (dump0 && dump0[0])
  {
    std::vector<double> b0;
    copy_out(s->U, b0, nb, is, js, ks);
    if (write_ekst(dump0, dim, nb, is, js, ks, p.ghostWidth, s->m_iteration, s->m_t, {}, b0) != 0)
      return 3;
  }
  std::vector<double> dts;
  for (int n = 0; n < nsteps && !s->finished(); ++n)
  {
    s->next_iteration();
    dts.push_back(s->m_dt);
  }
  // EK_REF_SAVE set: write the final state with the reference's own output
  // path (save_solution -> IO_ReadWrite -> save_VTK_2D/3D, as configured by
  // the [output] section of the .ini)
  if (std::getenv("EK_REF_SAVE"))
    s->save_solution();
  std::vector<double> buf;
  if (s->m_iteration % 2 == 0)
    copy_out(s->U, buf, nb, is, js, ks);
  else
    copy_out(s->U2, buf, nb, is, js, ks);
  return write_ekst(out, dim, nb, is, js, ks, p.ghostWidth, s->m_iteration, s->m_t, dts, buf);
}

int
harness_main(int argc, char * argv[])
{
  if (argc < 4)
  {
    std::fprintf(stderr, "usage: %s <file.ini> <nsteps> <out.ekst> [<U0.ekst>]\n", argv[0]);
    return 1;
  }
  int            pargc = 1;
  char **        pargv = argv;
  ParallelEnv    par_env(pargc, pargv);
  euler_kokkos::ConfigMap configMap(argv[1]);
  euler_kokkos::HydroParams params(configMap, par_env);
  std::string    name = configMap.getString("run", "solver_name", "unknown");
  SolverBase *   base = SolverFactory::Instance().create(name, params, configMap);
  const int      nsteps = std::atoi(argv[2]);
  const char *   in = argc > 4 ? argv[4] : nullptr;
  int            rc = 1;
  if (name == "Hydro_Muscl_2D")
    rc = run(dynamic_cast<muscl::SolverHydroMuscl<2> *>(base), params, nsteps, argv[3], in, false);
  else if (name == "Hydro_Muscl_3D")
    rc = run(dynamic_cast<muscl::SolverHydroMuscl<3> *>(base), params, nsteps, argv[3], in, false);
  else if (name == "MHD_Muscl_2D")
    rc = run(dynamic_cast<muscl::SolverMHDMuscl<2> *>(base), params, nsteps, argv[3], in, true);
  else if (name == "MHD_Muscl_3D")
    rc = run(dynamic_cast<muscl::SolverMHDMuscl<3> *>(base), params, nsteps, argv[3], in, true);
  delete base;
  return rc;
}

} // namespace ekh

int
main(int argc, char * argv[])
{
  return ekh::harness_main(argc, argv);
}
