/*
 * ek_oracle.c -- CPU restatement of the euler_kokkos MUSCL-Hancock step.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle and timed CPU baseline); the CUDA
 * product never links it.  Every function names the reference file:line it
 * restates.  Expressions keep the reference's evaluation order; build with
 * -ffp-contract=off for bitwise parity with the reference.
 */
#include "ek_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define HALF 0.5
#define ONE 1.0
#define ZERO 0.0

int
eko_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

struct eko_solver
{
  eko_params p;
  double *   U;  /* ping */
  double *   U2; /* pong */
  double *   Q;
  /* hydro v0 work arrays */
  double * Fx;
  double * Fy;
  double * Fz;
  double * Sx; /* slopes */
  double * Sy;
  double * Sz;
  /* MHD v0 work arrays */
  double * E;      /* 3 components, edge electric field */
  double * dA;     /* DeltaA/B/C: 3 components each */
  double * dB;
  double * dC;
  double * Qm[3];  /* face traces */
  double * Qp[3];
  double * QE[4][3]; /* edge traces [RT,RB,LT,LB][x,y,z] */
  double * Emf;    /* 3 components: I_EMFZ=0, I_EMFY=1, I_EMFX=2 (enums.h:215-220) */
  double * G;      /* static gravity field, dim components (SolverHydroMuscl.h:86-87) */
  double   t, dt;
  int      iteration;
  long     ncell;
};

/* index helpers (LayoutLeft, kokkos_shared.h:24-42) */
#define IDX(s, i, j, k) ((long)(i) + (long)(s)->p.isize * ((long)(j) + (long)(s)->p.jsize * (long)(k)))
#define AT(a, s, var, c) ((a)[(long)(var) * (s)->ncell + (c)])

long
eko_ncells(const eko_params * p)
{
  return (long)p->isize * p->jsize * (p->dim == 3 ? p->ksize : 1);
}

/* ===================================================================== */
/* boundaries: BoundariesFunctors.h:17-531 (hydro), :534-1057 (MHD);       */
/* applied face by face in the order of SolverBase.cpp:488-512            */
/* ===================================================================== */
static void
fill_face(eko_solver * s, double * U, int face)
{
  const eko_params * p = &s->p;
  const int gw = p->gw, nb = p->nbvar, mhd = p->mhd;
  const int ks = p->dim == 3 ? p->ksize : 1;
  const int dir = face / 2, hi = face % 2;
  const int n = dir == 0 ? p->nx : (dir == 1 ? p->ny : p->nz);
  const int bt = p->bc[face];
  /* normal velocity / normal field component flipped by a reflecting wall */
  const int iv_n = EKO_IU + dir;
  const int ib_n = EKO_IA + dir;
  const int ni = dir == 0 ? gw : p->isize;
  const int nj = dir == 1 ? gw : p->jsize;
  const int nk = dir == 2 ? gw : ks;
#pragma omp parallel for collapse(2) schedule(static)
  for (int kk = 0; kk < nk; ++kk)
    for (int jj = 0; jj < nj; ++jj)
      for (int ii = 0; ii < ni; ++ii)
      {
        int g[3] = { ii, jj, kk };
        int x = g[dir]; /* 0..gw-1 */
        int ghost = hi ? x + n + gw : x;
        int src;
        if (bt == EKO_BC_DIRICHLET)
          src = hi ? 2 * n + 2 * gw - 1 - ghost : 2 * gw - 1 - ghost;
        else if (bt == EKO_BC_NEUMANN)
          src = hi ? n + gw - 1 : gw;
        else
          src = hi ? ghost - n : n + ghost;
        int gi[3] = { ii, jj, kk }, si[3] = { ii, jj, kk };
        gi[dir] = ghost;
        si[dir] = src;
        long cg = IDX(s, gi[0], gi[1], gi[2]);
        long cs = IDX(s, si[0], si[1], si[2]);
        for (int var = 0; var < nb; ++var)
        {
          double sign = 1.0;
          if (bt == EKO_BC_DIRICHLET && (var == iv_n || (mhd && var == ib_n)))
            sign = -1.0;
          AT(U, s, var, cg) = AT(U, s, var, cs) * sign;
        }
      }
}

static void
make_boundaries(eko_solver * s, double * U)
{
  const int nf = s->p.dim == 3 ? 6 : 4;
  for (int f = 0; f < nf; ++f)
    fill_face(s, U, f);
}

/* ===================================================================== */
/* shared scalar pieces                                                   */
/* ===================================================================== */

/* slope_unsplit_hydro_{2d,3d}_scalar, one direction:
 * HydroBaseFunctor2D.h:423-453, HydroBaseFunctor3D.h:413-462,
 * MHDBaseFunctor3D.h:264-320 */
static inline double
slope1(double q, double qp, double qm, double st)
{
  double dlft = st * (q - qm);
  double drgt = st * (qp - q);
  double dcen = HALF * (qp - qm);
  double dsgn = (dcen >= ZERO) ? ONE : -ONE;
  double slop = fmin(fabs(dlft), fabs(drgt));
  double dlim = slop;
  if ((dlft * drgt) <= ZERO)
    dlim = ZERO;
  return dsgn * fmin(dlim, fabs(dcen));
}

/* cmpflx: RiemannSolvers.h:20-53 (nt transverse velocities) */
static void
cmpflx(const double * qg, double * flux, int nt, const eko_params * p)
{
  flux[EKO_ID] = qg[EKO_ID] * qg[EKO_IU];
  flux[EKO_IU] = flux[EKO_ID] * qg[EKO_IU] + qg[EKO_IP];
  flux[EKO_IV] = flux[EKO_ID] * qg[EKO_IV];
  if (nt == 2)
    flux[EKO_IW] = flux[EKO_ID] * qg[EKO_IW];
  double entho = ONE / (p->gamma0 - ONE);
  double ekin = HALF * qg[EKO_ID] * (qg[EKO_IU] * qg[EKO_IU] + qg[EKO_IV] * qg[EKO_IV]);
  if (nt == 2)
    ekin += HALF * qg[EKO_ID] * (qg[EKO_IW] * qg[EKO_IW]);
  double etot = qg[EKO_IP] * entho + ekin;
  flux[EKO_IP] = qg[EKO_IU] * (etot + qg[EKO_IP]);
}

/* riemann_approx: RiemannSolvers.h:60-200 (10 Newton iterations at most) */
static void
riemann_approx(const double * ql, const double * qr, double * flux, int nt, const eko_params * p)
{
  const double gamma0 = p->gamma0, gamma6 = p->gamma6, smallr = p->smallr, smallc = p->smallc,
               smallp = p->smallp, smallpp = p->smallpp;
  double rl = fmax(ql[EKO_ID], smallr), ul = ql[EKO_IU], pl = fmax(ql[EKO_IP], rl * smallp);
  double rr = fmax(qr[EKO_ID], smallr), ur = qr[EKO_IU], pr = fmax(qr[EKO_IP], rr * smallp);
  double cl = gamma0 * pl * rl;
  double cr = gamma0 * pr * rr;
  double wl = sqrt(cl);
  double wr = sqrt(cr);
  double pstar = fmax(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), (double)ZERO);
  double pold = pstar;
  double conv = ONE;
  for (int iter = 0; (iter < 10) && (conv > 1e-6); ++iter)
  {
    double wwl = sqrt(cl * (ONE + gamma6 * (pold - pl) / pl));
    double wwr = sqrt(cr * (ONE + gamma6 * (pold - pr) / pr));
    double qql = 2.0 * wwl * wwl * wwl / (wwl * wwl + cl);
    double qqr = 2.0 * wwr * wwr * wwr / (wwr * wwr + cr);
    double usl = ul - (pold - pl) / wwl;
    double usr = ur + (pold - pr) / wwr;
    double delp = fmax(qqr * qql / (qqr + qql) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabs(delp / (pold + smallpp));
  }
  pstar = pold;
  wl = sqrt(cl * (ONE + gamma6 * (pstar - pl) / pl));
  wr = sqrt(cr * (ONE + gamma6 * (pstar - pr) / pr));
  double ustar = HALF * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  double sgnm = copysign(ONE, ustar);
  double ro, uo, po, wo;
  if (sgnm > ZERO)
  {
    ro = rl, uo = ul, po = pl, wo = wl;
  }
  else
  {
    ro = rr, uo = ur, po = pr, wo = wr;
  }
  double co = fmax(smallc, sqrt(fabs(gamma0 * po / ro)));
  double rstar = fmax((double)(ro / (ONE + ro * (po - pstar) / (wo * wo))), (double)(smallr));
  double cstar = fmax(smallc, sqrt(fabs(gamma0 * pstar / rstar)));
  double spout = co - sgnm * uo;
  double spin = cstar - sgnm * ustar;
  double ushock = wo / ro - sgnm * uo;
  if (pstar >= po)
  {
    spin = ushock;
    spout = ushock;
  }
  double scr = fmax(spout - spin, smallc + fabs(spout + spin));
  double frac = HALF * (ONE + (spout + spin) / scr);
  if (frac != frac)
    frac = 0.0;
  else
    frac = frac >= 1.0 ? 1.0 : frac <= 0.0 ? 0.0 : frac;
  double qg[5];
  qg[EKO_ID] = frac * rstar + (ONE - frac) * ro;
  qg[EKO_IU] = frac * ustar + (ONE - frac) * uo;
  qg[EKO_IP] = frac * pstar + (ONE - frac) * po;
  if (spout < ZERO)
  {
    qg[EKO_ID] = ro, qg[EKO_IU] = uo, qg[EKO_IP] = po;
  }
  if (spin > ZERO)
  {
    qg[EKO_ID] = rstar, qg[EKO_IU] = ustar, qg[EKO_IP] = pstar;
  }
  if (sgnm > ZERO)
  {
    qg[EKO_IV] = ql[EKO_IV];
    if (nt == 2)
      qg[EKO_IW] = ql[EKO_IW];
  }
  else
  {
    qg[EKO_IV] = qr[EKO_IV];
    if (nt == 2)
      qg[EKO_IW] = qr[EKO_IW];
  }
  cmpflx(qg, flux, nt, p);
}

/* conservative state and flux of a primitive state, as riemann_llf and
 * riemann_hll build them (RiemannSolvers.h:262-320, 384-420) */
static void
hydro_uf(const double * q, double * u, double * f, int nt, double entho)
{
  u[EKO_ID] = q[EKO_ID];
  u[EKO_IP] = q[EKO_IP] * entho + HALF * q[EKO_ID] * q[EKO_IU] * q[EKO_IU];
  u[EKO_IP] += HALF * q[EKO_ID] * q[EKO_IV] * q[EKO_IV];
  if (nt == 2)
    u[EKO_IP] += HALF * q[EKO_ID] * q[EKO_IW] * q[EKO_IW];
  u[EKO_IU] = q[EKO_ID] * q[EKO_IU];
  u[EKO_IV] = q[EKO_ID] * q[EKO_IV];
  if (nt == 2)
    u[EKO_IW] = q[EKO_ID] * q[EKO_IW];
  f[EKO_ID] = u[EKO_ID] * q[EKO_IU];
  f[EKO_IP] = q[EKO_IU] * (u[EKO_IP] + q[EKO_IP]);
  f[EKO_IU] = q[EKO_IP] + u[EKO_IU] * q[EKO_IU];
  f[EKO_IV] = f[EKO_ID] * q[EKO_IV];
  if (nt == 2)
    f[EKO_IW] = f[EKO_ID] * q[EKO_IW];
}

/* riemann_llf: RiemannSolvers.h:218-330 */
static void
riemann_llf(const double * ql, const double * qr, double * flux, int nt, const eko_params * p)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp;
  const double entho = ONE / (gamma0 - ONE);
  double rl = fmax(ql[EKO_ID], smallr), ul = ql[EKO_IU], pl = fmax(ql[EKO_IP], rl * smallp);
  double rr = fmax(qr[EKO_ID], smallr), ur = qr[EKO_IU], pr = fmax(qr[EKO_IP], rr * smallp);
  double cl = sqrt(gamma0 * pl / rl);
  double cr = sqrt(gamma0 * pr / rr);
  double cmax = fmax(fabs(ul) + cl, fabs(ur) + cr);
  double uleft[5], uright[5], fleft[5], fright[5];
  hydro_uf(ql, uleft, fleft, nt, entho);
  hydro_uf(qr, uright, fright, nt, entho);
  for (int v = 0; v < 4; v++)
    flux[v] = HALF * (fleft[v] + fright[v] - cmax * (uright[v] - uleft[v]));
  if (nt == 2)
    flux[EKO_IW] = HALF * (fleft[EKO_IW] + fright[EKO_IW] - cmax * (uright[EKO_IW] - uleft[EKO_IW]));
}

/* riemann_hll: RiemannSolvers.h:344-432 (fleft[ID] is uleft[IU] here) */
static void
riemann_hll(const double * ql, const double * qr, double * flux, int nt, const eko_params * p)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp;
  const double entho = ONE / (gamma0 - ONE);
  double rl = fmax(ql[EKO_ID], smallr), ul = ql[EKO_IU], pl = fmax(ql[EKO_IP], rl * smallp);
  double rr = fmax(qr[EKO_ID], smallr), ur = qr[EKO_IU], pr = fmax(qr[EKO_IP], rr * smallp);
  double cl = sqrt(gamma0 * pl / rl);
  double cr = sqrt(gamma0 * pr / rr);
  double SL = fmin(fmin(ul, ur) - fmax(cl, cr), (double)ZERO);
  double SR = fmax(fmax(ul, ur) + fmax(cl, cr), (double)ZERO);
  double uleft[5], uright[5], fleft[5], fright[5];
  hydro_uf(ql, uleft, fleft, nt, entho);
  hydro_uf(qr, uright, fright, nt, entho);
  fleft[EKO_ID] = uleft[EKO_IU];
  fright[EKO_ID] = uright[EKO_IU];
  fleft[EKO_IV] = fleft[EKO_ID] * ql[EKO_IV];
  fright[EKO_IV] = fright[EKO_ID] * qr[EKO_IV];
  if (nt == 2)
  {
    fleft[EKO_IW] = fleft[EKO_ID] * ql[EKO_IW];
    fright[EKO_IW] = fright[EKO_ID] * qr[EKO_IW];
  }
  for (int v = 0; v < 4; v++)
    flux[v] = (SR * fleft[v] - SL * fright[v] + SR * SL * (uright[v] - uleft[v])) / (SR - SL);
  if (nt == 2)
    flux[EKO_IW] =
      (SR * fleft[EKO_IW] - SL * fright[EKO_IW] + SR * SL * (uright[EKO_IW] - uleft[EKO_IW])) / (SR - SL);
}

static void hllc(const double * ql, const double * qr, double * flux, int nt, const eko_params * p);

/* riemann_hydro: RiemannSolvers.h:573-640 (the 3D dispatch has no HLL
 * branch; HLL is refused for 3D by eko_create) */
static void
riemann_hydro(const double * ql, const double * qr, double * flux, int nt, const eko_params * p)
{
  if (p->riemann == EKO_RIEMANN_APPROX)
    riemann_approx(ql, qr, flux, nt, p);
  else if (p->riemann == EKO_RIEMANN_HLL)
    riemann_hll(ql, qr, flux, nt, p);
  else if (p->riemann == EKO_RIEMANN_LLF)
    riemann_llf(ql, qr, flux, nt, p);
  else
    hllc(ql, qr, flux, nt, p);
}

/* riemann_hllc: RiemannSolvers.h:445-568.  nt = number of transverse
 * velocities (1 in 2D: IV; 2 in 3D: IV, IW).  q layout [ID,IP,IU,IV,(IW)] */
static void
hllc(const double * ql, const double * qr, double * flux, int nt, const eko_params * p)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp, smallc = p->smallc;
  const double entho = ONE / (gamma0 - ONE);

  double rl = fmax(ql[EKO_ID], smallr);
  double pl = fmax(ql[EKO_IP], rl * smallp);
  double ul = ql[EKO_IU];
  double ecinl = HALF * rl * ul * ul;
  ecinl += HALF * rl * ql[EKO_IV] * ql[EKO_IV];
  if (nt == 2)
    ecinl += HALF * rl * ql[EKO_IW] * ql[EKO_IW];
  double etotl = pl * entho + ecinl;
  double ptotl = pl;

  double rr = fmax(qr[EKO_ID], smallr);
  double pr = fmax(qr[EKO_IP], rr * smallp);
  double ur = qr[EKO_IU];
  double ecinr = HALF * rr * ur * ur;
  ecinr += HALF * rr * qr[EKO_IV] * qr[EKO_IV];
  if (nt == 2)
    ecinr += HALF * rr * qr[EKO_IW] * qr[EKO_IW];
  double etotr = pr * entho + ecinr;
  double ptotr = pr;

  double cfastl = sqrt(fmax(gamma0 * pl / rl, smallc * smallc));
  double cfastr = sqrt(fmax(gamma0 * pr / rr, smallc * smallc));

  double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  double SR = fmax(ul, ur) + fmax(cfastl, cfastr);

  double rcl = rl * (ul - SL);
  double rcr = rr * (SR - ur);

  double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  double rstarl = rl * (SL - ul) / (SL - ustar);
  double etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
  double rstarr = rr * (SR - ur) / (SR - ustar);
  double etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);

  double ro, uo, ptoto, etoto;
  if (SL > ZERO)
  {
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (ustar > ZERO)
  {
    ro = rstarl;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarl;
  }
  else if (SR > ZERO)
  {
    ro = rstarr;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarr;
  }
  else
  {
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }
  flux[EKO_ID] = ro * uo;
  flux[EKO_IU] = ro * uo * uo + ptoto;
  flux[EKO_IP] = (etoto + ptoto) * uo;
  if (flux[EKO_ID] > ZERO)
    flux[EKO_IV] = flux[EKO_ID] * ql[EKO_IV];
  else
    flux[EKO_IV] = flux[EKO_ID] * qr[EKO_IV];
  if (nt == 2)
  {
    if (flux[EKO_ID] > ZERO)
      flux[EKO_IW] = flux[EKO_ID] * ql[EKO_IW];
    else
      flux[EKO_IW] = flux[EKO_ID] * qr[EKO_IW];
  }
}

/* ===================================================================== */
/* hydro                                                                  */
/* ===================================================================== */

/* computePrimitives: HydroBaseFunctor2D.h:78-102, HydroBaseFunctor3D.h:80-106 */
static inline void
hydro_prims(const double * u, double * q, double * c, int dim, const eko_params * p)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp;
  double d = fmax(u[EKO_ID], smallr);
  double ux = u[EKO_IU] / d;
  double uy = u[EKO_IV] / d;
  double eken;
  double uz = 0.0;
  if (dim == 2)
    eken = HALF * (ux * ux + uy * uy);
  else
  {
    uz = u[EKO_IW] / d;
    eken = HALF * (ux * ux + uy * uy + uz * uz);
  }
  double e = u[EKO_IP] / d - eken;
  double pr = fmax((gamma0 - 1.0) * d * e, d * smallp);
  *c = sqrt(gamma0 * (pr) / d);
  q[EKO_ID] = d;
  q[EKO_IP] = pr;
  q[EKO_IU] = ux;
  q[EKO_IV] = uy;
  if (dim == 3)
    q[EKO_IW] = uz;
}

/* the CFL term of ComputeDtGravityFunctor2D/3D (HydroRunFunctors2D.h:158-169,
 * HydroRunFunctors3D.h:162-183): g dt^2 / (2 dx) + u dt / dx <= cfl with
 * u = sum(|v_i| + c), g = sum(|g_i|), dx = min(dx, dy[, dz]) */
static inline double
grav_invdt(const eko_solver * s, const double * q, double cs, long c)
{
  const eko_params * p = &s->p;
  double dxm = fmin(p->dx, p->dy);
  if (p->dim == 3)
    dxm = fmin(dxm, p->dz);
  double velocity = 0.0;
  velocity += cs + fabs(q[EKO_IU]);
  velocity += cs + fabs(q[EKO_IV]);
  double kk = fabs(AT(s->G, s, 0, c)) + fabs(AT(s->G, s, 1, c));
  if (p->dim == 3)
  {
    velocity += cs + fabs(q[EKO_IW]);
    kk = kk + fabs(AT(s->G, s, 2, c));
  }
  kk *= p->cfl * dxm / (velocity * velocity);
  kk = fmax(kk, 1e-4);
  velocity *= kk / (sqrt(1.0 + 2.0 * kk) - 1.0);
  return velocity / dxm;
}

/* ComputeDtFunctor2D/3D: HydroRunFunctors2D.h:18-88, HydroRunFunctors3D.h:16-87 */
static double
hydro_compute_dt_local(eko_solver * s, const double * U)
{
  const eko_params * p = &s->p;
  const int gw = p->gw, dim = p->dim;
  const int ks = dim == 3 ? p->ksize : 1;
  const int k0 = dim == 3 ? gw : 0, k1 = dim == 3 ? ks - gw : 1;
  double invDt = -DBL_MAX;
#pragma omp parallel
  {
    double local = -DBL_MAX;
#pragma omp for collapse(2) schedule(static)
    for (int k = k0; k < k1; ++k)
      for (int j = gw; j < p->jsize - gw; ++j)
        for (int i = gw; i < p->isize - gw; ++i)
        {
          long   c = IDX(s, i, j, k);
          double u[5], q[5], cs;
          for (int v = 0; v < p->nbvar; ++v)
            u[v] = AT(U, s, v, c);
          hydro_prims(u, q, &cs, dim, p);
          if (p->grav_enabled)
          {
            local = fmax(local, grav_invdt(s, q, cs, c));
            continue;
          }
          double vx = cs + fabs(q[EKO_IU]);
          double vy = cs + fabs(q[EKO_IV]);
          if (dim == 2)
            local = fmax(local, vx / p->dx + vy / p->dy);
          else
          {
            double vz = cs + fabs(q[EKO_IW]);
            local = fmax(local, vx / p->dx + vy / p->dy + vz / p->dz);
          }
        }
#pragma omp critical
    invDt = local > invDt ? local : invDt;
  }
  return p->cfl / invDt;
}

/* trace_unsplit_{2d,3d}_along_dir: HydroBaseFunctor2D.h:216-293,
 * HydroBaseFunctor3D.h:276-367.  face: 0 XMIN,1 XMAX,2 YMIN,3 YMAX,4 ZMIN,5 ZMAX */
static void
hydro_trace(const double * q, const double * dqX, const double * dqY, const double * dqZ,
            double dtdx, double dtdy, double dtdz, int face, double * qf, int dim,
            const eko_params * p)
{
  const double gamma0 = p->gamma0, smallr = p->smallr;
  double r = q[EKO_ID], pp = q[EKO_IP], u = q[EKO_IU], v = q[EKO_IV];
  double drx = dqX[EKO_ID], dpx = dqX[EKO_IP], dux = dqX[EKO_IU], dvx = dqX[EKO_IV];
  double dry = dqY[EKO_ID], dpy = dqY[EKO_IP], duy = dqY[EKO_IU], dvy = dqY[EKO_IV];
  if (dim == 2)
  {
    double sr0 = -u * drx - v * dry - (dux + dvy) * r;
    double sp0 = -u * dpx - v * dpy - (dux + dvy) * gamma0 * pp;
    double su0 = -u * dux - v * duy - (dpx) / r;
    double sv0 = -u * dvx - v * dvy - (dpy) / r;
    const double * d = face < 2 ? dqX : dqY;
    double         dtd = face < 2 ? dtdx : dtdy;
    double         sgn = (face % 2 == 0) ? -1.0 : 1.0;
    if (sgn < 0)
    {
      qf[EKO_ID] = r - HALF * d[EKO_ID] + sr0 * dtd * HALF;
      qf[EKO_IP] = pp - HALF * d[EKO_IP] + sp0 * dtd * HALF;
      qf[EKO_IU] = u - HALF * d[EKO_IU] + su0 * dtd * HALF;
      qf[EKO_IV] = v - HALF * d[EKO_IV] + sv0 * dtd * HALF;
    }
    else
    {
      qf[EKO_ID] = r + HALF * d[EKO_ID] + sr0 * dtd * HALF;
      qf[EKO_IP] = pp + HALF * d[EKO_IP] + sp0 * dtd * HALF;
      qf[EKO_IU] = u + HALF * d[EKO_IU] + su0 * dtd * HALF;
      qf[EKO_IV] = v + HALF * d[EKO_IV] + sv0 * dtd * HALF;
    }
    qf[EKO_ID] = fmax(smallr, qf[EKO_ID]);
  }
  else
  {
    double w = q[EKO_IW];
    double dwx = dqX[EKO_IW], dwy = dqY[EKO_IW];
    double drz = dqZ[EKO_ID], dpz = dqZ[EKO_IP], duz = dqZ[EKO_IU], dvz = dqZ[EKO_IV],
           dwz = dqZ[EKO_IW];
    double sr0 = -u * drx - v * dry - w * drz - (dux + dvy + dwz) * r;
    double sp0 = -u * dpx - v * dpy - w * dpz - (dux + dvy + dwz) * gamma0 * pp;
    double su0 = -u * dux - v * duy - w * duz - (dpx) / r;
    double sv0 = -u * dvx - v * dvy - w * dvz - (dpy) / r;
    double sw0 = -u * dwx - v * dwy - w * dwz - (dpz) / r;
    const double * d = face < 2 ? dqX : (face < 4 ? dqY : dqZ);
    double         dtd = face < 2 ? dtdx : (face < 4 ? dtdy : dtdz);
    if (face % 2 == 0)
    {
      qf[EKO_ID] = r - HALF * d[EKO_ID] + sr0 * dtd * HALF;
      qf[EKO_IP] = pp - HALF * d[EKO_IP] + sp0 * dtd * HALF;
      qf[EKO_IU] = u - HALF * d[EKO_IU] + su0 * dtd * HALF;
      qf[EKO_IV] = v - HALF * d[EKO_IV] + sv0 * dtd * HALF;
      qf[EKO_IW] = w - HALF * d[EKO_IW] + sw0 * dtd * HALF;
    }
    else
    {
      qf[EKO_ID] = r + HALF * d[EKO_ID] + sr0 * dtd * HALF;
      qf[EKO_IP] = pp + HALF * d[EKO_IP] + sp0 * dtd * HALF;
      qf[EKO_IU] = u + HALF * d[EKO_IU] + su0 * dtd * HALF;
      qf[EKO_IV] = v + HALF * d[EKO_IV] + sv0 * dtd * HALF;
      qf[EKO_IW] = w + HALF * d[EKO_IW] + sw0 * dtd * HALF;
    }
    qf[EKO_ID] = fmax(smallr, qf[EKO_ID]);
  }
}

static inline void
swapd(double * a, double * b)
{
  double t = *a;
  *a = *b;
  *b = t;
}

/* godunov_unsplit_impl v0 (SolverHydroMuscl.cpp:214-243 and :304-330):
 * make_boundaries(in); out = in; Q = prims(in);
 * ComputeAndStoreFluxesFunctor (HydroRunFunctors2D.h:489-770,
 * HydroRunFunctors3D.h:271-717); UpdateFunctor (HydroRunFunctors2D.h:773-848,
 * HydroRunFunctors3D.h:722-820). */
static void
hydro_godunov(eko_solver * s, double * in, double * out, double dt)
{
  const eko_params * p = &s->p;
  const int dim = p->dim, nb = p->nbvar, gw = p->gw;
  const int is = p->isize, js = p->jsize, ks = dim == 3 ? p->ksize : 1;
  const double dtdx = dt / p->dx, dtdy = dt / p->dy, dtdz = dt / p->dz;
  const long ncell = s->ncell;

  make_boundaries(s, in);
  memcpy(out, in, sizeof(double) * ncell * nb);

  /* ConvertToPrimitivesFunctor: all cells */
#pragma omp parallel for schedule(static)
  for (long c = 0; c < ncell; ++c)
  {
    double u[5], q[5], cs;
    for (int v = 0; v < nb; ++v)
      u[v] = AT(in, s, v, c);
    hydro_prims(u, q, &cs, dim, p);
    for (int v = 0; v < nb; ++v)
      AT(s->Q, s, v, c) = q[v];
  }

  /* slopes of every cell with a full neighbourhood (the reference
   * recomputes them per face; the values are identical) */
  const int kl = dim == 3 ? 1 : 0, kh = dim == 3 ? ks - 1 : 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = kl; k < kh; ++k)
    for (int j = 1; j < js - 1; ++j)
      for (int i = 1; i < is - 1; ++i)
      {
        long c = IDX(s, i, j, k);
        long cxp = c + 1, cxm = c - 1, cyp = c + is, cym = c - is;
        long czp = c + (long)is * js, czm = c - (long)is * js;
        for (int v = 0; v < nb; ++v)
        {
          double q = AT(s->Q, s, v, c);
          AT(s->Sx, s, v, c) = slope1(q, AT(s->Q, s, v, cxp), AT(s->Q, s, v, cxm), p->slope_type);
          AT(s->Sy, s, v, c) = slope1(q, AT(s->Q, s, v, cyp), AT(s->Q, s, v, cym), p->slope_type);
          if (dim == 3)
            AT(s->Sz, s, v, c) =
              slope1(q, AT(s->Q, s, v, czp), AT(s->Q, s, v, czm), p->slope_type);
        }
      }

  /* fluxes at the left faces of i in [gw, isize-gw] (inclusive) */
  const int kf0 = dim == 3 ? gw : 0, kf1 = dim == 3 ? ks - gw : 0;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = kf0; k <= kf1; ++k)
    for (int j = gw; j <= js - gw; ++j)
      for (int i = gw; i <= is - gw; ++i)
      {
        long   c = IDX(s, i, j, k);
        double q[5], dqx[5], dqy[5], dqz[5] = { 0, 0, 0, 0, 0 };
        double qn[5], dnx[5], dny[5], dnz[5] = { 0, 0, 0, 0, 0 };
        double ql[5], qr[5], fl[5];
        for (int v = 0; v < nb; ++v)
        {
          q[v] = AT(s->Q, s, v, c);
          dqx[v] = AT(s->Sx, s, v, c);
          dqy[v] = AT(s->Sy, s, v, c);
          if (dim == 3)
            dqz[v] = AT(s->Sz, s, v, c);
        }
        long nbr[3] = { c - 1, c - is, c - (long)is * js };
        double dtdd[3] = { dtdx, dtdy, dtdz };
        double * F[3] = { s->Fx, s->Fy, s->Fz };
        for (int d = 0; d < dim; ++d)
        {
          long cn = nbr[d];
          for (int v = 0; v < nb; ++v)
          {
            qn[v] = AT(s->Q, s, v, cn);
            dnx[v] = AT(s->Sx, s, v, cn);
            dny[v] = AT(s->Sy, s, v, cn);
            if (dim == 3)
              dnz[v] = AT(s->Sz, s, v, cn);
          }
          hydro_trace(q, dqx, dqy, dqz, dtdx, dtdy, dtdz, 2 * d, qr, dim, p);
          hydro_trace(qn, dnx, dny, dnz, dtdx, dtdy, dtdz, 2 * d + 1, ql, dim, p);
          if (p->grav_enabled && p->grav_hancock)
          {
            /* gravity predictor, half time step (HydroRunFunctors2D.h:656-665,
             * HydroRunFunctors3D.h:489-500) */
            for (int e = 0; e < dim; ++e)
              ql[EKO_IU + e] += 0.5 * dt * AT(s->G, s, e, cn);
            for (int e = 0; e < dim; ++e)
              qr[EKO_IU + e] += 0.5 * dt * AT(s->G, s, e, c);
          }
          int it = EKO_IU + d; /* normal velocity index */
          if (d > 0)
          {
            swapd(&ql[EKO_IU], &ql[it]);
            swapd(&qr[EKO_IU], &qr[it]);
          }
          riemann_hydro(ql, qr, fl, dim == 3 ? 2 : 1, p);
          if (d > 0)
            swapd(&fl[EKO_IU], &fl[it]);
          for (int v = 0; v < nb; ++v)
            AT(F[d], s, v, c) = fl[v] * dtdd[d];
        }
      }

  /* update interior */
  const int ku0 = dim == 3 ? gw : 0, ku1 = dim == 3 ? ks - gw : 1;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = ku0; k < ku1; ++k)
    for (int j = gw; j < js - gw; ++j)
      for (int i = gw; i < is - gw; ++i)
      {
        long c = IDX(s, i, j, k);
        for (int v = 0; v < nb; ++v)
        {
          double u = AT(out, s, v, c);
          u += AT(s->Fx, s, v, c);
          u -= AT(s->Fx, s, v, c + 1);
          u += AT(s->Fy, s, v, c);
          u -= AT(s->Fy, s, v, c + is);
          if (dim == 3)
          {
            u += AT(s->Fz, s, v, c);
            u -= AT(s->Fz, s, v, c + (long)is * js);
          }
          AT(out, s, v, c) = u;
        }
      }

  if (p->grav_enabled)
  {
    /* GravitySourceTermFunctor2D/3D (HydroRunFunctors2D.h:1555-1630,
     * HydroRunFunctors3D.h:1903-1980); the 2D form floors the new density */
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = ku0; k < ku1; ++k)
      for (int j = gw; j < js - gw; ++j)
        for (int i = gw; i < is - gw; ++i)
        {
          long   c = IDX(s, i, j, k);
          double rhoOld = AT(in, s, EKO_ID, c);
          double rhoNew = dim == 2 ? fmax(p->smallr, AT(out, s, EKO_ID, c)) : AT(out, s, EKO_ID, c);
          double rhou = AT(out, s, EKO_IU, c), rhov = AT(out, s, EKO_IV, c), rhow = 0.0;
          double ekin_old, ekin_new;
          if (dim == 2)
            ekin_old = 0.5 * (rhou * rhou + rhov * rhov) / rhoNew;
          else
          {
            rhow = AT(out, s, EKO_IW, c);
            ekin_old = 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rhoNew;
          }
          rhou += 0.5 * dt * AT(s->G, s, 0, c) * (rhoOld + rhoNew);
          rhov += 0.5 * dt * AT(s->G, s, 1, c) * (rhoOld + rhoNew);
          AT(out, s, EKO_IU, c) = rhou;
          AT(out, s, EKO_IV, c) = rhov;
          if (dim == 2)
            ekin_new = 0.5 * (rhou * rhou + rhov * rhov) / rhoNew;
          else
          {
            rhow += 0.5 * dt * AT(s->G, s, 2, c) * (rhoOld + rhoNew);
            AT(out, s, EKO_IW, c) = rhow;
            ekin_new = 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rhoNew;
          }
          AT(out, s, EKO_IP, c) += (ekin_new - ekin_old);
        }
  }
}

/* ===================================================================== */
/* MHD 3D                                                                 */
/* ===================================================================== */

/* constoprim_mhd: MHDBaseFunctor3D.h:194-242 */
static inline void
mhd_constoprim(const double * u, const double * bnb, double * q, const eko_params * p)
{
  q[EKO_ID] = fmax(u[EKO_ID], p->smallr);
  q[EKO_IU] = u[EKO_IU] / q[EKO_ID];
  q[EKO_IV] = u[EKO_IV] / q[EKO_ID];
  q[EKO_IW] = u[EKO_IW] / q[EKO_ID];
  q[EKO_IA] = 0.5 * (u[EKO_IA] + bnb[0]);
  q[EKO_IB] = 0.5 * (u[EKO_IB] + bnb[1]);
  q[EKO_IC] = 0.5 * (u[EKO_IC] + bnb[2]);
  double eken = 0.5 * (q[EKO_IU] * q[EKO_IU] + q[EKO_IV] * q[EKO_IV] + q[EKO_IW] * q[EKO_IW]);
  double emag = 0.5 * (q[EKO_IA] * q[EKO_IA] + q[EKO_IB] * q[EKO_IB] + q[EKO_IC] * q[EKO_IC]);
  if (p->cIso > 0)
  {
    q[EKO_IP] = q[EKO_ID] * (p->cIso) * (p->cIso);
  }
  else
  {
    double eint = (u[EKO_IP] - emag) / q[EKO_ID] - eken;
    q[EKO_IP] = fmax((p->gamma0 - 1.0) * q[EKO_ID] * eint, q[EKO_ID] * p->smallp);
  }
}

/* find_speed_fast<dir>: mhd_utils.h:89-117 */
static inline double
speed_fast(const double * q, int dir, double gamma0)
{
  double d = q[EKO_ID], pp = q[EKO_IP], a = q[EKO_IA], b = q[EKO_IB], c = q[EKO_IC];
  double b2 = a * a + b * b + c * c;
  double c2 = gamma0 * pp / d;
  double d2 = 0.5 * (b2 / d + c2);
  double bn = dir == 0 ? a : (dir == 1 ? b : c);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * bn * bn / d));
}

/* find_speed_info<THREE_D>: mhd_utils.h:319-366 */
static inline void
speed_info3(const double * q, double * f, double gamma0)
{
  double d = q[EKO_ID], pp = q[EKO_IP], a = q[EKO_IA], b = q[EKO_IB], c = q[EKO_IC];
  double b2 = a * a + b * b + c * c;
  double c2 = gamma0 * pp / d;
  double d2 = 0.5 * (b2 / d + c2);
  double cf = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
  f[0] = cf + fabs(q[EKO_IU]);
  cf = sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
  f[1] = cf + fabs(q[EKO_IV]);
  cf = sqrt(d2 + sqrt(d2 * d2 - c2 * c * c / d));
  f[2] = cf + fabs(q[EKO_IW]);
}

/* riemann_hlld: RiemannSolvers_MHD.h:130-364 (qleft/qright are modified) */
static void
hlld(double * ql, double * qr, double * flux, const eko_params * p)
{
  const double gamma0 = p->gamma0;
  const double entho = 1.0 / (gamma0 - 1.0);
  double a = 0.5 * (ql[EKO_IA] + qr[EKO_IA]);
  double sgnm = (a >= 0) ? ONE : -ONE;
  ql[EKO_IA] = a;
  qr[EKO_IA] = a;
  if (p->cIso > 0)
  {
    ql[EKO_IP] = ql[EKO_ID] * p->cIso * p->cIso;
    qr[EKO_IP] = qr[EKO_ID] * p->cIso * p->cIso;
  }
  double rl = ql[EKO_ID], pl = ql[EKO_IP], ul = ql[EKO_IU], vl = ql[EKO_IV], wl = ql[EKO_IW],
         bl = ql[EKO_IB], cl = ql[EKO_IC];
  double ecinl = 0.5 * (ul * ul + vl * vl + wl * wl) * rl;
  double emagl = 0.5 * (a * a + bl * bl + cl * cl);
  double etotl = pl * entho + ecinl + emagl;
  double ptotl = pl + emagl;
  double vdotbl = ul * a + vl * bl + wl * cl;

  double rr = qr[EKO_ID], pr = qr[EKO_IP], ur = qr[EKO_IU], vr = qr[EKO_IV], wr = qr[EKO_IW],
         br = qr[EKO_IB], cr = qr[EKO_IC];
  double ecinr = 0.5 * (ur * ur + vr * vr + wr * wr) * rr;
  double emagr = 0.5 * (a * a + br * br + cr * cr);
  double etotr = pr * entho + ecinr + emagr;
  double ptotr = pr + emagr;
  double vdotbr = ur * a + vr * br + wr * cr;

  double cfastl = speed_fast(ql, 0, gamma0);
  double cfastr = speed_fast(qr, 0, gamma0);

  double sl = fmin(ul, ur) - fmax(cfastl, cfastr);
  double sr = fmax(ul, ur) + fmax(cfastl, cfastr);

  double rcl = rl * (ul - sl);
  double rcr = rr * (sr - ur);

  double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  double estar, rstarl, el;
  rstarl = rl * (sl - ul) / (sl - ustar);
  estar = rl * (sl - ul) * (sl - ustar) - a * a;
  el = rl * (sl - ul) * (sl - ul) - a * a;
  double vstarl, wstarl, bstarl, cstarl;
  if (a * a > 0 && fabs(estar / (a * a) - ONE) <= 1e-8)
  {
    vstarl = vl;
    bstarl = bl;
    wstarl = wl;
    cstarl = cl;
  }
  else
  {
    vstarl = vl - a * bl * (ustar - ul) / estar;
    bstarl = bl * el / estar;
    wstarl = wl - a * cl * (ustar - ul) / estar;
    cstarl = cl * el / estar;
  }
  double vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  double etotstarl =
    ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) / (sl - ustar);
  double sqrrstarl = sqrt(rstarl);
  double calfvenl = fabs(a) / sqrrstarl;
  double sal = ustar - calfvenl;

  double rstarr, er;
  rstarr = rr * (sr - ur) / (sr - ustar);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  er = rr * (sr - ur) * (sr - ur) - a * a;
  double vstarr, wstarr, bstarr, cstarr;
  if (a * a > 0 && fabs(estar / (a * a) - ONE) <= 1e-8)
  {
    vstarr = vr;
    bstarr = br;
    wstarr = wr;
    cstarr = cr;
  }
  else
  {
    vstarr = vr - a * br * (ustar - ur) / estar;
    bstarr = br * er / estar;
    wstarr = wr - a * cr * (ustar - ur) / estar;
    cstarr = cr * er / estar;
  }
  double vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  double etotstarr =
    ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) / (sr - ustar);
  double sqrrstarr = sqrt(rstarr);
  double calfvenr = fabs(a) / sqrrstarr;
  double sar = ustar + calfvenr;

  double vstarstar =
    (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) / (sqrrstarl + sqrrstarr);
  double wstarstar =
    (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) / (sqrrstarl + sqrrstarr);
  double bstarstar =
    (sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl)) /
    (sqrrstarl + sqrrstarr);
  double cstarstar =
    (sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl)) /
    (sqrrstarl + sqrrstarr);
  double vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
  double etotstarstarl = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
  double etotstarstarr = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);

  double ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > 0)
  {
    ro = rl; uo = ul; vo = vl; wo = wl; bo = bl; co = cl;
    ptoto = ptotl; etoto = etotl; vdotbo = vdotbl;
  }
  else if (sal > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarl; wo = wstarl; bo = bstarl; co = cstarl;
    ptoto = ptotstar; etoto = etotstarl; vdotbo = vdotbstarl;
  }
  else if (ustar > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarl; vdotbo = vdotbstarstar;
  }
  else if (sar > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarr; vdotbo = vdotbstarstar;
  }
  else if (sr > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarr; wo = wstarr; bo = bstarr; co = cstarr;
    ptoto = ptotstar; etoto = etotstarr; vdotbo = vdotbstarr;
  }
  else
  {
    ro = rr; uo = ur; vo = vr; wo = wr; bo = br; co = cr;
    ptoto = ptotr; etoto = etotr; vdotbo = vdotbr;
  }
  flux[EKO_ID] = ro * uo;
  flux[EKO_IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[EKO_IU] = ro * uo * uo - a * a + ptoto;
  flux[EKO_IV] = ro * uo * vo - a * bo;
  flux[EKO_IW] = ro * uo * wo - a * co;
  flux[EKO_IA] = 0.0;
  flux[EKO_IB] = bo * uo - a * vo;
  flux[EKO_IC] = co * uo - a * wo;
}

/* find_mhd_flux: mhd_utils.h:170-231 (cIso = 0) */
static void
find_mhd_flux(const double * q, double * cv, double * ff, const eko_params * p)
{
  const double pp = q[EKO_IP];
  const double entho = ONE / (p->gamma0 - ONE);
  const double d = q[EKO_ID], u = q[EKO_IU], v = q[EKO_IV], w = q[EKO_IW], a = q[EKO_IA], b = q[EKO_IB],
               c = q[EKO_IC];
  const double ecin = 0.5 * (u * u + v * v + w * w) * d;
  const double emag = 0.5 * (a * a + b * b + c * c);
  const double etot = pp * entho + ecin + emag;
  const double ptot = pp + emag;
  cv[EKO_ID] = d, cv[EKO_IP] = etot, cv[EKO_IU] = d * u, cv[EKO_IV] = d * v, cv[EKO_IW] = d * w;
  cv[EKO_IA] = a, cv[EKO_IB] = b, cv[EKO_IC] = c;
  ff[EKO_ID] = d * u;
  ff[EKO_IP] = (etot + ptot) * u - a * (a * u + b * v + c * w);
  ff[EKO_IU] = d * u * u - a * a + ptot;
  ff[EKO_IV] = d * u * v - a * b;
  ff[EKO_IW] = d * u * w - a * c;
  ff[EKO_IA] = 0.0;
  ff[EKO_IB] = b * u - a * v;
  ff[EKO_IC] = c * u - a * w;
}

/* riemann_hll (MHD): RiemannSolvers_MHD.h:27-62 (qleft/qright are modified) */
static void
mhd_hll(double * ql, double * qr, double * flux, const eko_params * p)
{
  double bx_mean = 0.5 * (ql[EKO_IA] + qr[EKO_IA]);
  ql[EKO_IA] = bx_mean;
  qr[EKO_IA] = bx_mean;
  double uleft[8], fleft[8], uright[8], fright[8];
  find_mhd_flux(ql, uleft, fleft, p);
  find_mhd_flux(qr, uright, fright, p);
  double cfleft = speed_fast(ql, 0, p->gamma0);
  double cfright = speed_fast(qr, 0, p->gamma0);
  double vleft = ql[EKO_IU], vright = qr[EKO_IU];
  double sl = fmin(fmin(vleft, vright) - fmax(cfleft, cfright), 0.0);
  double sr = fmax(fmax(vleft, vright) + fmax(cfleft, cfright), 0.0);
  for (int v = 0; v < 8; ++v)
    flux[v] = (sr * fleft[v] - sl * fright[v] + sr * sl * (uright[v] - uleft[v])) / (sr - sl);
}

/* riemann_llf (MHD): RiemannSolvers_MHD.h:77-104, find_speed_info of one
 * direction (mhd_utils.h:379-403) */
static void
mhd_llf(double * ql, double * qr, double * flux, const eko_params * p)
{
  double bx_mean = HALF * (ql[EKO_IA] + qr[EKO_IA]);
  ql[EKO_IA] = bx_mean;
  qr[EKO_IA] = bx_mean;
  double uleft[8], fleft[8], uright[8], fright[8];
  find_mhd_flux(ql, uleft, fleft, p);
  find_mhd_flux(qr, uright, fright, p);
  for (int v = 0; v < 8; ++v)
    flux[v] = (fleft[v] + fright[v]) / 2;
  double cleft = speed_fast(ql, 0, p->gamma0) + fabs(ql[EKO_IU]);
  double cright = speed_fast(qr, 0, p->gamma0) + fabs(qr[EKO_IU]);
  double vel_info = fmax(cleft, cright);
  for (int v = 0; v < 8; ++v)
    flux[v] -= vel_info * (uright[v] - uleft[v]) / 2;
}

static void hlld(double * ql, double * qr, double * flux, const eko_params * p);

/* riemann_mhd: RiemannSolvers_MHD.h:368-389 */
static void
riemann_mhd(double * ql, double * qr, double * flux, const eko_params * p)
{
  if (p->riemann == EKO_RIEMANN_HLL)
    mhd_hll(ql, qr, flux, p);
  else if (p->riemann == EKO_RIEMANN_LLF)
    mhd_llf(ql, qr, flux, p);
  else
    hlld(ql, qr, flux, p);
}

/* FMAX4/FMIN4/FMAX5: mhd_utils.h:38-75 */
static inline double
fmax4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  return r;
}
static inline double
fmin4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 < r) ? a1 : r;
  r = (a2 < r) ? a2 : r;
  r = (a3 < r) ? a3 : r;
  return r;
}
static inline double
fmax5(double a0, double a1, double a2, double a3, double a4)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  r = (a4 > r) ? a4 : r;
  return r;
}

/* mag_riemann2d_hlld: RiemannSolvers_MHD.h:395-627.  q[4][8] in the order
 * ILL, IRL, ILR, IRR (enums.h:205-211); e[4] the four edge emfs. */
static double
mag_riemann2d_hlld(double q[4][8], const double * e, const eko_params * p)
{
  const double *qLL = q[0], *qRL = q[1], *qLR = q[2], *qRR = q[3];
  const double ELL = e[0], ERL = e[1], ELR = e[2], ERR = e[3];
  const double g = p->gamma0;
  double rLL = qLL[EKO_ID], pLL = qLL[EKO_IP], uLL = qLL[EKO_IU], vLL = qLL[EKO_IV],
         aLL = qLL[EKO_IA], bLL = qLL[EKO_IB], cLL = qLL[EKO_IC];
  double rLR = qLR[EKO_ID], pLR = qLR[EKO_IP], uLR = qLR[EKO_IU], vLR = qLR[EKO_IV],
         aLR = qLR[EKO_IA], bLR = qLR[EKO_IB], cLR = qLR[EKO_IC];
  double rRL = qRL[EKO_ID], pRL = qRL[EKO_IP], uRL = qRL[EKO_IU], vRL = qRL[EKO_IV],
         aRL = qRL[EKO_IA], bRL = qRL[EKO_IB], cRL = qRL[EKO_IC];
  double rRR = qRR[EKO_ID], pRR = qRR[EKO_IP], uRR = qRR[EKO_IU], vRR = qRR[EKO_IV],
         aRR = qRR[EKO_IA], bRR = qRR[EKO_IB], cRR = qRR[EKO_IC];

  double cFastLLx = speed_fast(qLL, 0, g), cFastLRx = speed_fast(qLR, 0, g);
  double cFastRLx = speed_fast(qRL, 0, g), cFastRRx = speed_fast(qRR, 0, g);
  double cFastLLy = speed_fast(qLL, 1, g), cFastLRy = speed_fast(qLR, 1, g);
  double cFastRLy = speed_fast(qRL, 1, g), cFastRRy = speed_fast(qRR, 1, g);

  double SL = fmin4(uLL, uLR, uRL, uRR) - fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  double SR = fmax4(uLL, uLR, uRL, uRR) + fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  double SB = fmin4(vLL, vLR, vRL, vRR) - fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  double ST = fmax4(vLL, vLR, vRL, vRR) + fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);

  double PtotLL = pLL + HALF * (aLL * aLL + bLL * bLL + cLL * cLL);
  double PtotLR = pLR + HALF * (aLR * aLR + bLR * bLR + cLR * cLR);
  double PtotRL = pRL + HALF * (aRL * aRL + bRL * bRL + cRL * cRL);
  double PtotRR = pRR + HALF * (aRR * aRR + bRR * bRR + cRR * cRR);

  double rcLLx = rLL * (uLL - SL);
  double rcRLx = rRL * (SR - uRL);
  double rcLRx = rLR * (uLR - SL);
  double rcRRx = rRR * (SR - uRR);
  double rcLLy = rLL * (vLL - SB);
  double rcLRy = rLR * (ST - vLR);
  double rcRLy = rRL * (vRL - SB);
  double rcRRy = rRR * (ST - vRR);

  double ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  double vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  double rstarLLx = rLL * (SL - uLL) / (SL - ustar);
  double BstarLL = bLL * (SL - uLL) / (SL - ustar);
  double rstarLLy = rLL * (SB - vLL) / (SB - vstar);
  double AstarLL = aLL * (SB - vLL) / (SB - vstar);
  double rstarLL = rLL * (SL - uLL) / (SL - ustar) * (SB - vLL) / (SB - vstar);
  double EstarLLx = ustar * BstarLL - vLL * aLL;
  double EstarLLy = uLL * bLL - vstar * AstarLL;
  double EstarLL = ustar * BstarLL - vstar * AstarLL;

  double rstarLRx = rLR * (SL - uLR) / (SL - ustar);
  double BstarLR = bLR * (SL - uLR) / (SL - ustar);
  double rstarLRy = rLR * (ST - vLR) / (ST - vstar);
  double AstarLR = aLR * (ST - vLR) / (ST - vstar);
  double rstarLR = rLR * (SL - uLR) / (SL - ustar) * (ST - vLR) / (ST - vstar);
  double EstarLRx = ustar * BstarLR - vLR * aLR;
  double EstarLRy = uLR * bLR - vstar * AstarLR;
  double EstarLR = ustar * BstarLR - vstar * AstarLR;

  double rstarRLx = rRL * (SR - uRL) / (SR - ustar);
  double BstarRL = bRL * (SR - uRL) / (SR - ustar);
  double rstarRLy = rRL * (SB - vRL) / (SB - vstar);
  double AstarRL = aRL * (SB - vRL) / (SB - vstar);
  double rstarRL = rRL * (SR - uRL) / (SR - ustar) * (SB - vRL) / (SB - vstar);
  double EstarRLx = ustar * BstarRL - vRL * aRL;
  double EstarRLy = uRL * bRL - vstar * AstarRL;
  double EstarRL = ustar * BstarRL - vstar * AstarRL;

  double rstarRRx = rRR * (SR - uRR) / (SR - ustar);
  double BstarRR = bRR * (SR - uRR) / (SR - ustar);
  double rstarRRy = rRR * (ST - vRR) / (ST - vstar);
  double AstarRR = aRR * (ST - vRR) / (ST - vstar);
  double rstarRR = rRR * (SR - uRR) / (SR - ustar) * (ST - vRR) / (ST - vstar);
  double EstarRRx = ustar * BstarRR - vRR * aRR;
  double EstarRRy = uRR * bRR - vstar * AstarRR;
  double EstarRR = ustar * BstarRR - vstar * AstarRR;

  double calfvenL = fmax5(fabs(aLR) / sqrt(rstarLRx), fabs(AstarLR) / sqrt(rstarLR),
                          fabs(aLL) / sqrt(rstarLLx), fabs(AstarLL) / sqrt(rstarLL), p->smallc);
  double calfvenR = fmax5(fabs(aRR) / sqrt(rstarRRx), fabs(AstarRR) / sqrt(rstarRR),
                          fabs(aRL) / sqrt(rstarRLx), fabs(AstarRL) / sqrt(rstarRL), p->smallc);
  double calfvenB = fmax5(fabs(bLL) / sqrt(rstarLLy), fabs(BstarLL) / sqrt(rstarLL),
                          fabs(bRL) / sqrt(rstarRLy), fabs(BstarRL) / sqrt(rstarRL), p->smallc);
  double calfvenT = fmax5(fabs(bLR) / sqrt(rstarLRy), fabs(BstarLR) / sqrt(rstarLR),
                          fabs(bRR) / sqrt(rstarRRy), fabs(BstarRR) / sqrt(rstarRR), p->smallc);

  double SAL = fmin(ustar - calfvenL, ZERO);
  double SAR = fmax(ustar + calfvenR, ZERO);
  double SAB = fmin(vstar - calfvenB, ZERO);
  double SAT = fmax(vstar + calfvenT, ZERO);

  double AstarT = (SAR * AstarRR - SAL * AstarLR) / (SAR - SAL);
  double AstarB = (SAR * AstarRL - SAL * AstarLL) / (SAR - SAL);
  double BstarR = (SAT * BstarRR - SAB * BstarRL) / (SAT - SAB);
  double BstarL = (SAT * BstarLR - SAB * BstarLL) / (SAT - SAB);

  double E = 0, tmpE = 0;
  int SB_pos = (int)(1 + copysign(ONE, SB)) / 2, SB_neg = 1 - SB_pos;
  int ST_pos = (int)(1 + copysign(ONE, ST)) / 2, ST_neg = 1 - ST_pos;
  int SL_pos = (int)(1 + copysign(ONE, SL)) / 2, SL_neg = 1 - SL_pos;
  int SR_pos = (int)(1 + copysign(ONE, SR)) / 2, SR_neg = 1 - SR_pos;

  tmpE = (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) /
           (SAR - SAL) / (SAT - SAB) -
         SAT * SAB / (SAT - SAB) * (AstarT - AstarB) + SAR * SAL / (SAR - SAL) * (BstarR - BstarL);
  E += (SB_neg * ST_pos * SL_neg * SR_pos) * tmpE;

  tmpE = (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) / (SAR - SAL);
  tmpE = SL_pos * ELL + SL_neg * SR_neg * ERL + SL_neg * SR_pos * tmpE;
  E += SB_pos * tmpE;

  tmpE = (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) / (SAR - SAL);
  tmpE = SL_pos * ELR + SL_neg * SR_neg * ERR + SL_neg * SR_pos * tmpE;
  E += (SB_neg * ST_neg) * tmpE;

  tmpE = (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_pos) * tmpE;

  tmpE = (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_neg * SR_neg) * tmpE;
  return E;
}

/* compute_emf<EmfDir>: RiemannSolvers_MHD.h:648-871.  qE in the order
 * IRT, IRB, ILT, ILB (enums.h:196-202).  emfDir: 0 EMFX, 1 EMFY, 2 EMFZ */
static double
compute_emf(const double * qRT, const double * qRB, const double * qLT, const double * qLB,
            int emfDir, const eko_params * p)
{
  double q[4][8]; /* ILL, IRL, ILR, IRR */
  double *qLL = q[0], *qRL = q[1], *qLR = q[2], *qRR = q[3];
  qLL[EKO_ID] = qRT[EKO_ID];
  qRL[EKO_ID] = qLT[EKO_ID];
  qLR[EKO_ID] = qRB[EKO_ID];
  qRR[EKO_ID] = qLB[EKO_ID];
  if (p->cIso > 0)
  {
    qLL[EKO_IP] = qLL[EKO_ID] * p->cIso * p->cIso;
    qRL[EKO_IP] = qRL[EKO_ID] * p->cIso * p->cIso;
    qLR[EKO_IP] = qLR[EKO_ID] * p->cIso * p->cIso;
    qRR[EKO_IP] = qRR[EKO_ID] * p->cIso * p->cIso;
  }
  else
  {
    qLL[EKO_IP] = qRT[EKO_IP];
    qRL[EKO_IP] = qLT[EKO_IP];
    qLR[EKO_IP] = qRB[EKO_IP];
    qRR[EKO_IP] = qLB[EKO_IP];
  }
  /* parallel / orthogonal components: (iu,iv,iw,ia,ib,ic) */
  int iu, iv, iw, ia, ib, ic;
  if (emfDir == 2)
  {
    iu = EKO_IU; iv = EKO_IV; iw = EKO_IW; ia = EKO_IA; ib = EKO_IB; ic = EKO_IC;
  }
  else if (emfDir == 1)
  {
    iu = EKO_IW; iv = EKO_IU; iw = EKO_IV; ia = EKO_IC; ib = EKO_IA; ic = EKO_IB;
  }
  else
  {
    iu = EKO_IV; iv = EKO_IW; iw = EKO_IU; ia = EKO_IB; ib = EKO_IC; ic = EKO_IA;
  }
  qLL[EKO_IU] = qRT[iu];
  qRL[EKO_IU] = qLT[iu];
  qLR[EKO_IU] = qRB[iu];
  qRR[EKO_IU] = qLB[iu];
  qLL[EKO_IV] = qRT[iv];
  qRL[EKO_IV] = qLT[iv];
  qLR[EKO_IV] = qRB[iv];
  qRR[EKO_IV] = qLB[iv];
  qLL[EKO_IA] = HALF * (qRT[ia] + qLT[ia]);
  qRL[EKO_IA] = HALF * (qRT[ia] + qLT[ia]);
  qLR[EKO_IA] = HALF * (qRB[ia] + qLB[ia]);
  qRR[EKO_IA] = HALF * (qRB[ia] + qLB[ia]);
  qLL[EKO_IB] = HALF * (qRT[ib] + qRB[ib]);
  qRL[EKO_IB] = HALF * (qLT[ib] + qLB[ib]);
  qLR[EKO_IB] = HALF * (qRT[ib] + qRB[ib]);
  qRR[EKO_IB] = HALF * (qLT[ib] + qLB[ib]);
  qLL[EKO_IW] = qRT[iw];
  qRL[EKO_IW] = qLT[iw];
  qLR[EKO_IW] = qRB[iw];
  qRR[EKO_IW] = qLB[iw];
  qLL[EKO_IC] = qRT[ic];
  qRL[EKO_IC] = qLT[ic];
  qLR[EKO_IC] = qRB[ic];
  qRR[EKO_IC] = qLB[ic];
  double e[4];
  e[0] = qLL[EKO_IU] * qLL[EKO_IB] - qLL[EKO_IV] * qLL[EKO_IA];
  e[1] = qRL[EKO_IU] * qRL[EKO_IB] - qRL[EKO_IV] * qRL[EKO_IA];
  e[2] = qLR[EKO_IU] * qLR[EKO_IB] - qLR[EKO_IV] * qLR[EKO_IA];
  e[3] = qRR[EKO_IU] * qRR[EKO_IB] - qRR[EKO_IV] * qRR[EKO_IA];
  return mag_riemann2d_hlld(q, e, p);
}

/* trace_unsplit_mhd_3d_simpler: MHDBaseFunctor3D.h:690-1114 (Omega0 = 0
 * shearing terms included for completeness).  dq[3][8] is scaled in place.
 * Outputs qm[3][8], qp[3][8], qE[4][3][8] ([RT,RB,LT,LB][x,y,z]). */
static void
mhd_trace3d(const double * q, double dq[3][8], const double * bfNb, const double * dbf,
            double elec[3][2][2], double dtdx, double dtdy, double dtdz, double xPos,
            double qm[3][8], double qp[3][8], double qE[4][3][8], const eko_params * p)
{
  const double gamma = p->gamma0, smallR = p->smallr, smallp = p->smallp, Omega0 = p->Omega0;
  const double dx = p->dx;
  const double ELL = elec[0][0][0], ELR = elec[0][0][1], ERL = elec[0][1][0], ERR = elec[0][1][1];
  const double FLL = elec[1][0][0], FLR = elec[1][0][1], FRL = elec[1][1][0], FRR = elec[1][1][1];
  const double GLL = elec[2][0][0], GLR = elec[2][0][1], GRL = elec[2][1][0], GRR = elec[2][1][1];

  double r = q[EKO_ID], pp = q[EKO_IP], u = q[EKO_IU], v = q[EKO_IV], w = q[EKO_IW];
  double A = q[EKO_IA], B = q[EKO_IB], C = q[EKO_IC];
  double AL = bfNb[0], AR = bfNb[1], BL = bfNb[2], BR = bfNb[3], CL = bfNb[4], CR = bfNb[5];

  double drx = dq[0][EKO_ID] *= HALF;
  double dpx = dq[0][EKO_IP] *= HALF;
  double dux = dq[0][EKO_IU] *= HALF;
  double dvx = dq[0][EKO_IV] *= HALF;
  double dwx = dq[0][EKO_IW] *= HALF;
  double dCx = dq[0][EKO_IC] *= HALF;
  double dBx = dq[0][EKO_IB] *= HALF;
  double dry = dq[1][EKO_ID] *= HALF;
  double dpy = dq[1][EKO_IP] *= HALF;
  double duy = dq[1][EKO_IU] *= HALF;
  double dvy = dq[1][EKO_IV] *= HALF;
  double dwy = dq[1][EKO_IW] *= HALF;
  double dCy = dq[1][EKO_IC] *= HALF;
  double dAy = dq[1][EKO_IA] *= HALF;
  double drz = dq[2][EKO_ID] *= HALF;
  double dpz = dq[2][EKO_IP] *= HALF;
  double duz = dq[2][EKO_IU] *= HALF;
  double dvz = dq[2][EKO_IV] *= HALF;
  double dwz = dq[2][EKO_IW] *= HALF;
  double dAz = dq[2][EKO_IA] *= HALF;
  double dBz = dq[2][EKO_IB] *= HALF;

  double dALy = HALF * dbf[0], dALz = HALF * dbf[1], dBLx = HALF * dbf[2], dBLz = HALF * dbf[3];
  double dCLx = HALF * dbf[4], dCLy = HALF * dbf[5], dARy = HALF * dbf[6], dARz = HALF * dbf[7];
  double dBRx = HALF * dbf[8], dBRz = HALF * dbf[9], dCRx = HALF * dbf[10], dCRy = HALF * dbf[11];

  double dAx = HALF * (AR - AL);
  double dBy = HALF * (BR - BL);
  double dCz = HALF * (CR - CL);

  double sr0, su0, sv0, sw0, sp0, sA0, sB0, sC0;
  double sAL0, sAR0, sBL0, sBR0, sCL0, sCR0;
  sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
  su0 = (-u * dux - (dpx + B * dBx + C * dCx) / r) * dtdx + (-v * duy + B * dAy / r) * dtdy +
        (-w * duz + C * dAz / r) * dtdz;
  sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) / r) * dtdy +
        (-w * dvz + C * dBz / r) * dtdz;
  sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
        (-w * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
  sp0 = (-u * dpx - dux * gamma * pp) * dtdx + (-v * dpy - dvy * gamma * pp) * dtdy +
        (-w * dpz - dwz * gamma * pp) * dtdz;
  sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy +
        (u * dCz + C * duz - w * dAz - A * dwz) * dtdz;
  sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx +
        (v * dCz + C * dvz - w * dBz - B * dwz) * dtdz;
  sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx +
        (w * dBy + B * dwy - v * dCy - C * dvy) * dtdy;
  if (Omega0 > 0)
  {
    double shear = -1.5 * Omega0 * xPos;
    sr0 = sr0 - shear * dry * dtdy;
    su0 = su0 - shear * duy * dtdy;
    sv0 = sv0 - shear * dvy * dtdy;
    sw0 = sw0 - shear * dwy * dtdy;
    sp0 = sp0 - shear * dpy * dtdy;
    sA0 = sA0 - shear * dAy * dtdy;
    sB0 = sB0 + (shear * dAx - 1.5 * Omega0 * A * dx) * dtdx + shear * dBz * dtdz;
    sC0 = sC0 - shear * dCy * dtdy;
  }
  sAL0 = +(GLR - GLL) * dtdy * HALF - (FLR - FLL) * dtdz * HALF;
  sAR0 = +(GRR - GRL) * dtdy * HALF - (FRR - FRL) * dtdz * HALF;
  sBL0 = -(GRL - GLL) * dtdx * HALF + (ELR - ELL) * dtdz * HALF;
  sBR0 = -(GRR - GLR) * dtdx * HALF + (ERR - ERL) * dtdz * HALF;
  sCL0 = +(FRL - FLL) * dtdx * HALF - (ERL - ELL) * dtdy * HALF;
  sCR0 = +(FRR - FLR) * dtdx * HALF - (ERR - ELR) * dtdy * HALF;

  r = r + sr0;
  u = u + su0;
  v = v + sv0;
  w = w + sw0;
  pp = pp + sp0;
  A = A + sA0;
  B = B + sB0;
  C = C + sC0;
  AL = AL + sAL0;
  AR = AR + sAR0;
  BL = BL + sBL0;
  BR = BR + sBR0;
  CL = CL + sCL0;
  CR = CR + sCR0;

#define SETQ(dst, R, U, V, W, P, AA, BB, CC)                                                        \
  do                                                                                                \
  {                                                                                                 \
    (dst)[EKO_ID] = (R);                                                                            \
    (dst)[EKO_IU] = (U);                                                                            \
    (dst)[EKO_IV] = (V);                                                                            \
    (dst)[EKO_IW] = (W);                                                                            \
    (dst)[EKO_IP] = (P);                                                                            \
    (dst)[EKO_IA] = (AA);                                                                           \
    (dst)[EKO_IB] = (BB);                                                                           \
    (dst)[EKO_IC] = (CC);                                                                           \
    (dst)[EKO_ID] = fmax(smallR, (dst)[EKO_ID]);                                                    \
    (dst)[EKO_IP] = fmax(smallp, (dst)[EKO_IP]);                                                    \
  } while (0)

  SETQ(qp[0], r - drx, u - dux, v - dvx, w - dwx, pp - dpx, AL, B - dBx, C - dCx);
  SETQ(qm[0], r + drx, u + dux, v + dvx, w + dwx, pp + dpx, AR, B + dBx, C + dCx);
  SETQ(qp[1], r - dry, u - duy, v - dvy, w - dwy, pp - dpy, A - dAy, BL, C - dCy);
  SETQ(qm[1], r + dry, u + duy, v + dvy, w + dwy, pp + dpy, A + dAy, BR, C + dCy);
  SETQ(qp[2], r - drz, u - duz, v - dvz, w - dwz, pp - dpz, A - dAz, B - dBz, CL);
  SETQ(qm[2], r + drz, u + duz, v + dvz, w + dwz, pp + dpz, A + dAz, B + dBz, CR);

  /* X edges */
  SETQ(qE[0][0], r + (+dry + drz), u + (+duy + duz), v + (+dvy + dvz), w + (+dwy + dwz),
       pp + (+dpy + dpz), A + (+dAy + dAz), BR + (+dBRz), CR + (+dCRy));
  SETQ(qE[1][0], r + (+dry - drz), u + (+duy - duz), v + (+dvy - dvz), w + (+dwy - dwz),
       pp + (+dpy - dpz), A + (+dAy - dAz), BR + (-dBRz), CL + (+dCLy));
  SETQ(qE[2][0], r + (-dry + drz), u + (-duy + duz), v + (-dvy + dvz), w + (-dwy + dwz),
       pp + (-dpy + dpz), A + (-dAy + dAz), BL + (+dBLz), CR + (-dCRy));
  SETQ(qE[3][0], r + (-dry - drz), u + (-duy - duz), v + (-dvy - dvz), w + (-dwy - dwz),
       pp + (-dpy - dpz), A + (-dAy - dAz), BL + (-dBLz), CL + (-dCLy));
  /* Y edges */
  SETQ(qE[0][1], r + (+drx + drz), u + (+dux + duz), v + (+dvx + dvz), w + (+dwx + dwz),
       pp + (+dpx + dpz), AR + (+dARz), B + (+dBx + dBz), CR + (+dCRx));
  SETQ(qE[1][1], r + (+drx - drz), u + (+dux - duz), v + (+dvx - dvz), w + (+dwx - dwz),
       pp + (+dpx - dpz), AR + (-dARz), B + (+dBx - dBz), CL + (+dCLx));
  SETQ(qE[2][1], r + (-drx + drz), u + (-dux + duz), v + (-dvx + dvz), w + (-dwx + dwz),
       pp + (-dpx + dpz), AL + (+dALz), B + (-dBx + dBz), CR + (-dCRx));
  SETQ(qE[3][1], r + (-drx - drz), u + (-dux - duz), v + (-dvx - dvz), w + (-dwx - dwz),
       pp + (-dpx - dpz), AL + (-dALz), B + (-dBx - dBz), CL + (-dCLx));
  /* Z edges */
  SETQ(qE[0][2], r + (+drx + dry), u + (+dux + duy), v + (+dvx + dvy), w + (+dwx + dwy),
       pp + (+dpx + dpy), AR + (+dARy), BR + (+dBRx), C + (+dCx + dCy));
  SETQ(qE[1][2], r + (+drx - dry), u + (+dux - duy), v + (+dvx - dvy), w + (+dwx - dwy),
       pp + (+dpx - dpy), AR + (-dARy), BL + (+dBLx), C + (+dCx - dCy));
  SETQ(qE[2][2], r + (-drx + dry), u + (-dux + duy), v + (-dvx + dvy), w + (-dwx + dwy),
       pp + (-dpx + dpy), AL + (+dALy), BR + (-dBRx), C + (-dCx + dCy));
  SETQ(qE[3][2], r + (-drx - dry), u + (-dux - duy), v + (-dvx - dvy), w + (-dwx - dwy),
       pp + (-dpx - dpy), AL + (-dALy), BL + (-dBLx), C + (-dCx - dCy));
#undef SETQ
}

/* ConvertToPrimitivesFunctor3D_MHD: MHDRunFunctors3D.h:88-163 (i,j,k < size-1) */
static void
mhd_convert_prims(eko_solver * s, const double * U)
{
  const eko_params * p = &s->p;
  const int is = p->isize, js = p->jsize, ks = p->ksize;
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 0; k < ks - 1; ++k)
    for (int j = 0; j < js - 1; ++j)
      for (int i = 0; i < is - 1; ++i)
      {
        long   c = IDX(s, i, j, k);
        double u[8], q[8], bnb[3];
        for (int v = 0; v < 8; ++v)
          u[v] = AT(U, s, v, c);
        bnb[0] = AT(U, s, EKO_IA, c + 1);
        bnb[1] = AT(U, s, EKO_IB, c + is);
        bnb[2] = AT(U, s, EKO_IC, c + (long)is * js);
        mhd_constoprim(u, bnb, q, p);
        for (int v = 0; v < 8; ++v)
          AT(s->Q, s, v, c) = q[v];
      }
}

/* ComputeDtFunctor3D_MHD: MHDRunFunctors3D.h:16-83 (on Q) */
static double
mhd_compute_dt_local(eko_solver * s)
{
  const eko_params * p = &s->p;
  const int gw = p->gw;
  double    invDt = -DBL_MAX;
#pragma omp parallel
  {
    double local = -DBL_MAX;
#pragma omp for collapse(2) schedule(static)
    for (int k = gw; k < p->ksize - gw; ++k)
      for (int j = gw; j < p->jsize - gw; ++j)
        for (int i = gw; i < p->isize - gw; ++i)
        {
          long   c = IDX(s, i, j, k);
          double q[8], f[3];
          for (int v = 0; v < 8; ++v)
            q[v] = AT(s->Q, s, v, c);
          speed_info3(q, f, p->gamma0);
          local = fmax(local, f[0] / p->dx + f[1] / p->dy + f[2] / p->dz);
        }
#pragma omp critical
    invDt = local > invDt ? local : invDt;
  }
  return p->cfl / invDt;
}

/* godunov_unsplit_impl v0 for MHD 3D: SolverMHDMuscl.cpp:461-505 */
static void
mhd3d_godunov(eko_solver * s, double * in, double * out)
{
  const eko_params * p = &s->p;
  const int is = p->isize, js = p->jsize, ks = p->ksize, gw = p->gw;
  const long sy = is, sz = (long)is * js;
  const long ncell = s->ncell;

  make_boundaries(s, in);
  memcpy(out, in, sizeof(double) * ncell * 8);
  mhd_convert_prims(s, in);

  /* compute_dt() after the primitives (SolverMHDMuscl.cpp:479-484) */
  s->dt = mhd_compute_dt_local(s);
  if (s->t + s->dt > p->tEnd)
    s->dt = p->tEnd - s->t;
  const double dt = s->dt;
  const double dtdx = dt / p->dx, dtdy = dt / p->dy, dtdz = dt / p->dz;

  /* ComputeElecFieldFunctor3D: MHDRunFunctors3D.h:278-362 */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k < ks - 1; ++k)
    for (int j = 1; j < js - 1; ++j)
      for (int i = 1; i < is - 1; ++i)
      {
        long   c = IDX(s, i, j, k);
        const double * Q = s->Q;
        double u, v, w, A, B, C;
        v = 0.25 * (AT(Q, s, EKO_IV, c - sy - sz) + AT(Q, s, EKO_IV, c - sy) +
                    AT(Q, s, EKO_IV, c - sz) + AT(Q, s, EKO_IV, c));
        w = 0.25 * (AT(Q, s, EKO_IW, c - sy - sz) + AT(Q, s, EKO_IW, c - sy) +
                    AT(Q, s, EKO_IW, c - sz) + AT(Q, s, EKO_IW, c));
        B = HALF * (AT(in, s, EKO_IB, c - sz) + AT(in, s, EKO_IB, c));
        C = HALF * (AT(in, s, EKO_IC, c - sy) + AT(in, s, EKO_IC, c));
        AT(s->E, s, 0, c) = v * C - w * B;
        u = 0.25 * (AT(Q, s, EKO_IU, c - 1 - sz) + AT(Q, s, EKO_IU, c - 1) +
                    AT(Q, s, EKO_IU, c - sz) + AT(Q, s, EKO_IU, c));
        w = 0.25 * (AT(Q, s, EKO_IW, c - 1 - sz) + AT(Q, s, EKO_IW, c - 1) +
                    AT(Q, s, EKO_IW, c - sz) + AT(Q, s, EKO_IW, c));
        A = HALF * (AT(in, s, EKO_IA, c - sz) + AT(in, s, EKO_IA, c));
        C = HALF * (AT(in, s, EKO_IC, c - 1) + AT(in, s, EKO_IC, c));
        AT(s->E, s, 1, c) = w * A - u * C;
        u = 0.25 * (AT(Q, s, EKO_IU, c - 1 - sy) + AT(Q, s, EKO_IU, c - 1) +
                    AT(Q, s, EKO_IU, c - sy) + AT(Q, s, EKO_IU, c));
        v = 0.25 * (AT(Q, s, EKO_IV, c - 1 - sy) + AT(Q, s, EKO_IV, c - 1) +
                    AT(Q, s, EKO_IV, c - sy) + AT(Q, s, EKO_IV, c));
        A = HALF * (AT(in, s, EKO_IA, c - sy) + AT(in, s, EKO_IA, c));
        B = HALF * (AT(in, s, EKO_IB, c - 1) + AT(in, s, EKO_IB, c));
        AT(s->E, s, 2, c) = u * B - v * A;
      }

  /* ComputeMagSlopesFunctor3D + slope_unsplit_mhd_3d: MHDRunFunctors3D.h:441-538,
   * MHDBaseFunctor3D.h:563-668 */
  const double xst = fmin(p->slope_type, 2.0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k < ks - 1; ++k)
    for (int j = 1; j < js - 1; ++j)
      for (int i = 1; i < is - 1; ++i)
      {
        long   c = IDX(s, i, j, k);
        double bfx = AT(in, s, EKO_IA, c), bfy = AT(in, s, EKO_IB, c), bfz = AT(in, s, EKO_IC, c);
        /* DeltaA = (dbfX[IX], dbfY[IX], dbfZ[IX]) with dbfX[IX] = 0 */
        AT(s->dA, s, 0, c) = 0.0;
        AT(s->dA, s, 1, c) = slope1(bfx, AT(in, s, EKO_IA, c + sy), AT(in, s, EKO_IA, c - sy), xst);
        AT(s->dA, s, 2, c) = slope1(bfx, AT(in, s, EKO_IA, c + sz), AT(in, s, EKO_IA, c - sz), xst);
        AT(s->dB, s, 0, c) = slope1(bfy, AT(in, s, EKO_IB, c + 1), AT(in, s, EKO_IB, c - 1), xst);
        AT(s->dB, s, 1, c) = 0.0;
        AT(s->dB, s, 2, c) = slope1(bfy, AT(in, s, EKO_IB, c + sz), AT(in, s, EKO_IB, c - sz), xst);
        AT(s->dC, s, 0, c) = slope1(bfz, AT(in, s, EKO_IC, c + 1), AT(in, s, EKO_IC, c - 1), xst);
        AT(s->dC, s, 1, c) = slope1(bfz, AT(in, s, EKO_IC, c + sy), AT(in, s, EKO_IC, c - sy), xst);
        AT(s->dC, s, 2, c) = 0.0;
      }

  /* ComputeTraceFunctor3D_MHD: MHDRunFunctors3D.h:543-856.  The reference
   * range is [gw-2, size-gw+1); only [gw-1, size-gw] is consumed by the
   * flux and emf functors, so that is the range computed here. */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = gw - 1; k <= ks - gw; ++k)
    for (int j = gw - 1; j <= js - gw; ++j)
      for (int i = gw - 1; i <= is - gw; ++i)
      {
        long   c = IDX(s, i, j, k);
        double q[8], qpx[8], qmx[8], qpy[8], qmy[8], qpz[8], qmz[8], dq[3][8];
        const double * Q = s->Q;
        for (int v = 0; v < 8; ++v)
        {
          q[v] = AT(Q, s, v, c);
          qpx[v] = AT(Q, s, v, c + 1);
          qmx[v] = AT(Q, s, v, c - 1);
          qpy[v] = AT(Q, s, v, c + sy);
          qmy[v] = AT(Q, s, v, c - sy);
          qpz[v] = AT(Q, s, v, c + sz);
          qmz[v] = AT(Q, s, v, c - sz);
        }
        /* slope_unsplit_hydro_3d (MHDBaseFunctor3D.h:340-470) incl. its
         * z-slope of IC taken with qMinusY[IC] */
        if (p->slope_type == 1 || p->slope_type == 2)
        {
          for (int v = 0; v < 8; ++v)
          {
            dq[0][v] = slope1(q[v], qpx[v], qmx[v], p->slope_type);
            dq[1][v] = slope1(q[v], qpy[v], qmy[v], p->slope_type);
            dq[2][v] = slope1(q[v], qpz[v], (v == EKO_IC) ? qmy[v] : qmz[v], p->slope_type);
          }
        }
        else
        {
          for (int v = 0; v < 8; ++v)
            dq[0][v] = dq[1][v] = dq[2][v] = 0.0;
        }
        double bfNb[6], dbf[12], elec[3][2][2];
        bfNb[0] = AT(in, s, EKO_IA, c);
        bfNb[1] = AT(in, s, EKO_IA, c + 1);
        bfNb[2] = AT(in, s, EKO_IB, c);
        bfNb[3] = AT(in, s, EKO_IB, c + sy);
        bfNb[4] = AT(in, s, EKO_IC, c);
        bfNb[5] = AT(in, s, EKO_IC, c + sz);
        dbf[0] = AT(s->dA, s, 1, c);
        dbf[1] = AT(s->dA, s, 2, c);
        dbf[2] = AT(s->dB, s, 0, c);
        dbf[3] = AT(s->dB, s, 2, c);
        dbf[4] = AT(s->dC, s, 0, c);
        dbf[5] = AT(s->dC, s, 1, c);
        dbf[6] = AT(s->dA, s, 1, c + 1);
        dbf[7] = AT(s->dA, s, 2, c + 1);
        dbf[8] = AT(s->dB, s, 0, c + sy);
        dbf[9] = AT(s->dB, s, 2, c + sy);
        dbf[10] = AT(s->dC, s, 0, c + sz);
        dbf[11] = AT(s->dC, s, 1, c + sz);
        elec[0][0][0] = AT(s->E, s, 0, c);
        elec[0][0][1] = AT(s->E, s, 0, c + sz);
        elec[0][1][0] = AT(s->E, s, 0, c + sy);
        elec[0][1][1] = AT(s->E, s, 0, c + sy + sz);
        elec[1][0][0] = AT(s->E, s, 1, c);
        elec[1][0][1] = AT(s->E, s, 1, c + sz);
        elec[1][1][0] = AT(s->E, s, 1, c + 1);
        elec[1][1][1] = AT(s->E, s, 1, c + 1 + sz);
        elec[2][0][0] = AT(s->E, s, 2, c);
        elec[2][0][1] = AT(s->E, s, 2, c + sy);
        elec[2][1][0] = AT(s->E, s, 2, c + 1);
        elec[2][1][1] = AT(s->E, s, 2, c + 1 + sy);
        double xPos = p->xmin + p->dx / 2 + (i - gw) * p->dx;
        double qm[3][8], qp[3][8], qE[4][3][8];
        mhd_trace3d(q, dq, bfNb, dbf, elec, dtdx, dtdy, dtdz, xPos, qm, qp, qE, p);
        for (int v = 0; v < 8; ++v)
        {
          for (int d = 0; d < 3; ++d)
          {
            AT(s->Qm[d], s, v, c) = qm[d][v];
            AT(s->Qp[d], s, v, c) = qp[d][v];
            for (int e = 0; e < 4; ++e)
              AT(s->QE[e][d], s, v, c) = qE[e][d][v];
          }
        }
      }

  /* ComputeFluxesAndStoreFunctor3D_MHD (MHDRunFunctors3D.h:1783-1909) and
   * ComputeEmfAndStoreFunctor3D (MHDRunFunctors3D.h:2100-2238), range
   * [gw, size-gw] in every direction */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = gw; k <= ks - gw; ++k)
    for (int j = gw; j <= js - gw; ++j)
      for (int i = gw; i <= is - gw; ++i)
      {
        long   c = IDX(s, i, j, k);
        double ql[8], qr[8], fl[8];
        /* x */
        for (int v = 0; v < 8; ++v)
        {
          ql[v] = AT(s->Qm[0], s, v, c - 1);
          qr[v] = AT(s->Qp[0], s, v, c);
        }
        riemann_mhd(ql, qr, fl, p);
        for (int v = 0; v < 8; ++v)
          AT(s->Fx, s, v, c) = fl[v];
        /* y: swap IU<->IV and IA<->IB */
        for (int v = 0; v < 8; ++v)
        {
          ql[v] = AT(s->Qm[1], s, v, c - sy);
          qr[v] = AT(s->Qp[1], s, v, c);
        }
        swapd(&ql[EKO_IU], &ql[EKO_IV]);
        swapd(&ql[EKO_IA], &ql[EKO_IB]);
        swapd(&qr[EKO_IU], &qr[EKO_IV]);
        swapd(&qr[EKO_IA], &qr[EKO_IB]);
        riemann_mhd(ql, qr, fl, p);
        for (int v = 0; v < 8; ++v)
          AT(s->Fy, s, v, c) = fl[v];
        /* z: swap IU<->IW and IA<->IC */
        for (int v = 0; v < 8; ++v)
        {
          ql[v] = AT(s->Qm[2], s, v, c - sz);
          qr[v] = AT(s->Qp[2], s, v, c);
        }
        swapd(&ql[EKO_IU], &ql[EKO_IW]);
        swapd(&ql[EKO_IA], &ql[EKO_IC]);
        swapd(&qr[EKO_IU], &qr[EKO_IW]);
        swapd(&qr[EKO_IA], &qr[EKO_IC]);
        riemann_mhd(ql, qr, fl, p);
        for (int v = 0; v < 8; ++v)
          AT(s->Fz, s, v, c) = fl[v];

        /* emfs.  QE index [0 RT,1 RB,2 LT,3 LB][dir] */
        double a[8], b[8], cc[8], d[8];
        for (int v = 0; v < 8; ++v)
        {
          a[v] = AT(s->QE[0][2], s, v, c - 1 - sy);
          b[v] = AT(s->QE[1][2], s, v, c - 1);
          cc[v] = AT(s->QE[2][2], s, v, c - sy);
          d[v] = AT(s->QE[3][2], s, v, c);
        }
        AT(s->Emf, s, 0, c) = compute_emf(a, b, cc, d, 2, p);
        /* EMFY: RT <- RT2(i-1,k-1), RB <- LT2(i,k-1), LT <- RB2(i-1,k), LB <- LB2(i,k) */
        for (int v = 0; v < 8; ++v)
        {
          a[v] = AT(s->QE[0][1], s, v, c - 1 - sz);
          b[v] = AT(s->QE[2][1], s, v, c - sz);
          cc[v] = AT(s->QE[1][1], s, v, c - 1);
          d[v] = AT(s->QE[3][1], s, v, c);
        }
        AT(s->Emf, s, 1, c) = compute_emf(a, b, cc, d, 1, p);
        for (int v = 0; v < 8; ++v)
        {
          a[v] = AT(s->QE[0][0], s, v, c - sy - sz);
          b[v] = AT(s->QE[1][0], s, v, c - sy);
          cc[v] = AT(s->QE[2][0], s, v, c - sz);
          d[v] = AT(s->QE[3][0], s, v, c);
        }
        AT(s->Emf, s, 2, c) = compute_emf(a, b, cc, d, 0, p);
      }

  /* UpdateFunctor3D_MHD (MHDRunFunctors3D.h:2430-2544) then UpdateEmfFunctor3D
   * (MHDRunFunctors3D.h:2549-2628) */
#pragma omp parallel for collapse(2) schedule(static)
  for (int k = gw; k < ks - gw; ++k)
    for (int j = gw; j < js - gw; ++j)
      for (int i = gw; i < is - gw; ++i)
      {
        long   c = IDX(s, i, j, k);
        double ud[8];
        for (int v = 0; v < 8; ++v)
          ud[v] = AT(out, s, v, c);
        const double *Fx = s->Fx, *Fy = s->Fy, *Fz = s->Fz;
        ud[EKO_ID] += AT(Fx, s, EKO_ID, c) * dtdx;
        ud[EKO_IP] += AT(Fx, s, EKO_IP, c) * dtdx;
        ud[EKO_IU] += AT(Fx, s, EKO_IU, c) * dtdx;
        ud[EKO_IV] += AT(Fx, s, EKO_IV, c) * dtdx;
        ud[EKO_IW] += AT(Fx, s, EKO_IW, c) * dtdx;
        ud[EKO_ID] -= AT(Fx, s, EKO_ID, c + 1) * dtdx;
        ud[EKO_IP] -= AT(Fx, s, EKO_IP, c + 1) * dtdx;
        ud[EKO_IU] -= AT(Fx, s, EKO_IU, c + 1) * dtdx;
        ud[EKO_IV] -= AT(Fx, s, EKO_IV, c + 1) * dtdx;
        ud[EKO_IW] -= AT(Fx, s, EKO_IW, c + 1) * dtdx;

        ud[EKO_ID] += AT(Fy, s, EKO_ID, c) * dtdy;
        ud[EKO_IP] += AT(Fy, s, EKO_IP, c) * dtdy;
        ud[EKO_IU] += AT(Fy, s, EKO_IV, c) * dtdy;
        ud[EKO_IV] += AT(Fy, s, EKO_IU, c) * dtdy;
        ud[EKO_IW] += AT(Fy, s, EKO_IW, c) * dtdy;
        ud[EKO_ID] -= AT(Fy, s, EKO_ID, c + sy) * dtdy;
        ud[EKO_IP] -= AT(Fy, s, EKO_IP, c + sy) * dtdy;
        ud[EKO_IU] -= AT(Fy, s, EKO_IV, c + sy) * dtdy;
        ud[EKO_IV] -= AT(Fy, s, EKO_IU, c + sy) * dtdy;
        ud[EKO_IW] -= AT(Fy, s, EKO_IW, c + sy) * dtdy;

        ud[EKO_ID] += AT(Fz, s, EKO_ID, c) * dtdz;
        ud[EKO_IP] += AT(Fz, s, EKO_IP, c) * dtdz;
        ud[EKO_IU] += AT(Fz, s, EKO_IW, c) * dtdz;
        ud[EKO_IV] += AT(Fz, s, EKO_IV, c) * dtdz;
        ud[EKO_IW] += AT(Fz, s, EKO_IU, c) * dtdz;
        ud[EKO_ID] -= AT(Fz, s, EKO_ID, c + sz) * dtdz;
        ud[EKO_IP] -= AT(Fz, s, EKO_IP, c + sz) * dtdz;
        ud[EKO_IU] -= AT(Fz, s, EKO_IW, c + sz) * dtdz;
        ud[EKO_IV] -= AT(Fz, s, EKO_IV, c + sz) * dtdz;
        ud[EKO_IW] -= AT(Fz, s, EKO_IU, c + sz) * dtdz;

        const double * Emf = s->Emf;
        ud[EKO_IA] += (AT(Emf, s, 0, c + sy) - AT(Emf, s, 0, c)) * dtdy;
        ud[EKO_IB] -= (AT(Emf, s, 0, c + 1) - AT(Emf, s, 0, c)) * dtdx;
        ud[EKO_IA] -= (AT(Emf, s, 1, c + sz) - AT(Emf, s, 1, c)) * dtdz;
        ud[EKO_IB] += (AT(Emf, s, 2, c + sz) - AT(Emf, s, 2, c)) * dtdz;
        ud[EKO_IC] += (AT(Emf, s, 1, c + 1) - AT(Emf, s, 1, c)) * dtdx;
        ud[EKO_IC] -= (AT(Emf, s, 2, c + sy) - AT(Emf, s, 2, c)) * dtdy;
        for (int v = 0; v < 8; ++v)
          AT(out, s, v, c) = ud[v];
      }
}

/* ===================================================================== */
/* MHD 2D                                                                 */
/* ===================================================================== */

/* ConvertToPrimitivesFunctor2D_MHD: MHDRunFunctors2D.h:85-160 (i,j < size-1).
 * The z neighbour field is 0 (MHDRunFunctors2D.h:133), so the cell-centred Bz
 * is half the stored value. */
static void
mhd2d_convert_prims(eko_solver * s, const double * U)
{
  const eko_params * p = &s->p;
  const int is = p->isize, js = p->jsize;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < js - 1; ++j)
    for (int i = 0; i < is - 1; ++i)
    {
      long   c = IDX(s, i, j, 0);
      double u[8], q[8], bnb[3];
      for (int v = 0; v < 8; ++v)
        u[v] = AT(U, s, v, c);
      bnb[0] = AT(U, s, EKO_IA, c + 1);
      bnb[1] = AT(U, s, EKO_IB, c + is);
      bnb[2] = 0.0;
      mhd_constoprim(u, bnb, q, p);
      for (int v = 0; v < 8; ++v)
        AT(s->Q, s, v, c) = q[v];
    }
}

/* ComputeDtFunctor2D_MHD: MHDRunFunctors2D.h:16-80, find_speed_info<TWO_D>
 * (mhd_utils.h:319-366) */
static double
mhd2d_compute_dt_local(eko_solver * s)
{
  const eko_params * p = &s->p;
  const int gw = p->gw;
  double    invDt = -DBL_MAX;
#pragma omp parallel
  {
    double local = -DBL_MAX;
#pragma omp for schedule(static)
    for (int j = gw; j < p->jsize - gw; ++j)
      for (int i = gw; i < p->isize - gw; ++i)
      {
        long   c = IDX(s, i, j, 0);
        double q[8], f[3];
        for (int v = 0; v < 8; ++v)
          q[v] = AT(s->Q, s, v, c);
        speed_info3(q, f, p->gamma0);
        local = fmax(local, f[0] / p->dx + f[1] / p->dy);
      }
#pragma omp critical
    invDt = local > invDt ? local : invDt;
  }
  return p->cfl / invDt;
}

/* slope_unsplit_mhd_2d: MHDBaseFunctor2D.h:455-518.  bfn = bfx, bfx_yplus,
 * bfx_yminus, bfy, bfy_xplus, bfy_xminus; returns dbfY[IX] and dbfX[IY]. */
static void
mhd2d_bslopes(const double * bfn, double st, double * dbfy_x, double * dbfx_y)
{
  *dbfy_x = slope1(bfn[0], bfn[1], bfn[2], st);
  *dbfx_y = slope1(bfn[3], bfn[4], bfn[5], st);
}

/* trace_unsplit_mhd_2d: MHDBaseFunctor2D.h:775-1114.  qNb: primitive states
 * of the 3x3 neighbourhood, bfNb: face fields of the 4x4 neighbourhood (the
 * cell at [1][1]); qE in the order RT, RB, LT, LB. */
static void
mhd_trace2d(double qNb[3][3][8], double bfNb[4][4][3], double dtdx, double dtdy, double qm[2][8],
            double qp[2][8], double qE[4][8], const eko_params * p)
{
  const double smallR = p->smallr, smallp = p->smallp, gamma = p->gamma0, st = p->slope_type;
  double       Ez[2][2];
  for (int di = 0; di < 2; di++)
    for (int dj = 0; dj < 2; dj++)
    {
      int    cx = 1 + di, cy = 1 + dj;
      double u = 0.25 * (qNb[cx - 1][cy - 1][EKO_IU] + qNb[cx - 1][cy][EKO_IU] + qNb[cx][cy - 1][EKO_IU] +
                         qNb[cx][cy][EKO_IU]);
      double v = 0.25 * (qNb[cx - 1][cy - 1][EKO_IV] + qNb[cx - 1][cy][EKO_IV] + qNb[cx][cy - 1][EKO_IV] +
                         qNb[cx][cy][EKO_IV]);
      double A = 0.5 * (bfNb[cx][cy - 1][0] + bfNb[cx][cy][0]);
      double B = 0.5 * (bfNb[cx - 1][cy][1] + bfNb[cx][cy][1]);
      Ez[di][dj] = u * B - v * A;
    }
  const double ELL = Ez[0][0], ELR = Ez[0][1], ERL = Ez[1][0], ERR = Ez[1][1];
  const double * q = qNb[1][1];
  double r = q[EKO_ID], pp = q[EKO_IP], u = q[EKO_IU], v = q[EKO_IV], w = q[EKO_IW], A = q[EKO_IA],
         B = q[EKO_IB], C = q[EKO_IC];
  double AL = bfNb[1][1][0], AR = bfNb[2][1][0], BL = bfNb[1][1][1], BR = bfNb[1][2][1];

  /* slope_unsplit_hydro_2d (MHDBaseFunctor2D.h:346-404), slope_type 1 or 2 */
  double dq[2][8];
  for (int var = 0; var < 8; ++var)
  {
    dq[0][var] = slope1(q[var], qNb[2][1][var], qNb[0][1][var], st);
    dq[1][var] = slope1(q[var], qNb[1][2][var], qNb[1][0][var], st);
  }
  double drx = dq[0][EKO_ID] * 0.5, dpx = dq[0][EKO_IP] * 0.5, dux = dq[0][EKO_IU] * 0.5,
         dvx = dq[0][EKO_IV] * 0.5, dwx = dq[0][EKO_IW] * 0.5, dCx = dq[0][EKO_IC] * 0.5,
         dBx = dq[0][EKO_IB] * 0.5;
  double dry = dq[1][EKO_ID] * 0.5, dpy = dq[1][EKO_IP] * 0.5, duy = dq[1][EKO_IU] * 0.5,
         dvy = dq[1][EKO_IV] * 0.5, dwy = dq[1][EKO_IW] * 0.5, dCy = dq[1][EKO_IC] * 0.5,
         dAy = dq[1][EKO_IA] * 0.5;

  double bfn[6], dbfy_x, dbfx_y;
  bfn[0] = bfNb[1][1][0], bfn[1] = bfNb[1][2][0], bfn[2] = bfNb[1][0][0];
  bfn[3] = bfNb[1][1][1], bfn[4] = bfNb[2][1][1], bfn[5] = bfNb[0][1][1];
  mhd2d_bslopes(bfn, st, &dbfy_x, &dbfx_y);
  const double dALy = 0.5 * dbfy_x, dBLx = 0.5 * dbfx_y;
  bfn[0] = bfNb[2][1][0], bfn[1] = bfNb[2][2][0], bfn[2] = bfNb[2][0][0];
  bfn[3] = bfNb[2][1][1], bfn[4] = bfNb[3][1][1], bfn[5] = bfNb[1][1][1];
  mhd2d_bslopes(bfn, st, &dbfy_x, &dbfx_y);
  const double dARy = 0.5 * dbfy_x;
  bfn[0] = bfNb[1][2][0], bfn[1] = bfNb[1][3][0], bfn[2] = bfNb[1][1][0];
  bfn[3] = bfNb[1][2][1], bfn[4] = bfNb[2][2][1], bfn[5] = bfNb[0][2][1];
  mhd2d_bslopes(bfn, st, &dbfy_x, &dbfx_y);
  const double dBRx = 0.5 * dbfx_y;

  const double dAx = 0.5 * (AR - AL);
  const double dBy = 0.5 * (BR - BL);

  /* source terms (cartesian), MHDBaseFunctor2D.h:969-995 */
  const double sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
  const double su0 =
    (-u * dux - dpx / r - B * dBx / r - C * dCx / r) * dtdx + (-v * duy + B * dAy / r) * dtdy;
  const double sv0 =
    (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - C * dCy / r) * dtdy;
  const double sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy;
  const double sp0 = (-u * dpx - dux * gamma * pp) * dtdx + (-v * dpy - dvy * gamma * pp) * dtdy;
  const double sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy;
  const double sB0 = (-u * dBx - B * dux + v * dAx + A * dvx) * dtdx;
  const double sC0 =
    (w * dAx + A * dwx - u * dCx - C * dux) * dtdx + (-v * dCy - C * dvy + w * dBy + B * dwy) * dtdy;
  const double sAL0 = +(ELR - ELL) * 0.5 * dtdy;
  const double sAR0 = +(ERR - ERL) * 0.5 * dtdy;
  const double sBL0 = -(ERL - ELL) * 0.5 * dtdx;
  const double sBR0 = -(ERR - ELR) * 0.5 * dtdx;

  r = r + sr0;
  u = u + su0;
  v = v + sv0;
  w = w + sw0;
  pp = pp + sp0;
  A = A + sA0;
  B = B + sB0;
  C = C + sC0;
  AL = AL + sAL0;
  AR = AR + sAR0;
  BL = BL + sBL0;
  BR = BR + sBR0;

#define EKO_FLOOR2(st_)                                                                            \
  do                                                                                               \
  {                                                                                                \
    (st_)[EKO_ID] = fmax(smallR, (st_)[EKO_ID]);                                                   \
    (st_)[EKO_IP] = fmax(smallp * (st_)[EKO_ID], (st_)[EKO_IP]);                                   \
  } while (0)
  qp[0][EKO_ID] = r - drx, qp[0][EKO_IU] = u - dux, qp[0][EKO_IV] = v - dvx, qp[0][EKO_IW] = w - dwx;
  qp[0][EKO_IP] = pp - dpx, qp[0][EKO_IA] = AL, qp[0][EKO_IB] = B - dBx, qp[0][EKO_IC] = C - dCx;
  EKO_FLOOR2(qp[0]);
  qm[0][EKO_ID] = r + drx, qm[0][EKO_IU] = u + dux, qm[0][EKO_IV] = v + dvx, qm[0][EKO_IW] = w + dwx;
  qm[0][EKO_IP] = pp + dpx, qm[0][EKO_IA] = AR, qm[0][EKO_IB] = B + dBx, qm[0][EKO_IC] = C + dCx;
  EKO_FLOOR2(qm[0]);
  qp[1][EKO_ID] = r - dry, qp[1][EKO_IU] = u - duy, qp[1][EKO_IV] = v - dvy, qp[1][EKO_IW] = w - dwy;
  qp[1][EKO_IP] = pp - dpy, qp[1][EKO_IA] = A - dAy, qp[1][EKO_IB] = BL, qp[1][EKO_IC] = C - dCy;
  EKO_FLOOR2(qp[1]);
  qm[1][EKO_ID] = r + dry, qm[1][EKO_IU] = u + duy, qm[1][EKO_IV] = v + dvy, qm[1][EKO_IW] = w + dwy;
  qm[1][EKO_IP] = pp + dpy, qm[1][EKO_IA] = A + dAy, qm[1][EKO_IB] = BR, qm[1][EKO_IC] = C + dCy;
  EKO_FLOOR2(qm[1]);

  double * qRT = qE[0];
  double * qRB = qE[1];
  double * qLT = qE[2];
  double * qLB = qE[3];
  qRT[EKO_ID] = r + (+drx + dry), qRT[EKO_IU] = u + (+dux + duy), qRT[EKO_IV] = v + (+dvx + dvy);
  qRT[EKO_IW] = w + (+dwx + dwy), qRT[EKO_IP] = pp + (+dpx + dpy), qRT[EKO_IA] = AR + (+dARy);
  qRT[EKO_IB] = BR + (+dBRx), qRT[EKO_IC] = C + (+dCx + dCy);
  EKO_FLOOR2(qRT);
  qRB[EKO_ID] = r + (+drx - dry), qRB[EKO_IU] = u + (+dux - duy), qRB[EKO_IV] = v + (+dvx - dvy);
  qRB[EKO_IW] = w + (+dwx - dwy), qRB[EKO_IP] = pp + (+dpx - dpy), qRB[EKO_IA] = AR + (-dARy);
  qRB[EKO_IB] = BL + (+dBLx), qRB[EKO_IC] = C + (+dCx - dCy);
  EKO_FLOOR2(qRB);
  qLB[EKO_ID] = r + (-drx - dry), qLB[EKO_IU] = u + (-dux - duy), qLB[EKO_IV] = v + (-dvx - dvy);
  qLB[EKO_IW] = w + (-dwx - dwy), qLB[EKO_IP] = pp + (-dpx - dpy), qLB[EKO_IA] = AL + (-dALy);
  qLB[EKO_IB] = BL + (-dBLx), qLB[EKO_IC] = C + (-dCx - dCy);
  EKO_FLOOR2(qLB);
  qLT[EKO_ID] = r + (-drx + dry), qLT[EKO_IU] = u + (-dux + duy), qLT[EKO_IV] = v + (-dvx + dvy);
  qLT[EKO_IW] = w + (-dwx + dwy), qLT[EKO_IP] = pp + (-dpx + dpy), qLT[EKO_IA] = AL + (+dALy);
  qLT[EKO_IB] = BR + (-dBRx), qLT[EKO_IC] = C + (-dCx + dCy);
  EKO_FLOOR2(qLT);
#undef EKO_FLOOR2
}

/* godunov_unsplit_impl v0 for MHD 2D: SolverMHDMuscl.cpp:369-420 */
static void
mhd2d_godunov(eko_solver * s, double * in, double * out)
{
  const eko_params * p = &s->p;
  const int is = p->isize, js = p->jsize, gw = p->gw;
  const long sy = is;
  const long ncell = s->ncell;

  make_boundaries(s, in);
  memcpy(out, in, sizeof(double) * ncell * 8);
  mhd2d_convert_prims(s, in);
  s->dt = mhd2d_compute_dt_local(s);
  if (s->t + s->dt > p->tEnd)
    s->dt = p->tEnd - s->t;
  const double dt = s->dt;
  const double dtdx = dt / p->dx, dtdy = dt / p->dy;

  /* ComputeTraceFunctor2D_MHD: MHDRunFunctors2D.h:782-918 */
#pragma omp parallel for schedule(static)
  for (int j = gw - 2; j < js - gw + 1; ++j)
    for (int i = gw - 2; i < is - gw + 1; ++i)
    {
      double qNb[3][3][8], bfNb[4][4][3], qm[2][8], qp[2][8], qE[4][8];
      for (int di = 0; di < 3; ++di)
        for (int dj = 0; dj < 3; ++dj)
        {
          long c = IDX(s, i + di - 1, j + dj - 1, 0);
          for (int v = 0; v < 8; ++v)
            qNb[di][dj][v] = AT(s->Q, s, v, c);
        }
      for (int di = 0; di < 4; ++di)
        for (int dj = 0; dj < 4; ++dj)
        {
          long c = IDX(s, i + di - 1, j + dj - 1, 0);
          bfNb[di][dj][0] = AT(in, s, EKO_IA, c);
          bfNb[di][dj][1] = AT(in, s, EKO_IB, c);
          bfNb[di][dj][2] = AT(in, s, EKO_IC, c);
        }
      mhd_trace2d(qNb, bfNb, dtdx, dtdy, qm, qp, qE, p);
      long c = IDX(s, i, j, 0);
      for (int v = 0; v < 8; ++v)
      {
        AT(s->Qm[0], s, v, c) = qm[0][v];
        AT(s->Qp[0], s, v, c) = qp[0][v];
        AT(s->Qm[1], s, v, c) = qm[1][v];
        AT(s->Qp[1], s, v, c) = qp[1][v];
        for (int e = 0; e < 4; ++e)
          AT(s->QE[e][0], s, v, c) = qE[e][v];
      }
    }

  /* ComputeFluxesAndStoreFunctor2D_MHD (MHDRunFunctors2D.h:375-470) and
   * ComputeEmfAndStoreFunctor2D (MHDRunFunctors2D.h:612-686) */
#pragma omp parallel for schedule(static)
  for (int j = gw; j < js - gw + 1; ++j)
    for (int i = gw; i < is - gw + 1; ++i)
    {
      long   c = IDX(s, i, j, 0);
      double ql[8], qr[8], flux[8], x;
      for (int v = 0; v < 8; ++v)
      {
        ql[v] = AT(s->Qm[0], s, v, c - 1);
        qr[v] = AT(s->Qp[0], s, v, c);
      }
      riemann_mhd(ql, qr, flux, p);
      for (int v = 0; v < 8; ++v)
        AT(s->Fx, s, v, c) = flux[v];
      for (int v = 0; v < 8; ++v)
      {
        ql[v] = AT(s->Qm[1], s, v, c - sy);
        qr[v] = AT(s->Qp[1], s, v, c);
      }
      x = ql[EKO_IU], ql[EKO_IU] = ql[EKO_IV], ql[EKO_IV] = x;
      x = ql[EKO_IA], ql[EKO_IA] = ql[EKO_IB], ql[EKO_IB] = x;
      x = qr[EKO_IU], qr[EKO_IU] = qr[EKO_IV], qr[EKO_IV] = x;
      x = qr[EKO_IA], qr[EKO_IA] = qr[EKO_IB], qr[EKO_IB] = x;
      riemann_mhd(ql, qr, flux, p);
      for (int v = 0; v < 8; ++v)
        AT(s->Fy, s, v, c) = flux[v];

      double a[8], b[8], cc[8], d[8];
      for (int v = 0; v < 8; ++v)
      {
        a[v] = AT(s->QE[0][0], s, v, c - 1 - sy);
        b[v] = AT(s->QE[1][0], s, v, c - 1);
        cc[v] = AT(s->QE[2][0], s, v, c - sy);
        d[v] = AT(s->QE[3][0], s, v, c);
      }
      AT(s->Emf, s, 0, c) = compute_emf(a, b, cc, d, 2, p);
    }

  /* UpdateFunctor2D_MHD (MHDRunFunctors2D.h:1539-1641) then UpdateEmfFunctor2D
   * (MHDRunFunctors2D.h:1646-1700) */
#pragma omp parallel for schedule(static)
  for (int j = gw; j < js - gw; ++j)
    for (int i = gw; i < is - gw; ++i)
    {
      long           c = IDX(s, i, j, 0);
      const double * Fx = s->Fx;
      const double * Fy = s->Fy;
      double         ud[8];
      for (int v = 0; v < 8; ++v)
        ud[v] = AT(out, s, v, c);
      ud[EKO_ID] += AT(Fx, s, EKO_ID, c) * dtdx;
      ud[EKO_IP] += AT(Fx, s, EKO_IP, c) * dtdx;
      ud[EKO_IU] += AT(Fx, s, EKO_IU, c) * dtdx;
      ud[EKO_IV] += AT(Fx, s, EKO_IV, c) * dtdx;
      ud[EKO_IW] += AT(Fx, s, EKO_IW, c) * dtdx;
      ud[EKO_IC] += AT(Fx, s, EKO_IC, c) * dtdx;
      ud[EKO_ID] -= AT(Fx, s, EKO_ID, c + 1) * dtdx;
      ud[EKO_IP] -= AT(Fx, s, EKO_IP, c + 1) * dtdx;
      ud[EKO_IU] -= AT(Fx, s, EKO_IU, c + 1) * dtdx;
      ud[EKO_IV] -= AT(Fx, s, EKO_IV, c + 1) * dtdx;
      ud[EKO_IW] -= AT(Fx, s, EKO_IW, c + 1) * dtdx;
      ud[EKO_IC] -= AT(Fx, s, EKO_IC, c + 1) * dtdx;
      ud[EKO_ID] += AT(Fy, s, EKO_ID, c) * dtdy;
      ud[EKO_IP] += AT(Fy, s, EKO_IP, c) * dtdy;
      ud[EKO_IU] += AT(Fy, s, EKO_IV, c) * dtdy;
      ud[EKO_IV] += AT(Fy, s, EKO_IU, c) * dtdy;
      ud[EKO_IW] += AT(Fy, s, EKO_IW, c) * dtdy;
      ud[EKO_IC] += AT(Fy, s, EKO_IC, c) * dtdy;
      ud[EKO_ID] -= AT(Fy, s, EKO_ID, c + sy) * dtdy;
      ud[EKO_IP] -= AT(Fy, s, EKO_IP, c + sy) * dtdy;
      ud[EKO_IU] -= AT(Fy, s, EKO_IV, c + sy) * dtdy;
      ud[EKO_IV] -= AT(Fy, s, EKO_IU, c + sy) * dtdy;
      ud[EKO_IW] -= AT(Fy, s, EKO_IW, c + sy) * dtdy;
      ud[EKO_IC] -= AT(Fy, s, EKO_IC, c + sy) * dtdy;
      const double * Emf = s->Emf;
      ud[EKO_IA] += (AT(Emf, s, 0, c + sy) - AT(Emf, s, 0, c)) * dtdy;
      ud[EKO_IB] -= (AT(Emf, s, 0, c + 1) - AT(Emf, s, 0, c)) * dtdx;
      for (int v = 0; v < 8; ++v)
        AT(out, s, v, c) = ud[v];
    }
}

/* ===================================================================== */
/* driver                                                                 */
/* ===================================================================== */

static double *
zalloc(long n)
{
  return (double *)calloc((size_t)n, sizeof(double));
}

eko_solver *
eko_create(const eko_params * p, const double * U0, double t0)
{
  if (!p || !U0)
    return NULL;
  /* riemann_hydro (3D) has no HLL branch and riemann_mhd only HLLD/HLL/LLF:
   * the reference leaves the flux unset there (RiemannSolvers.h:608-640,
   * RiemannSolvers_MHD.h:368-389) */
  if (!p->mhd && p->dim == 3 && p->riemann == EKO_RIEMANN_HLL)
    return NULL;
  if (p->mhd && p->riemann != EKO_RIEMANN_HLLD && p->riemann != EKO_RIEMANN_HLL &&
      p->riemann != EKO_RIEMANN_LLF)
    return NULL;
  if (!p->mhd && p->riemann == EKO_RIEMANN_HLLD)
    return NULL;
  eko_solver * s = (eko_solver *)calloc(1, sizeof(eko_solver));
  s->p = *p;
  s->ncell = eko_ncells(p);
  const long n = s->ncell, nb = p->nbvar;
  s->U = zalloc(n * nb);
  s->U2 = zalloc(n * nb);
  s->Q = zalloc(n * nb);
  memcpy(s->U, U0, sizeof(double) * n * nb);
  if (!p->mhd && p->grav_enabled)
  {
    /* the field the Rayleigh-Taylor init writes on every cell (ghosts
     * included); zero for the other problems */
    s->G = zalloc(n * p->dim);
    for (int e = 0; e < p->dim; ++e)
      for (long c = 0; c < n; ++c)
        s->G[(long)e * n + c] = p->gravity[e];
  }
  if (!p->mhd)
  {
    s->Fx = zalloc(n * nb);
    s->Fy = zalloc(n * nb);
    s->Sx = zalloc(n * nb);
    s->Sy = zalloc(n * nb);
    if (p->dim == 3)
    {
      s->Fz = zalloc(n * nb);
      s->Sz = zalloc(n * nb);
    }
  }
  else
  {
    s->Fx = zalloc(n * 8);
    s->Fy = zalloc(n * 8);
    s->Fz = zalloc(n * 8);
    s->E = zalloc(n * 3);
    s->dA = zalloc(n * 3);
    s->dB = zalloc(n * 3);
    s->dC = zalloc(n * 3);
    s->Emf = zalloc(n * 3);
    for (int d = 0; d < 3; ++d)
    {
      s->Qm[d] = zalloc(n * 8);
      s->Qp[d] = zalloc(n * 8);
      for (int e = 0; e < 4; ++e)
        s->QE[e][d] = zalloc(n * 8);
    }
  }
  s->t = t0;
  s->iteration = 0;
  /* constructor tail */
  make_boundaries(s, s->U);
  memcpy(s->U2, s->U, sizeof(double) * n * nb);
  if (p->mhd && p->dim == 2)
  {
    mhd2d_convert_prims(s, s->U);
    s->dt = mhd2d_compute_dt_local(s);
  }
  else if (p->mhd)
  {
    mhd_convert_prims(s, s->U);
    s->dt = mhd_compute_dt_local(s);
  }
  else
    s->dt = hydro_compute_dt_local(s, s->U);
  if (s->t + s->dt > p->tEnd)
    s->dt = p->tEnd - s->t;
  return s;
}

void
eko_destroy(eko_solver * s)
{
  if (!s)
    return;
  free(s->U);
  free(s->U2);
  free(s->Q);
  free(s->Fx);
  free(s->Fy);
  free(s->Fz);
  free(s->Sx);
  free(s->Sy);
  free(s->Sz);
  free(s->E);
  free(s->dA);
  free(s->dB);
  free(s->dC);
  free(s->Emf);
  free(s->G);
  for (int d = 0; d < 3; ++d)
  {
    free(s->Qm[d]);
    free(s->Qp[d]);
    for (int e = 0; e < 4; ++e)
      free(s->QE[e][d]);
  }
  free(s);
}

int
eko_next_iteration(eko_solver * s)
{
  double * in = (s->iteration % 2 == 0) ? s->U : s->U2;
  double * out = (s->iteration % 2 == 0) ? s->U2 : s->U;
  if (!s->p.mhd)
  {
    /* SolverHydroMuscl::next_iteration_impl (SolverHydroMuscl.h:635-679):
     * compute_dt() on the current state, then godunov_unsplit(m_dt) */
    s->dt = hydro_compute_dt_local(s, in);
    if (s->t + s->dt > s->p.tEnd)
      s->dt = s->p.tEnd - s->t;
    hydro_godunov(s, in, out, s->dt);
  }
  else
  {
    /* SolverMHDMuscl::next_iteration_impl (SolverMHDMuscl.h:741-780) */
    if (s->p.dim == 2)
      mhd2d_godunov(s, in, out);
    else
      mhd3d_godunov(s, in, out);
  }
  s->iteration += 1;
  s->t += s->dt;
  return 0;
}

int
eko_set_gravity_field(eko_solver * s, const double * G)
{
  if (!s || !G || !s->G)
    return -1;
  memcpy(s->G, G, sizeof(double) * s->ncell * s->p.dim);
  const double * cur = (s->iteration % 2 == 0) ? s->U : s->U2;
  s->dt = hydro_compute_dt_local(s, cur);
  if (s->t + s->dt > s->p.tEnd)
    s->dt = s->p.tEnd - s->t;
  return 0;
}

int
eko_finished(const eko_solver * s)
{
  return s->t >= (s->p.tEnd - 1e-14) || s->iteration >= s->p.nStepmax;
}

void
eko_get_state(const eko_solver * s, double * U)
{
  const double * cur = (s->iteration % 2 == 0) ? s->U : s->U2;
  memcpy(U, cur, sizeof(double) * s->ncell * s->p.nbvar);
}

double
eko_time(const eko_solver * s)
{
  return s->t;
}
double
eko_dt(const eko_solver * s)
{
  return s->dt;
}
int
eko_iteration(const eko_solver * s)
{
  return s->iteration;
}
