// Hydro cell/face arithmetic of the unsplit MUSCL-Hancock step, written for
// one cell or one face so the fused kernels can call it on shared-memory
// tiles.  Every expression keeps the evaluation order of the reference so the
// FP64 build compiled without FMA contraction reproduces it bit for bit; the
// cited reference lines define the arithmetic.
#pragma once

#include "ek_common.cuh"

namespace EK_NS
{

template <class R>
struct HydroConst
{
  R gamma0, smallr, smallp, smallc, slope_type, gamma6, smallpp;
  R entho; // 1 / (gamma0 - 1), the value every Riemann solver of the reference computes
};


// slope_unsplit_hydro_3d_scalar, one direction (HydroBaseFunctor3D.h:413-462,
// HydroBaseFunctor2D.h:423-453): minmod (slope_type 1) / MC (slope_type 2)
template <class R>
__device__ __forceinline__ R
slope1(R q, R qp, R qm, R st)
{
  if constexpr (sizeof(R) == 4)
  {
    // the same limiter, FP32 form (signed zeros may differ).  st is 0, 1 or
    // 2, so scaling by it is exact and min(|st dl|, |st dr|) = st min(|dl|,
    // |dr|) (0 for first order).
    // Where dl and dr have one sign, so has dcen, and |dcen| >= min(|dl|,
    // |dr|) after rounding too (rounding is monotonic): with st = 1 (minmod)
    // the centred difference never binds.
    const float dl = q - qm, dr = qp - q;
    float       m = st * fminf(fabsf(dl), fabsf(dr));
    if (st != 1.f)
      m = fminf(m, fabsf(0.5f * (qp - qm)));
    return (dl * dr > 0.f) ? copysignf(m, dl) : 0.f;
  }
  if constexpr (kShareRecip)
  {
    // FP64 FMA build: the minima of non-negative values as integer minima of
    // their bit patterns (same order; a NaN pattern is the larger, as fmin
    // drops NaN) and the sign by copysign, on the integer pipes instead of
    // GB300's 1/64-rate FP64 pipe.  As in the FP32 form, the scaling by st
    // (0, 1 or 2) is applied once to the minimum, and the centred difference
    // only where it can bind (st = 2); a non-zero slope has dl's sign (dl, dr
    // and dcen share it).  Only the sign of a zero slope can differ.
    auto minpos = [](double a, double b) {
      return __longlong_as_double(min(__double_as_longlong(a), __double_as_longlong(b)));
    };
    const R dl = q - qm, dr = qp - q;
    R       m = minpos(fabs(dl), fabs(dr));
    if (st != R(1))
      m = minpos(st * m, fabs(R(0.5) * (qp - qm)));
    return copysign((dl * dr <= R(0)) ? R(0) : m, dl);
  }
  const R dlft = st * (q - qm);
  const R drgt = st * (qp - q);
  const R dcen = R(0.5) * (qp - qm);
  const R dsgn = (dcen >= R(0)) ? R(1) : R(-1);
  const R slop = fmin(fabs(dlft), fabs(drgt));
  R       dlim = slop;
  if ((dlft * drgt) <= R(0))
    dlim = R(0);
  return dsgn * fmin(dlim, fabs(dcen));
}

// computePrimitives (HydroBaseFunctor2D.h:78-102, HydroBaseFunctor3D.h:80-106).
// In the mixed form (R = float) the internal energy is recomputed in FP64
// when E/rho and the kinetic energy cancel to fewer than ~7 significant bits.
template <class R, int NV>
__device__ __forceinline__ void
hydro_prims(const R (&u)[NV], R (&q)[NV], const HydroConst<R> & C)
{
  const R d = fmax(u[ID], C.smallr);
  // one reciprocal of the density for the four quotients (FP32: approximate;
  // FP64 exact build: four divisions)
  R id = R(0);
  if constexpr (sizeof(R) == 4)
    id = rcp_a(d);
  else if constexpr (kShareRecip)
    id = R(1) / d;
  auto over_d = [&](R x) {
    if constexpr (sizeof(R) == 4 || kShareRecip)
      return x * id;
    else
      return x / d;
  };
  const R ux = over_d(u[IU]);
  const R uy = over_d(u[IV]);
  R       eken, uz = R(0);
  if constexpr (NV == 4)
    eken = R(0.5) * (ux * ux + uy * uy);
  else
  {
    uz = over_d(u[IW]);
    eken = R(0.5) * (ux * ux + uy * uy + uz * uz);
  }
  const R ed = over_d(u[IP]);
  R       e = ed - eken;
  if constexpr (sizeof(R) == 4)
  {
    if (e < R(1.0 / 128.0) * ed)
    {
      // FP64 island: cancellation between total and kinetic energy
      const double dd = (double)d;
      const double vx = (double)u[IU] / dd, vy = (double)u[IV] / dd;
      double       ek = vx * vx + vy * vy;
      if constexpr (NV == 5)
      {
        const double vz = (double)u[IW] / dd;
        ek += vz * vz;
      }
      e = (R)((double)u[IP] / dd - 0.5 * ek);
    }
  }
  const R p = fmax((C.gamma0 - R(1)) * d * e, d * C.smallp);
  q[ID] = d;
  q[IP] = p;
  q[IU] = ux;
  q[IV] = uy;
  if constexpr (NV == 5)
    q[IW] = uz;
}

// sound speed as computePrimitives computes it: sqrt(gamma0 * p / d)
template <class R>
__device__ __forceinline__ R
hydro_sound(R d, R p, const HydroConst<R> & C)
{
  if constexpr (sizeof(R) == 4)
    return sqrt_a(C.gamma0 * p * rcp_a(d));
  else
    return sqrt(C.gamma0 * (p) / d);
}

// Per-cell source terms of trace_unsplit_{2d,3d}_along_dir
// (HydroBaseFunctor2D.h:250-253, HydroBaseFunctor3D.h:321-325).  They do not
// depend on the face, so they are computed once per cell.
template <class R, int NV>
__device__ __forceinline__ void
hydro_sources(const R (&q)[NV], const R (&dx)[NV], const R (&dy)[NV], const R (&dz)[NV], R (&s)[NV],
              const HydroConst<R> & C)
{
  const R r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  R       ir = R(0);
  if constexpr (sizeof(R) == 4)
    ir = rcp_a(r);
  else if constexpr (kShareRecip)
    ir = R(1) / r;
  auto over_r = [&](R x) {
    if constexpr (sizeof(R) == 4 || kShareRecip)
      return x * ir;
    else
      return x / r;
  };
  if constexpr (NV == 4)
  {
    s[ID] = -u * dx[ID] - v * dy[ID] - (dx[IU] + dy[IV]) * r;
    s[IP] = -u * dx[IP] - v * dy[IP] - (dx[IU] + dy[IV]) * C.gamma0 * p;
    s[IU] = -u * dx[IU] - v * dy[IU] - over_r(dx[IP]);
    s[IV] = -u * dx[IV] - v * dy[IV] - over_r(dy[IP]);
  }
  else
  {
    const R w = q[IW];
    s[ID] = -u * dx[ID] - v * dy[ID] - w * dz[ID] - (dx[IU] + dy[IV] + dz[IW]) * r;
    s[IP] = -u * dx[IP] - v * dy[IP] - w * dz[IP] - (dx[IU] + dy[IV] + dz[IW]) * C.gamma0 * p;
    s[IU] = -u * dx[IU] - v * dy[IU] - w * dz[IU] - over_r(dx[IP]);
    s[IV] = -u * dx[IV] - v * dy[IV] - w * dz[IV] - over_r(dy[IP]);
    s[IW] = -u * dx[IW] - v * dy[IW] - w * dz[IW] - over_r(dz[IP]);
  }
}

// face state of trace_unsplit_*_along_dir: q -/+ dq/2 + s*dtdx/2, rho floored
// (HydroBaseFunctor3D.h:327-365); sgn = -1 for the MIN face, +1 for MAX
template <class R, int NV>
__device__ __forceinline__ void
hydro_face(const R (&q)[NV], const R (&d)[NV], const R (&s)[NV], R dtd, bool plus, R (&f)[NV],
           R smallr)
{
  if constexpr (sizeof(R) == 4 || kShareRecip)
  {
    // mixed form and FP64 FMA build: two fused multiply-adds per variable
    const R hdtd = R(0.5) * dtd, hd = plus ? R(0.5) : R(-0.5);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      f[v] = fma(hd, d[v], fma(s[v], hdtd, q[v]));
  }
  else
  {
#pragma unroll
    for (int v = 0; v < NV; ++v)
    {
      if (plus)
        f[v] = q[v] + R(0.5) * d[v] + s[v] * dtd * R(0.5);
      else
        f[v] = q[v] - R(0.5) * d[v] + s[v] * dtd * R(0.5);
    }
  }
  f[ID] = fmax(smallr, f[ID]);
}

// riemann_hllc (RiemannSolvers.h:445-568).  States are in the face frame
// (normal velocity in IU); NV = 4 (2D) or 5 (3D).
template <class R, int NV>
__device__ __forceinline__ void
hllc(const R (&ql)[NV], const R (&qr)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  const R entho = C.entho;
  R       rl, pl, ul, etotl, rr, pr, ur, etotr, cmax; // cmax: the larger sound speed
  if constexpr (sizeof(R) == 4)
  {
    // mixed form: the two states in the lanes of packed FP32 pairs
    const float2 r = f2(fmaxf(ql[ID], C.smallr), fmaxf(qr[ID], C.smallr));
    const float2 ps = mul2(r, f2s(C.smallp));
    const float2 p = f2(fmaxf(ql[IP], ps.x), fmaxf(qr[IP], ps.y));
    const float2 u = f2(ql[IU], qr[IU]), v = f2(ql[IV], qr[IV]);
    float2       k2 = fma2(v, v, mul2(u, u));
    if constexpr (NV == 5)
      k2 = fma2(f2(ql[IW], qr[IW]), f2(ql[IW], qr[IW]), k2);
    const float2 etot = fma2(p, f2s(entho), mul2(mul2(f2s(0.5f), r), k2));
    const float2 c2 = mul2(mul2(f2s(C.gamma0), p), f2(rcp_a(r.x), rcp_a(r.y)));
    const float  sc2 = C.smallc * C.smallc;
    rl = r.x, pl = p.x, ul = u.x, etotl = etot.x;
    rr = r.y, pr = p.y, ur = u.y, etotr = etot.y;
    cmax = sqrt_a(fmaxf(fmaxf(c2.x, c2.y), sc2));
  }
  else
  {
    rl = fmax(ql[ID], C.smallr);
    pl = fmax(ql[IP], rl * C.smallp);
    ul = ql[IU];
    R ecinl = R(0.5) * rl * ul * ul;
    ecinl += R(0.5) * rl * ql[IV] * ql[IV];
    if constexpr (NV == 5)
      ecinl += R(0.5) * rl * ql[IW] * ql[IW];
    etotl = pl * entho + ecinl;

    rr = fmax(qr[ID], C.smallr);
    pr = fmax(qr[IP], rr * C.smallp);
    ur = qr[IU];
    R ecinr = R(0.5) * rr * ur * ur;
    ecinr += R(0.5) * rr * qr[IV] * qr[IV];
    if constexpr (NV == 5)
      ecinr += R(0.5) * rr * qr[IW] * qr[IW];
    etotr = pr * entho + ecinr;

    if constexpr (kShareRecip)
    {
      // FP64 FMA build: the larger sound speed squared with one division (the
      // densities are positive, so p_l / rho_l >= p_r / rho_r where p_l rho_r
      // >= p_r rho_l, up to rounding ties), then one square root (a correctly
      // rounded square root is monotonic)
      const bool lbig = pl * rr >= pr * rl;
      cmax = sqrt(fmax(C.gamma0 * (lbig ? pl : pr) / (lbig ? rl : rr), C.smallc * C.smallc));
    }
    else
      cmax = fmax(sqrt(fmax(C.gamma0 * pl / rl, C.smallc * C.smallc)),
                  sqrt(fmax(C.gamma0 * pr / rr, C.smallc * C.smallc)));
  }
  const R ptotl = pl, ptotr = pr;

  const R SL = fmin(ul, ur) - cmax;
  const R SR = fmax(ul, ur) + cmax;

  const R rcl = rl * (ul - SL);
  const R rcr = rr * (SR - ur);

  R ustar, ptotstar;
  if constexpr (sizeof(R) == 4)
  {
    const float irc = rcp_a(rcr + rcl);
    ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) * irc;
    ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) * irc;
  }
  else if constexpr (kShareRecip)
  {
    const R irc = R(1) / (rcr + rcl);
    ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) * irc;
    ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) * irc;
  }
  else
  {
    ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
    ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  }

  R ro, uo, ptoto, etoto;
  if constexpr (sizeof(R) == 4)
  {
    // FP32: the reference's four-way choice without branches -- the star
    // state is formed once, on the side of the contact (left when ustar > 0)
    const bool  left = ustar > 0.f;
    const float Sk = left ? SL : SR, rk = left ? rl : rr, uk = left ? ul : ur;
    const float ek = left ? etotl : etotr, pk = left ? ptotl : ptotr;
    const float is = rcp_a(Sk - ustar);
    const float rs = rk * (Sk - uk) * is;
    const float es = ((Sk - uk) * ek - pk * uk + ptotstar * ustar) * is;
    const bool  cL = SL > 0.f;                       // left state
    const bool  cR = !cL && !left && !(SR > 0.f);    // right state
    ro = cL ? rl : (cR ? rr : rs);
    uo = cL ? ul : (cR ? ur : ustar);
    ptoto = cL ? ptotl : (cR ? ptotr : ptotstar);
    etoto = cL ? etotl : (cR ? etotr : es);
  }
  else if (SL > R(0))
  {
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (ustar > R(0))
  {
    uo = ustar;
    ptoto = ptotstar;
    if constexpr (kShareRecip)
    {
      const R is = R(1) / (SL - ustar);
      ro = rl * (SL - ul) * is;
      etoto = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) * is;
    }
    else
    {
      ro = rl * (SL - ul) / (SL - ustar);
      etoto = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
    }
  }
  else if (SR > R(0))
  {
    uo = ustar;
    ptoto = ptotstar;
    if constexpr (kShareRecip)
    {
      const R is = R(1) / (SR - ustar);
      ro = rr * (SR - ur) * is;
      etoto = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) * is;
    }
    else
    {
      ro = rr * (SR - ur) / (SR - ustar);
      etoto = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
    }
  }
  else
  {
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }
  flux[ID] = ro * uo;
  flux[IU] = ro * uo * uo + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = flux[ID] * ((flux[ID] > R(0)) ? ql[IV] : qr[IV]);
  if constexpr (NV == 5)
    flux[IW] = flux[ID] * ((flux[ID] > R(0)) ? ql[IW] : qr[IW]);
}

// cmpflx (RiemannSolvers.h:20-53): flux of a Godunov state
template <class R, int NV>
__device__ __forceinline__ void
cmpflx(const R (&qg)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  flux[ID] = qg[ID] * qg[IU];
  flux[IU] = flux[ID] * qg[IU] + qg[IP];
  flux[IV] = flux[ID] * qg[IV];
  if constexpr (NV == 5)
    flux[IW] = flux[ID] * qg[IW];
  const R entho = C.entho;
  R       ekin = R(0.5) * qg[ID] * (qg[IU] * qg[IU] + qg[IV] * qg[IV]);
  if constexpr (NV == 5)
    ekin += R(0.5) * qg[ID] * (qg[IW] * qg[IW]);
  const R etot = qg[IP] * entho + ekin;
  flux[IP] = qg[IU] * (etot + qg[IP]);
}

// riemann_approx (RiemannSolvers.h:60-200): two-shock iterative solver,
// at most 10 Newton iterations on p*
template <class R, int NV>
__device__ __forceinline__ void
riemann_approx(const R (&ql)[NV], const R (&qr)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  const R gamma0 = C.gamma0, gamma6 = C.gamma6, smallr = C.smallr, smallc = C.smallc, smallp = C.smallp;
  const R rl = fmax(ql[ID], smallr), ul = ql[IU], pl = fmax(ql[IP], rl * smallp);
  const R rr = fmax(qr[ID], smallr), ur = qr[IU], pr = fmax(qr[IP], rr * smallp);
  const R cl = gamma0 * pl * rl;
  const R cr = gamma0 * pr * rr;
  R       wl = sqrt(cl);
  R       wr = sqrt(cr);
  R       pstar = fmax(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), R(0));
  R       pold = pstar;
  R       conv = R(1);
  for (int iter = 0; (iter < 10) && (conv > R(1e-6)); ++iter)
  {
    const R wwl = sqrt(cl * (R(1) + gamma6 * (pold - pl) / pl));
    const R wwr = sqrt(cr * (R(1) + gamma6 * (pold - pr) / pr));
    const R qql = R(2) * wwl * wwl * wwl / (wwl * wwl + cl);
    const R qqr = R(2) * wwr * wwr * wwr / (wwr * wwr + cr);
    const R usl = ul - (pold - pl) / wwl;
    const R usr = ur + (pold - pr) / wwr;
    const R delp = fmax(qqr * qql / (qqr + qql) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabs(delp / (pold + C.smallpp));
  }
  pstar = pold;
  wl = sqrt(cl * (R(1) + gamma6 * (pstar - pl) / pl));
  wr = sqrt(cr * (R(1) + gamma6 * (pstar - pr) / pr));
  const R ustar = R(0.5) * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  const R sgnm = copysign(R(1), ustar);
  R       ro, uo, po, wo;
  if (sgnm > R(0))
    ro = rl, uo = ul, po = pl, wo = wl;
  else
    ro = rr, uo = ur, po = pr, wo = wr;
  const R co = fmax(smallc, sqrt(fabs(gamma0 * po / ro)));
  const R rstar = fmax(R(ro / (R(1) + ro * (po - pstar) / (wo * wo))), smallr);
  const R cstar = fmax(smallc, sqrt(fabs(gamma0 * pstar / rstar)));
  R       spout = co - sgnm * uo;
  R       spin = cstar - sgnm * ustar;
  const R ushock = wo / ro - sgnm * uo;
  if (pstar >= po)
  {
    spin = ushock;
    spout = ushock;
  }
  const R scr = fmax(spout - spin, smallc + fabs(spout + spin));
  R       frac = R(0.5) * (R(1) + (spout + spin) / scr);
  if (frac != frac)
    frac = R(0);
  else
    frac = frac >= R(1) ? R(1) : frac <= R(0) ? R(0) : frac;
  R qg[NV];
  qg[ID] = frac * rstar + (R(1) - frac) * ro;
  qg[IU] = frac * ustar + (R(1) - frac) * uo;
  qg[IP] = frac * pstar + (R(1) - frac) * po;
  if (spout < R(0))
    qg[ID] = ro, qg[IU] = uo, qg[IP] = po;
  if (spin > R(0))
    qg[ID] = rstar, qg[IU] = ustar, qg[IP] = pstar;
  qg[IV] = sgnm > R(0) ? ql[IV] : qr[IV];
  if constexpr (NV == 5)
    qg[IW] = sgnm > R(0) ? ql[IW] : qr[IW];
  cmpflx<R, NV>(qg, flux, C);
}

// conservative state and flux of a primitive state, as riemann_llf and
// riemann_hll build them (RiemannSolvers.h:262-320, 384-420)
template <class R, int NV>
__device__ __forceinline__ void
hydro_uf(const R (&q)[NV], R (&u)[NV], R (&f)[NV], R entho)
{
  u[ID] = q[ID];
  u[IP] = q[IP] * entho + R(0.5) * q[ID] * q[IU] * q[IU];
  u[IP] += R(0.5) * q[ID] * q[IV] * q[IV];
  if constexpr (NV == 5)
    u[IP] += R(0.5) * q[ID] * q[IW] * q[IW];
  u[IU] = q[ID] * q[IU];
  u[IV] = q[ID] * q[IV];
  if constexpr (NV == 5)
    u[IW] = q[ID] * q[IW];
  f[ID] = u[ID] * q[IU];
  f[IP] = q[IU] * (u[IP] + q[IP]);
  f[IU] = q[IP] + u[IU] * q[IU];
  f[IV] = f[ID] * q[IV];
  if constexpr (NV == 5)
    f[IW] = f[ID] * q[IW];
}

// riemann_llf (RiemannSolvers.h:218-330)
template <class R, int NV>
__device__ __forceinline__ void
riemann_llf(const R (&ql)[NV], const R (&qr)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  const R entho = C.entho;
  const R rl = fmax(ql[ID], C.smallr), ul = ql[IU], pl = fmax(ql[IP], rl * C.smallp);
  const R rr = fmax(qr[ID], C.smallr), ur = qr[IU], pr = fmax(qr[IP], rr * C.smallp);
  const R cl = sqrt(C.gamma0 * pl / rl);
  const R cr = sqrt(C.gamma0 * pr / rr);
  const R cmax = fmax(fabs(ul) + cl, fabs(ur) + cr);
  R       uleft[NV], uright[NV], fleft[NV], fright[NV];
  hydro_uf<R, NV>(ql, uleft, fleft, entho);
  hydro_uf<R, NV>(qr, uright, fright, entho);
#pragma unroll
  for (int v = 0; v < NV; ++v)
    flux[v] = R(0.5) * (fleft[v] + fright[v] - cmax * (uright[v] - uleft[v]));
}

// riemann_hll (RiemannSolvers.h:344-432); used for 2D only, as the
// reference's 3D dispatch has no HLL branch
template <class R, int NV>
__device__ __forceinline__ void
riemann_hll(const R (&ql)[NV], const R (&qr)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  const R entho = C.entho;
  const R rl = fmax(ql[ID], C.smallr), ul = ql[IU], pl = fmax(ql[IP], rl * C.smallp);
  const R rr = fmax(qr[ID], C.smallr), ur = qr[IU], pr = fmax(qr[IP], rr * C.smallp);
  const R cl = sqrt(C.gamma0 * pl / rl);
  const R cr = sqrt(C.gamma0 * pr / rr);
  const R SL = fmin(fmin(ul, ur) - fmax(cl, cr), R(0));
  const R SR = fmax(fmax(ul, ur) + fmax(cl, cr), R(0));
  R       uleft[NV], uright[NV], fleft[NV], fright[NV];
  hydro_uf<R, NV>(ql, uleft, fleft, entho);
  hydro_uf<R, NV>(qr, uright, fright, entho);
#pragma unroll
  for (int v = 0; v < NV; ++v)
    flux[v] = (SR * fleft[v] - SL * fright[v] + SR * SL * (uright[v] - uleft[v])) / (SR - SL);
}

// riemann_hydro (RiemannSolvers.h:573-640) with the solver fixed at compile
// time: RS = the reference's riemannSolverType (0 approx, 1 llf, 2 hll, 3 hllc)
template <int RS, class R, int NV>
__device__ __forceinline__ void
hydro_riemann(const R (&ql)[NV], const R (&qr)[NV], R (&flux)[NV], const HydroConst<R> & C)
{
  if constexpr (RS == 0)
    riemann_approx<R, NV>(ql, qr, flux, C);
  else if constexpr (RS == 1)
    riemann_llf<R, NV>(ql, qr, flux, C);
  else if constexpr (RS == 2)
    riemann_hll<R, NV>(ql, qr, flux, C);
  else
    hllc<R, NV>(ql, qr, flux, C);
}

// per-cell CFL candidate of ComputeDtFunctor{2D,3D}
// (HydroRunFunctors2D.h:56-84, HydroRunFunctors3D.h:49-84), in the working
// precision: FP64 keeps the reference's expression; the mixed form uses the
// FP32 inverse cell sizes.  Threads keep a NaN-ignoring max (fmax, as the
// reference's reduction) and convert to the FP64 key once.
template <class R, int NV>
__device__ __forceinline__ R
hydro_invdt(const R (&u)[NV], const HydroConst<R> & C, const KParams & P)
{
  R q[NV];
  hydro_prims<R, NV>(u, q, C);
  const R c = hydro_sound<R>(q[ID], q[IP], C);
  const R vx = c + fabs(q[IU]);
  const R vy = c + fabs(q[IV]);
  if constexpr (sizeof(R) == 8 && !kShareRecip)
  {
    if constexpr (NV == 4)
      return vx / P.dx + vy / P.dy;
    else
    {
      const R vz = c + fabs(q[IW]);
      return vx / P.dx + vy / P.dy + vz / P.dz;
    }
  }
  else if constexpr (sizeof(R) == 8)
  {
    // FP64 FMA build: the inverse cell sizes prepared on the host
    if constexpr (NV == 4)
      return vx * P.idxd + vy * P.idyd;
    else
    {
      const R vz = c + fabs(q[IW]);
      return vx * P.idxd + vy * P.idyd + vz * P.idzd;
    }
  }
  else
  {
    if constexpr (NV == 4)
      return vx * P.idx + vy * P.idy;
    else
    {
      const R vz = c + fabs(q[IW]);
      return vx * P.idx + vy * P.idy + vz * P.idz;
    }
  }
}

// ---------------------------------------------------------------------------
// Static gravity (SolverHydroMuscl with [gravity] enabled)
// ---------------------------------------------------------------------------

// gravity vector of cell (i, j, k) in raw array indexes (ghosts included;
// the field is read as stored, not mapped through the boundary conditions).
// Indexes past the array (cells of partial tiles, whose results are
// discarded) are clamped.
template <class S, class R, int NV>
__device__ __forceinline__ void
grav_at(const KParams & P, int i, int j, int k, R (&g)[3])
{
  if (P.gfield)
  {
    i = min(max(i, 0), P.isize - 1);
    j = min(max(j, 0), P.jsize - 1);
    k = min(max(k, 0), P.ksize - 1);
    const S *       G = (const S *)P.gfield;
    const long long off = (long long)k * P.plane + (long long)j * P.isize + i;
    g[0] = (R)ldg(G + off);
    g[1] = (R)ldg(G + P.vstride + off);
    g[2] = NV == 5 ? (R)ldg(G + 2 * P.vstride + off) : R(0);
  }
  else if constexpr (sizeof(R) == 8)
  {
    g[0] = P.g[0], g[1] = P.g[1], g[2] = P.g[2];
  }
  else
  {
    g[0] = P.gf[0], g[1] = P.gf[1], g[2] = P.gf[2];
  }
}

// Hancock gravity predictor of one face state: q += (dt/2) g of the cell the
// state was traced from, on the velocity components in the cell's own frame
// (before any IU/IV/IW swap; HydroRunFunctors2D.h:656-665,
// HydroRunFunctors3D.h:489-500).  hg = (0.5 dt) g.
template <class R, int NV>
__device__ __forceinline__ void
grav_kick(R (&q)[NV], const R (&hg)[3])
{
  q[IU] += hg[0];
  q[IV] += hg[1];
  if constexpr (NV == 5)
    q[IW] += hg[2];
}

// GravitySourceTermFunctor2D/3D (HydroRunFunctors2D.h:1555-1630,
// HydroRunFunctors3D.h:1903-1980) on the updated state u of one cell:
// momentum += (dt/2) g (rho_old + rho_new), energy += the kinetic energy
// change; the 2D form floors rho_new at smallr.  FP64 keeps the reference's
// expression (ekin_new - ekin_old); FP32 uses the equal form
// sum du (m + du/2) / rho_new, which has no cancellation.
template <class R, int NV>
__device__ __forceinline__ void
grav_source(R (&u)[NV], R rho_old, const R (&g)[3], R hdt, const HydroConst<R> & C)
{
  const R rn = NV == 4 ? fmax(C.smallr, u[ID]) : u[ID];
  if constexpr (sizeof(R) == 8)
  {
    R ru = u[IU], rv = u[IV];
    if constexpr (NV == 4)
    {
      const R ek0 = R(0.5) * (ru * ru + rv * rv) / rn;
      ru += hdt * g[0] * (rho_old + rn);
      rv += hdt * g[1] * (rho_old + rn);
      u[IU] = ru;
      u[IV] = rv;
      const R ek1 = R(0.5) * (ru * ru + rv * rv) / rn;
      u[IP] += (ek1 - ek0);
    }
    else
    {
      R       rw = u[IW];
      const R ek0 = R(0.5) * (ru * ru + rv * rv + rw * rw) / rn;
      ru += hdt * g[0] * (rho_old + rn);
      rv += hdt * g[1] * (rho_old + rn);
      rw += hdt * g[2] * (rho_old + rn);
      u[IU] = ru;
      u[IV] = rv;
      u[IW] = rw;
      const R ek1 = R(0.5) * (ru * ru + rv * rv + rw * rw) / rn;
      u[IP] += (ek1 - ek0);
    }
  }
  else
  {
    const R rs = rho_old + rn;
    R       de = R(0);
#pragma unroll
    for (int e = 0; e < NV - 2; ++e)
    {
      const R du = hdt * g[e] * rs;
      de += du * (u[IU + e] + R(0.5) * du);
      u[IU + e] += du;
    }
    u[IP] += de * rcp_a(rn);
  }
}

// per-cell CFL candidate of ComputeDtGravityFunctor2D/3D
// (HydroRunFunctors2D.h:125-170, HydroRunFunctors3D.h:133-184):
// g dt^2 / (2 dx) + u dt / dx <= cfl, u = sum(|v_i| + c), g = sum(|g_i|),
// dx = min(dx, dy[, dz]).  FP64 keeps the reference's expression; FP32 writes
// the correction factor kk / (sqrt(1 + 2 kk) - 1) as (sqrt(1 + 2 kk) + 1) / 2,
// equal without the cancellation.
template <class R, int NV>
__device__ __forceinline__ R
hydro_invdt_grav(const R (&u)[NV], const R (&g)[3], const HydroConst<R> & C, const KParams & P)
{
  R q[NV];
  hydro_prims<R, NV>(u, q, C);
  const R c = hydro_sound<R>(q[ID], q[IP], C);
  R       velocity = c + fabs(q[IU]);
  velocity += c + fabs(q[IV]);
  R kk = fabs(g[0]) + fabs(g[1]);
  if constexpr (NV == 5)
  {
    velocity += c + fabs(q[IW]);
    kk = kk + fabs(g[2]);
  }
  if constexpr (sizeof(R) == 8)
  {
    kk *= P.cfl_dxmin / (velocity * velocity);
    kk = fmax(kk, 1e-4);
    velocity *= kk / (sqrt(1.0 + 2.0 * kk) - 1.0);
    return velocity / P.dxmin;
  }
  else
  {
    kk = fmax(kk * P.cfl_dxminf * rcp_a(velocity * velocity), 1e-4f);
    return velocity * (R(0.5) * (sqrt_a(R(1) + R(2) * kk) + R(1))) * P.idxminf;
  }
}

} // namespace EK_NS
