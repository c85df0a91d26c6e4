// CT-MHD cell/face/edge arithmetic (3D), one cell, face or edge at a time.
// Expressions keep the reference's evaluation order (cited per function), so
// the FP64 build without FMA contraction reproduces the reference bit for bit.
#pragma once

#include "ek_common.cuh"

namespace EK_NS
{

template <class R>
struct MhdConst
{
  R gamma0, smallr, smallp, smallc, slope_type;
};

// find_speed_fast<dir> (mhd_utils.h:89-117)
template <class R, int DIR>
__device__ __forceinline__ R
mhd_speed_fast(const R (&q)[8], R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  const R bn = DIR == 0 ? a : (DIR == 1 ? b : c);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * bn * bn / d));
}

// find_speed_info<THREE_D> summed as ComputeDtFunctor3D_MHD does
// (mhd_utils.h:319-366, MHDRunFunctors3D.h:58-76).  FP64: the reference's
// expression; mixed: the candidate is formed in FP32 with 1/dx (the
// max-reduction and dt stay FP64).
template <class R>
__device__ __forceinline__ R
mhd_invdt(const R (&q)[8], R gamma0, double dx, double dy, double dz, float idx, float idy, float idz)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  const R cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
  const R cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
  const R cfz = sqrt(d2 + sqrt(d2 * d2 - c2 * c * c / d));
  const R vx = cfx + fabs(q[IU]);
  const R vy = cfy + fabs(q[IV]);
  const R vz = cfz + fabs(q[IW]);
  if constexpr (sizeof(R) == 8)
    return vx / dx + vy / dy + vz / dz;
  else
    return vx * idx + vy * idy + vz * idz;
}

// constoprim_mhd (MHDBaseFunctor3D.h:194-242).  u: hydro variables of the
// cell, bl/br: face fields of the cell and of its +1 neighbours.  In the
// mixed form (R = float) the internal energy is recomputed in FP64 from the
// FP64 face fields (bl64/br64, only read then) when total and
// magnetic+kinetic energy cancel (low beta / high Mach).
template <class R, class FB>
__device__ __forceinline__ void
mhd_constoprim(const R (&u)[5], const R (&bl)[3], const R (&br)[3], R (&q)[8], const MhdConst<R> & C,
               FB && fp64_faces)
{
  q[ID] = fmax(u[ID], C.smallr);
  q[IU] = u[IU] / q[ID];
  q[IV] = u[IV] / q[ID];
  q[IW] = u[IW] / q[ID];
  q[IA] = R(0.5) * (bl[0] + br[0]);
  q[IB] = R(0.5) * (bl[1] + br[1]);
  q[IC] = R(0.5) * (bl[2] + br[2]);
  const R eken = R(0.5) * (q[IU] * q[IU] + q[IV] * q[IV] + q[IW] * q[IW]);
  const R emag = R(0.5) * (q[IA] * q[IA] + q[IB] * q[IB] + q[IC] * q[IC]);
  R       eint = (u[IP] - emag) / q[ID] - eken;
  if constexpr (sizeof(R) == 4)
  {
    // FP64 island: E - emag - rho*eken cancels (low beta or high Mach)
    if (fabs(eint * q[ID]) < R(1.0 / 128.0) * fabs(u[IP]))
    {
      double bl64[3], br64[3];
      fp64_faces(bl64, br64);
      const double ba = 0.5 * (bl64[0] + br64[0]), bb = 0.5 * (bl64[1] + br64[1]),
                   bc = 0.5 * (bl64[2] + br64[2]);
      const double em = 0.5 * (ba * ba + bb * bb + bc * bc);
      const double d = (double)q[ID];
      const double vx = (double)u[IU] / d, vy = (double)u[IV] / d, vz = (double)u[IW] / d;
      eint = (R)(((double)u[IP] - em) / d - 0.5 * (vx * vx + vy * vy + vz * vz));
    }
  }
  q[IP] = fmax((C.gamma0 - R(1.0)) * q[ID] * eint, q[ID] * C.smallp);
}

// riemann_hlld (RiemannSolvers_MHD.h:130-364), states in the face frame.
// Only the five hydro components of the flux are used by the 3D update.
template <class R>
__device__ __forceinline__ void
mhd_hlld(R (&ql)[8], R (&qr)[8], R (&flux)[5], R gamma0)
{
  const R entho = R(1.0) / (gamma0 - R(1.0));
  const R a = R(0.5) * (ql[IA] + qr[IA]);
  const R sgnm = (a >= R(0)) ? R(1) : R(-1);
  ql[IA] = a;
  qr[IA] = a;
  const R rl = ql[ID], pl = ql[IP], ul = ql[IU], vl = ql[IV], wl = ql[IW], bl = ql[IB], cl = ql[IC];
  const R ecinl = R(0.5) * (ul * ul + vl * vl + wl * wl) * rl;
  const R emagl = R(0.5) * (a * a + bl * bl + cl * cl);
  const R etotl = pl * entho + ecinl + emagl;
  const R ptotl = pl + emagl;
  const R vdotbl = ul * a + vl * bl + wl * cl;
  const R rr = qr[ID], pr = qr[IP], ur = qr[IU], vr = qr[IV], wr = qr[IW], br = qr[IB], cr = qr[IC];
  const R ecinr = R(0.5) * (ur * ur + vr * vr + wr * wr) * rr;
  const R emagr = R(0.5) * (a * a + br * br + cr * cr);
  const R etotr = pr * entho + ecinr + emagr;
  const R ptotr = pr + emagr;
  const R vdotbr = ur * a + vr * br + wr * cr;

  const R cfastl = mhd_speed_fast<R, 0>(ql, gamma0);
  const R cfastr = mhd_speed_fast<R, 0>(qr, gamma0);
  const R sl = fmin(ul, ur) - fmax(cfastl, cfastr);
  const R sr = fmax(ul, ur) + fmax(cfastl, cfastr);
  const R rcl = rl * (ul - sl);
  const R rcr = rr * (sr - ur);
  const R ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const R ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  R estar;
  const R rstarl = rl * (sl - ul) / (sl - ustar);
  estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const R el = rl * (sl - ul) * (sl - ul) - a * a;
  R       vstarl, wstarl, bstarl, cstarl;
  if (a * a > R(0) && fabs(estar / (a * a) - R(1)) <= R(1e-8))
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
  const R vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  const R etotstarl =
    ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) / (sl - ustar);
  const R sqrrstarl = sqrt(rstarl);
  const R calfvenl = fabs(a) / sqrrstarl;
  const R sal = ustar - calfvenl;

  const R rstarr = rr * (sr - ur) / (sr - ustar);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const R er = rr * (sr - ur) * (sr - ur) - a * a;
  R       vstarr, wstarr, bstarr, cstarr;
  if (a * a > R(0) && fabs(estar / (a * a) - R(1)) <= R(1e-8))
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
  const R vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  const R etotstarr =
    ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) / (sr - ustar);
  const R sqrrstarr = sqrt(rstarr);
  const R calfvenr = fabs(a) / sqrrstarr;
  const R sar = ustar + calfvenr;

  R ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > R(0))
  {
    ro = rl, uo = ul, vo = vl, wo = wl, bo = bl, co = cl;
    ptoto = ptotl, etoto = etotl, vdotbo = vdotbl;
  }
  else if (sal > R(0))
  {
    ro = rstarl, uo = ustar, vo = vstarl, wo = wstarl, bo = bstarl, co = cstarl;
    ptoto = ptotstar, etoto = etotstarl, vdotbo = vdotbstarl;
  }
  else if (sr > R(0) && !(ustar > R(0)) && !(sar > R(0)))
  {
    ro = rstarr, uo = ustar, vo = vstarr, wo = wstarr, bo = bstarr, co = cstarr;
    ptoto = ptotstar, etoto = etotstarr, vdotbo = vdotbstarr;
  }
  else if (!(sr > R(0)) && !(ustar > R(0)) && !(sar > R(0)))
  {
    ro = rr, uo = ur, vo = vr, wo = wr, bo = br, co = cr;
    ptoto = ptotr, etoto = etotr, vdotbo = vdotbr;
  }
  else
  {
    // double-star region (only evaluated when sampled)
    const R vstarstar =
      (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) / (sqrrstarl + sqrrstarr);
    const R wstarstar =
      (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) / (sqrrstarl + sqrrstarr);
    const R bstarstar =
      (sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl)) /
      (sqrrstarl + sqrrstarr);
    const R cstarstar =
      (sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl)) /
      (sqrrstarl + sqrrstarr);
    const R vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
    vo = vstarstar, wo = wstarstar, bo = bstarstar, co = cstarstar;
    uo = ustar, ptoto = ptotstar, vdotbo = vdotbstarstar;
    if (ustar > R(0))
    {
      ro = rstarl;
      etoto = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
    }
    else
    {
      ro = rstarr;
      etoto = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);
    }
  }
  flux[ID] = ro * uo;
  flux[IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[IU] = ro * uo * uo - a * a + ptoto;
  flux[IV] = ro * uo * vo - a * bo;
  flux[IW] = ro * uo * wo - a * co;
}

template <class R>
__device__ __forceinline__ R
fmax4(R a0, R a1, R a2, R a3)
{
  R r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  return r;
}
template <class R>
__device__ __forceinline__ R
fmin4(R a0, R a1, R a2, R a3)
{
  R r = a0;
  r = (a1 < r) ? a1 : r;
  r = (a2 < r) ? a2 : r;
  r = (a3 < r) ? a3 : r;
  return r;
}
template <class R>
__device__ __forceinline__ R
fmax5(R a0, R a1, R a2, R a3, R a4)
{
  R r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  r = (a4 > r) ? a4 : r;
  return r;
}

// The parallel-plane state of one edge corner as mag_riemann2d_hlld reads
// it: density, pressure, two parallel velocities, two parallel fields and the
// orthogonal field (compute_emf, RiemannSolvers_MHD.h:648-860).
template <class R>
struct EdgeQ
{
  R r, p, u, v, a, b, c;
};

// mag_riemann2d_hlld (RiemannSolvers_MHD.h:395-627); corners LL, RL, LR, RR
template <class R>
__device__ __forceinline__ R
mag_riemann2d_hlld(const EdgeQ<R> & LL, const EdgeQ<R> & RL, const EdgeQ<R> & LR,
                   const EdgeQ<R> & RR, R ELL, R ERL, R ELR, R ERR, R gamma0, R smallc)
{
  auto fast = [gamma0](const EdgeQ<R> & q, bool ydir) {
    const R b2 = q.a * q.a + q.b * q.b + q.c * q.c;
    const R c2 = gamma0 * q.p / q.r;
    const R d2 = R(0.5) * (b2 / q.r + c2);
    const R bn = ydir ? q.b : q.a;
    return sqrt(d2 + sqrt(d2 * d2 - c2 * bn * bn / q.r));
  };
  const R rLL = LL.r, pLL = LL.p, uLL = LL.u, vLL = LL.v, aLL = LL.a, bLL = LL.b, cLL = LL.c;
  const R rLR = LR.r, pLR = LR.p, uLR = LR.u, vLR = LR.v, aLR = LR.a, bLR = LR.b, cLR = LR.c;
  const R rRL = RL.r, pRL = RL.p, uRL = RL.u, vRL = RL.v, aRL = RL.a, bRL = RL.b, cRL = RL.c;
  const R rRR = RR.r, pRR = RR.p, uRR = RR.u, vRR = RR.v, aRR = RR.a, bRR = RR.b, cRR = RR.c;

  const R cFastLLx = fast(LL, false), cFastLRx = fast(LR, false);
  const R cFastRLx = fast(RL, false), cFastRRx = fast(RR, false);
  const R cFastLLy = fast(LL, true), cFastLRy = fast(LR, true);
  const R cFastRLy = fast(RL, true), cFastRRy = fast(RR, true);

  const R SL = fmin4(uLL, uLR, uRL, uRR) - fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const R SR = fmax4(uLL, uLR, uRL, uRR) + fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const R SB = fmin4(vLL, vLR, vRL, vRR) - fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  const R ST = fmax4(vLL, vLR, vRL, vRR) + fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);

  const R PtotLL = pLL + R(0.5) * (aLL * aLL + bLL * bLL + cLL * cLL);
  const R PtotLR = pLR + R(0.5) * (aLR * aLR + bLR * bLR + cLR * cLR);
  const R PtotRL = pRL + R(0.5) * (aRL * aRL + bRL * bRL + cRL * cRL);
  const R PtotRR = pRR + R(0.5) * (aRR * aRR + bRR * bRR + cRR * cRR);

  const R rcLLx = rLL * (uLL - SL);
  const R rcRLx = rRL * (SR - uRL);
  const R rcLRx = rLR * (uLR - SL);
  const R rcRRx = rRR * (SR - uRR);
  const R rcLLy = rLL * (vLL - SB);
  const R rcLRy = rLR * (ST - vLR);
  const R rcRLy = rRL * (vRL - SB);
  const R rcRRy = rRR * (ST - vRR);

  const R ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  const R vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  const R rstarLLx = rLL * (SL - uLL) / (SL - ustar);
  const R BstarLL = bLL * (SL - uLL) / (SL - ustar);
  const R rstarLLy = rLL * (SB - vLL) / (SB - vstar);
  const R AstarLL = aLL * (SB - vLL) / (SB - vstar);
  const R rstarLL = rLL * (SL - uLL) / (SL - ustar) * (SB - vLL) / (SB - vstar);
  const R EstarLLx = ustar * BstarLL - vLL * aLL;
  const R EstarLLy = uLL * bLL - vstar * AstarLL;
  const R EstarLL = ustar * BstarLL - vstar * AstarLL;

  const R rstarLRx = rLR * (SL - uLR) / (SL - ustar);
  const R BstarLR = bLR * (SL - uLR) / (SL - ustar);
  const R rstarLRy = rLR * (ST - vLR) / (ST - vstar);
  const R AstarLR = aLR * (ST - vLR) / (ST - vstar);
  const R rstarLR = rLR * (SL - uLR) / (SL - ustar) * (ST - vLR) / (ST - vstar);
  const R EstarLRx = ustar * BstarLR - vLR * aLR;
  const R EstarLRy = uLR * bLR - vstar * AstarLR;
  const R EstarLR = ustar * BstarLR - vstar * AstarLR;

  const R rstarRLx = rRL * (SR - uRL) / (SR - ustar);
  const R BstarRL = bRL * (SR - uRL) / (SR - ustar);
  const R rstarRLy = rRL * (SB - vRL) / (SB - vstar);
  const R AstarRL = aRL * (SB - vRL) / (SB - vstar);
  const R rstarRL = rRL * (SR - uRL) / (SR - ustar) * (SB - vRL) / (SB - vstar);
  const R EstarRLx = ustar * BstarRL - vRL * aRL;
  const R EstarRLy = uRL * bRL - vstar * AstarRL;
  const R EstarRL = ustar * BstarRL - vstar * AstarRL;

  const R rstarRRx = rRR * (SR - uRR) / (SR - ustar);
  const R BstarRR = bRR * (SR - uRR) / (SR - ustar);
  const R rstarRRy = rRR * (ST - vRR) / (ST - vstar);
  const R AstarRR = aRR * (ST - vRR) / (ST - vstar);
  const R rstarRR = rRR * (SR - uRR) / (SR - ustar) * (ST - vRR) / (ST - vstar);
  const R EstarRRx = ustar * BstarRR - vRR * aRR;
  const R EstarRRy = uRR * bRR - vstar * AstarRR;
  const R EstarRR = ustar * BstarRR - vstar * AstarRR;

  const R calfvenL = fmax5(fabs(aLR) / sqrt(rstarLRx), fabs(AstarLR) / sqrt(rstarLR),
                           fabs(aLL) / sqrt(rstarLLx), fabs(AstarLL) / sqrt(rstarLL), smallc);
  const R calfvenR = fmax5(fabs(aRR) / sqrt(rstarRRx), fabs(AstarRR) / sqrt(rstarRR),
                           fabs(aRL) / sqrt(rstarRLx), fabs(AstarRL) / sqrt(rstarRL), smallc);
  const R calfvenB = fmax5(fabs(bLL) / sqrt(rstarLLy), fabs(BstarLL) / sqrt(rstarLL),
                           fabs(bRL) / sqrt(rstarRLy), fabs(BstarRL) / sqrt(rstarRL), smallc);
  const R calfvenT = fmax5(fabs(bLR) / sqrt(rstarLRy), fabs(BstarLR) / sqrt(rstarLR),
                           fabs(bRR) / sqrt(rstarRRy), fabs(BstarRR) / sqrt(rstarRR), smallc);

  const R SAL = fmin(ustar - calfvenL, R(0));
  const R SAR = fmax(ustar + calfvenR, R(0));
  const R SAB = fmin(vstar - calfvenB, R(0));
  const R SAT = fmax(vstar + calfvenT, R(0));

  const R AstarT = (SAR * AstarRR - SAL * AstarLR) / (SAR - SAL);
  const R AstarB = (SAR * AstarRL - SAL * AstarLL) / (SAR - SAL);
  const R BstarR = (SAT * BstarRR - SAB * BstarRL) / (SAT - SAB);
  const R BstarL = (SAT * BstarLR - SAB * BstarLL) / (SAT - SAB);

  R       E = 0, tmpE = 0;
  const int SB_pos = (int)(1 + copysign(R(1), SB)) / 2, SB_neg = 1 - SB_pos;
  const int ST_pos = (int)(1 + copysign(R(1), ST)) / 2, ST_neg = 1 - ST_pos;
  const int SL_pos = (int)(1 + copysign(R(1), SL)) / 2, SL_neg = 1 - SL_pos;
  const int SR_pos = (int)(1 + copysign(R(1), SR)) / 2, SR_neg = 1 - SR_pos;

  tmpE = (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) /
           (SAR - SAL) / (SAT - SAB) -
         SAT * SAB / (SAT - SAB) * (AstarT - AstarB) + SAR * SAL / (SAR - SAL) * (BstarR - BstarL);
  E += (R)(SB_neg * ST_pos * SL_neg * SR_pos) * tmpE;

  tmpE = (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) / (SAR - SAL);
  tmpE = (R)SL_pos * ELL + (R)(SL_neg * SR_neg) * ERL + (R)(SL_neg * SR_pos) * tmpE;
  E += (R)SB_pos * tmpE;

  tmpE = (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) / (SAR - SAL);
  tmpE = (R)SL_pos * ELR + (R)(SL_neg * SR_neg) * ERR + (R)(SL_neg * SR_pos) * tmpE;
  E += (R)(SB_neg * ST_neg) * tmpE;

  tmpE = (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) / (SAT - SAB);
  E += (R)(SB_neg * ST_pos * SL_pos) * tmpE;

  tmpE = (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) / (SAT - SAB);
  E += (R)(SB_neg * ST_pos * SL_neg * SR_neg) * tmpE;
  return E;
}

// compute_emf<emfDir> (RiemannSolvers_MHD.h:648-871) on the four corner
// states of an edge.  Each corner carries the components compute_emf reads
// for the edge direction: the velocities and face fields along the two
// transverse directions (u, a along the first, v, b along the second) and the
// field along the edge (c).
template <class R>
struct EdgeCorner
{
  R r, p, u, v, a, b, c;
};

template <class R>
__device__ __forceinline__ R
mhd_emf_corners(const EdgeCorner<R> & RT, const EdgeCorner<R> & RB, const EdgeCorner<R> & LT,
                const EdgeCorner<R> & LB, R gamma0, R smallc)
{
  EdgeQ<R> LL, RL, LR, RR;
  LL.r = RT.r, RL.r = LT.r, LR.r = RB.r, RR.r = LB.r;
  LL.p = RT.p, RL.p = LT.p, LR.p = RB.p, RR.p = LB.p;
  LL.u = RT.u, RL.u = LT.u, LR.u = RB.u, RR.u = LB.u;
  LL.v = RT.v, RL.v = LT.v, LR.v = RB.v, RR.v = LB.v;
  LL.a = R(0.5) * (RT.a + LT.a);
  RL.a = R(0.5) * (RT.a + LT.a);
  LR.a = R(0.5) * (RB.a + LB.a);
  RR.a = R(0.5) * (RB.a + LB.a);
  LL.b = R(0.5) * (RT.b + RB.b);
  RL.b = R(0.5) * (LT.b + LB.b);
  LR.b = R(0.5) * (RT.b + RB.b);
  RR.b = R(0.5) * (LT.b + LB.b);
  LL.c = RT.c, RL.c = LT.c, LR.c = RB.c, RR.c = LB.c;
  const R ELL = LL.u * LL.b - LL.v * LL.a;
  const R ERL = RL.u * RL.b - RL.v * RL.a;
  const R ELR = LR.u * LR.b - LR.v * LR.a;
  const R ERR = RR.u * RR.b - RR.v * RR.a;
  return mag_riemann2d_hlld<R>(LL, RL, LR, RR, ELL, ERL, ELR, ERR, gamma0, smallc);
}

// -------------------------------------------------------------------------
// Compact trace.  trace_unsplit_mhd_3d_simpler (MHDBaseFunctor3D.h:690-1114)
// produces 6 face states and 12 edge states per cell, all of them simple
// combinations of 47 per-cell numbers: the time-advanced cell-centred state
// and face fields, and the half slopes.  The trace kernel stores those 47
// numbers; the flux/emf kernel rebuilds any face or edge state from them with
// the reference's own expressions, so the result is bit-identical.
// -------------------------------------------------------------------------
enum : int
{
  T_R = 0, T_P, T_U, T_V, T_W, T_A, T_B, T_C,            // advanced cell state
  T_AL, T_AR, T_BL, T_BR, T_CL, T_CR,                    // advanced face fields
  T_DRX, T_DPX, T_DUX, T_DVX, T_DWX, T_DBX, T_DCX,       // half slopes along x
  T_DRY, T_DPY, T_DUY, T_DVY, T_DWY, T_DAY, T_DCY,       // along y
  T_DRZ, T_DPZ, T_DUZ, T_DVZ, T_DWZ, T_DAZ, T_DBZ,       // along z
  T_DALY, T_DALZ, T_DBLX, T_DBLZ, T_DCLX, T_DCLY,        // face-field half slopes
  T_DARY, T_DARZ, T_DBRX, T_DBRZ, T_DCRX, T_DCRY,
  T_N
};

template <class R>
__device__ __forceinline__ void
floor_state(R (&q)[8], R smallr, R smallp)
{
  q[ID] = fmax(smallr, q[ID]);
  q[IP] = fmax(smallp, q[IP]);
}

// Trace field indices as functions of a direction (0 x, 1 y, 2 z), so one
// code path serves the faces and edges of every direction:
//   hydro half slope of variable f (T_R..T_W) along e
//   half slope of the cell-centred field f along e (f != e)
//   face value of field f on the left (0) / right (1) face
//   half slope of that face value along e (e != f)
__device__ __forceinline__ int
t_hslope(int e, int f)
{
  return T_DRX + 7 * e + f;
}
__device__ __forceinline__ int
t_bslope(int e, int f)
{
  return T_DRX + 7 * e + 5 + (f < e ? f : f - 1);
}
__device__ __forceinline__ int
t_bface(int f, int right)
{
  return T_AL + 2 * f + right;
}
__device__ __forceinline__ int
t_bfslope(int f, int right, int e)
{
  return T_DALY + 6 * right + 2 * f + (e < f ? e : e - 1);
}

// Face state of a cell on its face normal to d (PLUS: the right face, the
// left state of that face; otherwise the left face), in the face frame the
// flux functor hands to the Riemann solver: normal velocity in IU and normal
// field in IA, with the reference's component swaps for y (IU<->IV, IA<->IB)
// and z (IU<->IW, IA<->IC) faces (trace_unsplit_mhd_3d_simpler,
// MHDBaseFunctor3D.h:905-955; MHDRunFunctors3D.h:1839-1874).
template <class R, bool PLUS>
__device__ __forceinline__ void
face_state_dir(const R * t, long long st, int d, R (&q)[8], R smallr, R smallp)
{
  auto h = [&](int f) {
    const R c = t[f * st], s = t[t_hslope(d, f) * st];
    return PLUS ? c + s : c - s;
  };
  auto tb = [&](int f) {
    const R c = t[(T_A + f) * st], s = t[t_bslope(d, f) * st];
    return PLUS ? c + s : c - s;
  };
  q[ID] = h(T_R);
  q[IP] = h(T_P);
  q[IU] = h(T_U + d);
  q[IV] = h(d == 1 ? T_U : T_V);
  q[IW] = h(d == 2 ? T_U : T_W);
  q[IA] = t[t_bface(d, PLUS ? 1 : 0) * st];
  q[IB] = tb(d == 1 ? 0 : 1);
  q[IC] = tb(d == 2 ? 0 : 2);
  floor_state(q, smallr, smallp);
}

// One corner of an edge along d (MHDBaseFunctor3D.h:957-1113).  The
// transverse directions are p1 = (d+1)%3 and p2 = (d+2)%3, the order in which
// compute_emf<emfDir> reads them; S1/S2 are the sides (+1 right, -1 left) of
// the corner along p1/p2.  Each sum keeps the reference's operands, so the
// result is bit-identical to the per-direction expressions.
template <class R, int S1, int S2>
__device__ __forceinline__ EdgeCorner<R>
edge_corner(const R * t, long long st, int d, int p1, int p2, R smallr, R smallp)
{
  auto sg1 = [](R x) { return S1 > 0 ? x : -x; };
  auto sg2 = [](R x) { return S2 > 0 ? x : -x; };
  auto hyd = [&](int f) {
    return t[f * st] + (sg1(t[t_hslope(p1, f) * st]) + sg2(t[t_hslope(p2, f) * st]));
  };
  EdgeCorner<R> e;
  e.r = fmax(smallr, hyd(T_R));
  e.p = fmax(smallp, hyd(T_P));
  e.u = hyd(T_U + p1);
  e.v = hyd(T_U + p2);
  e.a = t[t_bface(p1, S1 > 0) * st] + sg2(t[t_bfslope(p1, S1 > 0, p2) * st]);
  e.b = t[t_bface(p2, S2 > 0) * st] + sg1(t[t_bfslope(p2, S2 > 0, p1) * st]);
  e.c = t[(T_A + d) * st] + (sg1(t[t_bslope(p1, d) * st]) + sg2(t[t_bslope(p2, d) * st]));
  return e;
}

} // namespace EK_NS
