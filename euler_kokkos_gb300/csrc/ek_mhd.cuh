// CT-MHD cell/face/edge arithmetic (3D), one cell, face or edge at a time.
// Expressions keep the reference's evaluation order (cited per function), so
// the FP64 build without FMA contraction reproduces the reference bit for bit.
#pragma once

#include <type_traits>

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
  const R bn = DIR == 0 ? a : (DIR == 1 ? b : c);
  if constexpr (kShareRecip)
  {
    const R id = R(1) / d;
    const R c2 = gamma0 * p * id;
    const R d2 = R(0.5) * (b2 * id + c2);
    return sqrt(d2 + sqrt(d2 * d2 - c2 * bn * bn * id));
  }
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * bn * bn / d));
}

// the square of find_speed_fast<dir> before its outer square root (FP64 FMA
// build).  A correctly rounded square root is monotonic, so the largest of
// several speeds is the square root of the largest of these, bit for bit,
// one square root instead of one per state.
template <class R, int DIR>
__device__ __forceinline__ R
mhd_speed_fast_sq(const R (&q)[8], R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R bn = DIR == 0 ? a : (DIR == 1 ? b : c);
  const R id = R(1) / d;
  const R c2 = gamma0 * p * id;
  const R d2 = R(0.5) * (b2 * id + c2);
  return d2 + sqrt(d2 * d2 - c2 * bn * bn * id);
}

// find_speed_info<THREE_D> summed as ComputeDtFunctor3D_MHD does
// (mhd_utils.h:319-366, MHDRunFunctors3D.h:58-76).  FP64: the reference's
// expression; mixed: the candidate is formed in FP32 with 1/dx (the
// max-reduction and dt stay FP64).
template <class R>
__device__ __forceinline__ R
mhd_invdt(const R (&q)[8], R gamma0, double dx, double dy, double dz, float idx, float idy, float idz,
          double idxd, double idyd, double idzd)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  if constexpr (sizeof(R) == 4)
  {
    const float id = rcp_a(d);
    const float c2 = gamma0 * p * id;
    const float d2 = 0.5f * (b2 * id + c2);
    const float dd = d2 * d2, cr = c2 * id;
    const float cfx = sqrt_a(d2 + sqrt_a(dd - cr * a * a));
    const float cfy = sqrt_a(d2 + sqrt_a(dd - cr * b * b));
    const float cfz = sqrt_a(d2 + sqrt_a(dd - cr * c * c));
    return (cfx + fabsf(q[IU])) * idx + (cfy + fabsf(q[IV])) * idy + (cfz + fabsf(q[IW])) * idz;
  }
  if constexpr (kShareRecip)
  {
    // FP64 FMA build: one reciprocal of the density, host-prepared 1/dx
    const R id = R(1) / d;
    const R c2 = gamma0 * p * id;
    const R d2 = R(0.5) * (b2 * id + c2);
    const R dd = d2 * d2, cr = c2 * id;
    const R cfx = sqrt(d2 + sqrt(dd - cr * a * a));
    const R cfy = sqrt(d2 + sqrt(dd - cr * b * b));
    const R cfz = sqrt(d2 + sqrt(dd - cr * c * c));
    return (cfx + fabs(q[IU])) * idxd + (cfy + fabs(q[IV])) * idyd + (cfz + fabs(q[IW])) * idzd;
  }
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  const R cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
  const R cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
  const R cfz = sqrt(d2 + sqrt(d2 * d2 - c2 * c * c / d));
  const R vx = cfx + fabs(q[IU]);
  const R vy = cfy + fabs(q[IV]);
  const R vz = cfz + fabs(q[IW]);
  return vx / dx + vy / dy + vz / dz;
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
  R id = R(0);
  if constexpr (sizeof(R) == 4)
  {
    id = rcp_a(q[ID]);
    q[IU] = u[IU] * id;
    q[IV] = u[IV] * id;
    q[IW] = u[IW] * id;
  }
  else if constexpr (kShareRecip)
  {
    id = R(1) / q[ID];
    q[IU] = u[IU] * id;
    q[IV] = u[IV] * id;
    q[IW] = u[IW] * id;
  }
  else
  {
    q[IU] = u[IU] / q[ID];
    q[IV] = u[IV] / q[ID];
    q[IW] = u[IW] / q[ID];
  }
  q[IA] = R(0.5) * (bl[0] + br[0]);
  q[IB] = R(0.5) * (bl[1] + br[1]);
  q[IC] = R(0.5) * (bl[2] + br[2]);
  const R eken = R(0.5) * (q[IU] * q[IU] + q[IV] * q[IV] + q[IW] * q[IW]);
  const R emag = R(0.5) * (q[IA] * q[IA] + q[IB] * q[IB] + q[IC] * q[IC]);
  R       eint;
  if constexpr (sizeof(R) == 4 || kShareRecip)
    eint = (u[IP] - emag) * id - eken;
  else
    eint = (u[IP] - emag) / q[ID] - eken;
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

// riemann_hlld in FP32 for the mixed form: the reference's solver with each
// shared denominator inverted once (rcp_a), |B_n| / sqrt(rho*) as a
// reciprocal square root, and the left and right states in the two lanes of
// packed FP32 pairs; the same branches, and the faces it cannot decide left
// to FP64 (below).

// The star-state denominators of HLLD, estar = rho (S - u)(S - ustar) - Bn^2,
// cancel as the state approaches the degenerate one (transverse field near
// zero, fast speed near the Alfven speed).  In FP32 their quotients
// (v*, B*, w*, C*) then lose all accuracy and a face flux can blow up the
// solution; FP64 keeps them accurate, as the reference's FP64 build shows.
// Below this fraction of Bn^2 the face is recomputed in FP64: FP32 rounding
// leaves estar an absolute error of a few 1e-7 Bn^2, so above the threshold the
// quotients keep a relative accuracy of about 1e-2 or better.  (A threshold of
// 2^-7 flags a few per cent of the Orszag-Tang faces, where the transverse
// field crosses zero; 2^-14 flags none of them.)
constexpr float kHlldStarTol = 1.0f / 16384.0f;

// false: a star-state denominator of this face is ill-conditioned in FP32
// (|estar| < kHlldStarTol Bn^2), or the reference's degenerate-state test
// |estar / Bn^2 - 1| <= 1e-8 cannot be decided in FP32; the face is then
// solved in FP64 (flux is not written)
template <int NF>
__device__ __forceinline__ bool
mhd_hlld_f32(const float (&ql)[8], const float (&qr)[8], float (&flux)[NF], float gamma0)
{
  // left state in lane x, right state in lane y
  const float  entho = rcp_a(gamma0 - 1.0f);
  const float  a = 0.5f * (ql[IA] + qr[IA]);
  const float  sgnm = (a >= 0.f) ? 1.f : -1.f;
  const float  a2 = a * a;
  const float2 A = f2s(a), A2 = f2s(a2), H = f2s(0.5f);
  const float2 r = f2(ql[ID], qr[ID]), p = f2(ql[IP], qr[IP]), u = f2(ql[IU], qr[IU]);
  const float2 v = f2(ql[IV], qr[IV]), w = f2(ql[IW], qr[IW]), b = f2(ql[IB], qr[IB]), c = f2(ql[IC], qr[IC]);
  const float2 bsq = fma2(c, c, fma2(b, b, A2));                         // a^2 + b^2 + c^2
  const float2 ecin = mul2(mul2(H, fma2(w, w, fma2(v, v, mul2(u, u)))), r);
  const float2 emag = mul2(H, bsq);
  const float2 etot = add2(fma2(p, f2s(entho), ecin), emag);
  const float2 ptot = add2(p, emag);
  const float2 vdotb = fma2(w, c, fma2(v, b, mul2(u, A)));

  // fast magnetosonic speeds (find_speed_fast, the normal field a)
  const float2 id = f2(rcp_a(r.x), rcp_a(r.y));
  const float2 c2 = mul2(mul2(f2s(gamma0), p), id);
  const float2 d2 = mul2(H, fma2(bsq, id, c2));
  const float2 dq = fma2(d2, d2, neg2(mul2(mul2(c2, A2), id)));
  const float2 cq = add2(d2, f2(sqrt_a(dq.x), sqrt_a(dq.y)));
  const float  cmax = sqrt_a(fmaxf(cq.x, cq.y)); // the larger fast speed
  const float  sl = fminf(u.x, u.y) - cmax;
  const float  sr = fmaxf(u.x, u.y) + cmax;
  const float2 S = f2(sl, sr);
  const float2 su = sub2(S, u);  // S - u
  const float2 rsu = mul2(r, su); // rho (S - u): -rcl, rcr
  const float  rcl = -rsu.x, rcr = rsu.y;
  const float  irc = rcp_a(rcr + rcl);
  const float  ustar = (rcr * u.y + rcl * u.x + (ptot.x - ptot.y)) * irc;
  const float  ptotstar = (rcr * ptot.x + rcl * ptot.y + rcl * rcr * (u.x - u.y)) * irc;
  const float2 US = f2s(ustar);
  const float2 sus = sub2(S, US);
  // the star-state denominators; the face goes to FP64 when one is
  // ill-conditioned, or within 1e-6 of the reference's degenerate-state test
  // |estar / Bn^2 - 1| <= 1e-8 (which FP32 cannot decide).  So that test is
  // false for every face solved here, and its branch is not needed below.
  const float2 estar = fma2(rsu, sus, neg2(A2));
  auto         ill = [&](float e) { return fabsf(e) < kHlldStarTol * a2 || fabsf(e - a2) <= 1e-6f * a2; };
  if (ill(estar.x) || ill(estar.y))
    return false;

  const float2 is = f2(rcp_a(sus.x), rcp_a(sus.y));
  const float2 rstar = mul2(rsu, is);
  const float2 e = fma2(rsu, su, neg2(A2)); // rho (S - u)^2 - Bn^2
  const float2 ie = f2(rcp_a(estar.x), rcp_a(estar.y));
  const float2 t = mul2(mul2(A, sub2(US, u)), ie);
  const float2 vstar = fma2(b, neg2(t), v);
  const float2 bstar = mul2(mul2(b, e), ie);
  const float2 wstar = fma2(c, neg2(t), w);
  const float2 cstar = mul2(mul2(c, e), ie);
  const float2 vdotbstar = fma2(wstar, cstar, fma2(vstar, bstar, mul2(US, A)));
  const float2 etotstar =
    mul2(add2(fma2(su, etot, neg2(mul2(ptot, u))), fma2(A, sub2(vdotb, vdotbstar), f2s(ptotstar * ustar))), is);
  const float  sqrrstarl = sqrt_a(rstar.x), sqrrstarr = sqrt_a(rstar.y);
  const float  sal = ustar - fabsf(a) * rsqrt_a(rstar.x);
  const float  sar = ustar + fabsf(a) * rsqrt_a(rstar.y);

  const float rl = r.x, ul = u.x, vl = v.x, wl = w.x, bl = b.x, cl = c.x;
  const float rr = r.y, ur = u.y, vr = v.y, wr = w.y, br = b.y, cr = c.y;
  const float ptotl = ptot.x, ptotr = ptot.y, etotl = etot.x, etotr = etot.y, vdotbl = vdotb.x, vdotbr = vdotb.y;
  const float rstarl = rstar.x, rstarr = rstar.y;
  const float vstarl = vstar.x, vstarr = vstar.y, wstarl = wstar.x, wstarr = wstar.y;
  const float bstarl = bstar.x, bstarr = bstar.y, cstarl = cstar.x, cstarr = cstar.y;
  const float vdotbstarl = vdotbstar.x, vdotbstarr = vdotbstar.y, etotstarl = etotstar.x, etotstarr = etotstar.y;

  float ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > 0.f)
  {
    ro = rl, uo = ul, vo = vl, wo = wl, bo = bl, co = cl;
    ptoto = ptotl, etoto = etotl, vdotbo = vdotbl;
  }
  else if (sal > 0.f)
  {
    ro = rstarl, uo = ustar, vo = vstarl, wo = wstarl, bo = bstarl, co = cstarl;
    ptoto = ptotstar, etoto = etotstarl, vdotbo = vdotbstarl;
  }
  else if (sr > 0.f && !(ustar > 0.f) && !(sar > 0.f))
  {
    ro = rstarr, uo = ustar, vo = vstarr, wo = wstarr, bo = bstarr, co = cstarr;
    ptoto = ptotstar, etoto = etotstarr, vdotbo = vdotbstarr;
  }
  else if (!(sr > 0.f) && !(ustar > 0.f) && !(sar > 0.f))
  {
    ro = rr, uo = ur, vo = vr, wo = wr, bo = br, co = cr;
    ptoto = ptotr, etoto = etotr, vdotbo = vdotbr;
  }
  else
  {
    const float iss = rcp_a(sqrrstarl + sqrrstarr);
    const float vss = (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) * iss;
    const float wss = (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) * iss;
    const float bss = (sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl)) * iss;
    const float css = (sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl)) * iss;
    const float vdotbss = ustar * a + vss * bss + wss * css;
    vo = vss, wo = wss, bo = bss, co = css;
    uo = ustar, ptoto = ptotstar, vdotbo = vdotbss;
    if (ustar > 0.f)
    {
      ro = rstarl;
      etoto = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbss);
    }
    else
    {
      ro = rstarr;
      etoto = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbss);
    }
  }
  flux[ID] = ro * uo;
  flux[IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[IU] = ro * uo * uo - a2 + ptoto;
  flux[IV] = ro * uo * vo - a * bo;
  flux[IW] = ro * uo * wo - a * co;
  if constexpr (NF > 5)
    flux[5] = co * uo - a * wo;
  return true;
}

// riemann_hlld (RiemannSolvers_MHD.h:130-364), states in the face frame.
// The 3D update uses the five hydro components of the flux (NF = 5); the 2D
// update also uses the Bz component, returned in flux[5] when NF = 6.
// Returns false when the FP32 solver leaves the face to its FP64 island (an
// ill-conditioned star state, see mhd_hlld_f32): the caller then solves it
// with mhd_hlld<double> from the same states.
template <class R, int NF = 5>
__device__ __forceinline__ bool
mhd_hlld(R (&ql)[8], R (&qr)[8], R (&flux)[NF], R gamma0)
{
  if constexpr (sizeof(R) == 4)
    return mhd_hlld_f32<NF>(ql, qr, flux, gamma0);
  else
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

  // the larger fast speed (FP64 FMA build: one outer square root, the same bits)
  R cmax;
  if constexpr (kShareRecip)
    cmax = sqrt(fmax(mhd_speed_fast_sq<R, 0>(ql, gamma0), mhd_speed_fast_sq<R, 0>(qr, gamma0)));
  else
    cmax = fmax(mhd_speed_fast<R, 0>(ql, gamma0), mhd_speed_fast<R, 0>(qr, gamma0));
  const R sl = fmin(ul, ur) - cmax;
  const R sr = fmax(ul, ur) + cmax;
  const R rcl = rl * (ul - sl);
  const R rcr = rr * (sr - ur);
  // FP64 FMA build: one reciprocal per shared denominator (kShareRecip)
  const R irc = kShareRecip ? R(1) / (rcr + rcl) : R(0);
  const R ustar = kShareRecip ? (rcr * ur + rcl * ul + (ptotl - ptotr)) * irc
                              : (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const R ptotstar = kShareRecip ? (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) * irc
                                 : (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  R estar;
  // the degenerate-state test divides both sides' estar by a^2: one
  // reciprocal in the FP64 FMA build
  const R ia2 = kShareRecip ? R(1) / (a * a) : R(0);
  auto    degenerate = [&](R e) {
    return a * a > R(0) && fabs((kShareRecip ? e * ia2 : e / (a * a)) - R(1)) <= R(1e-8);
  };
  const R isl = kShareRecip ? R(1) / (sl - ustar) : R(0);
  const R rstarl = kShareRecip ? rl * (sl - ul) * isl : rl * (sl - ul) / (sl - ustar);
  estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const R el = rl * (sl - ul) * (sl - ul) - a * a;
  R       vstarl, wstarl, bstarl, cstarl;
  if (degenerate(estar))
  {
    vstarl = vl;
    bstarl = bl;
    wstarl = wl;
    cstarl = cl;
  }
  else if constexpr (kShareRecip)
  {
    const R ie = R(1) / estar;
    vstarl = vl - a * bl * (ustar - ul) * ie;
    bstarl = bl * el * ie;
    wstarl = wl - a * cl * (ustar - ul) * ie;
    cstarl = cl * el * ie;
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
    kShareRecip ? ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) * isl
                : ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) / (sl - ustar);
  // sqrt(rho*) and |a| / sqrt(rho*): one reciprocal square root in the FP64
  // FMA build
  const R rsl = kShareRecip ? rsqrt(rstarl) : R(0);
  const R sqrrstarl = kShareRecip ? rstarl * rsl : sqrt(rstarl);
  const R calfvenl = kShareRecip ? fabs(a) * rsl : fabs(a) / sqrrstarl;
  const R sal = ustar - calfvenl;

  const R isr = kShareRecip ? R(1) / (sr - ustar) : R(0);
  const R rstarr = kShareRecip ? rr * (sr - ur) * isr : rr * (sr - ur) / (sr - ustar);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const R er = rr * (sr - ur) * (sr - ur) - a * a;
  R       vstarr, wstarr, bstarr, cstarr;
  if (degenerate(estar))
  {
    vstarr = vr;
    bstarr = br;
    wstarr = wr;
    cstarr = cr;
  }
  else if constexpr (kShareRecip)
  {
    const R ie = R(1) / estar;
    vstarr = vr - a * br * (ustar - ur) * ie;
    bstarr = br * er * ie;
    wstarr = wr - a * cr * (ustar - ur) * ie;
    cstarr = cr * er * ie;
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
    kShareRecip ? ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) * isr
                : ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) / (sr - ustar);
  const R rsr = kShareRecip ? rsqrt(rstarr) : R(0);
  const R sqrrstarr = kShareRecip ? rstarr * rsr : sqrt(rstarr);
  const R calfvenr = kShareRecip ? fabs(a) * rsr : fabs(a) / sqrrstarr;
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
    const R iss = kShareRecip ? R(1) / (sqrrstarl + sqrrstarr) : R(0);
    const R vstarstar =
      kShareRecip ? (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) * iss
                  : (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) / (sqrrstarl + sqrrstarr);
    const R wstarstar =
      kShareRecip ? (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) * iss
                  : (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) / (sqrrstarl + sqrrstarr);
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
  if constexpr (NF > 5)
    flux[5] = co * uo - a * wo;
  return true;
  }
}

// riemann_mhd (RiemannSolvers_MHD.h:368-389) with the solver fixed at compile
// time: RS = the reference's riemannSolverType (1 llf, 2 hll, 4 hlld)
template <int RS, class R, int NF>
__device__ __forceinline__ bool
mhd_riemann(R (&ql)[8], R (&qr)[8], R (&flux)[NF], R gamma0);

// find_mhd_flux (mhd_utils.h:170-231, cIso = 0): conservative state and
// flux of a face-frame primitive state; components ID, IP, IU, IV, IW and,
// for NF = 6, IC in slot 5
template <class R, int NF>
__device__ __forceinline__ void
find_mhd_flux(const R (&q)[8], R (&cv)[NF], R (&ff)[NF], R gamma0)
{
  const R entho = R(1.0) / (gamma0 - R(1.0));
  const R d = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW], a = q[IA], b = q[IB], c = q[IC];
  const R ecin = R(0.5) * (u * u + v * v + w * w) * d;
  const R emag = R(0.5) * (a * a + b * b + c * c);
  const R etot = p * entho + ecin + emag;
  const R ptot = p + emag;
  cv[ID] = d, cv[IP] = etot, cv[IU] = d * u, cv[IV] = d * v, cv[IW] = d * w;
  ff[ID] = d * u;
  ff[IP] = (etot + ptot) * u - a * (a * u + b * v + c * w);
  ff[IU] = d * u * u - a * a + ptot;
  ff[IV] = d * u * v - a * b;
  ff[IW] = d * u * w - a * c;
  if constexpr (NF > 5)
  {
    cv[5] = c;
    ff[5] = c * u - a * w;
  }
}

// riemann_hll for MHD (RiemannSolvers_MHD.h:27-62)
template <class R, int NF>
__device__ __forceinline__ void
mhd_hll(R (&ql)[8], R (&qr)[8], R (&flux)[NF], R gamma0)
{
  const R bx_mean = R(0.5) * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  R uleft[NF], fleft[NF], uright[NF], fright[NF];
  find_mhd_flux<R, NF>(ql, uleft, fleft, gamma0);
  find_mhd_flux<R, NF>(qr, uright, fright, gamma0);
  const R cfleft = mhd_speed_fast<R, 0>(ql, gamma0);
  const R cfright = mhd_speed_fast<R, 0>(qr, gamma0);
  const R vleft = ql[IU], vright = qr[IU];
  const R sl = fmin(fmin(vleft, vright) - fmax(cfleft, cfright), R(0.0));
  const R sr = fmax(fmax(vleft, vright) + fmax(cfleft, cfright), R(0.0));
#pragma unroll
  for (int v = 0; v < NF; ++v)
    flux[v] = (sr * fleft[v] - sl * fright[v] + sr * sl * (uright[v] - uleft[v])) / (sr - sl);
}

// riemann_llf for MHD (RiemannSolvers_MHD.h:77-104); the information speed
// is find_speed_info of the normal direction (mhd_utils.h:379-403)
template <class R, int NF>
__device__ __forceinline__ void
mhd_llf(R (&ql)[8], R (&qr)[8], R (&flux)[NF], R gamma0)
{
  const R bx_mean = R(0.5) * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  R uleft[NF], fleft[NF], uright[NF], fright[NF];
  find_mhd_flux<R, NF>(ql, uleft, fleft, gamma0);
  find_mhd_flux<R, NF>(qr, uright, fright, gamma0);
#pragma unroll
  for (int v = 0; v < NF; ++v)
    flux[v] = (fleft[v] + fright[v]) / R(2);
  const R cleft = mhd_speed_fast<R, 0>(ql, gamma0) + fabs(ql[IU]);
  const R cright = mhd_speed_fast<R, 0>(qr, gamma0) + fabs(qr[IU]);
  const R vel_info = fmax(cleft, cright);
#pragma unroll
  for (int v = 0; v < NF; ++v)
    flux[v] -= vel_info * (uright[v] - uleft[v]) / R(2);
}

// false: the FP32 HLLD left this face to its FP64 island (mhd_riemann_f64)
template <int RS, class R, int NF>
__device__ __forceinline__ bool
mhd_riemann(R (&ql)[8], R (&qr)[8], R (&flux)[NF], R gamma0)
{
  if constexpr (RS == 1)
    mhd_llf<R, NF>(ql, qr, flux, gamma0);
  else if constexpr (RS == 2)
    mhd_hll<R, NF>(ql, qr, flux, gamma0);
  else
    return mhd_hlld<R, NF>(ql, qr, flux, gamma0);
  return true;
}

// The FP64 island of the FP32 HLLD: the face solved in FP64 from the same
// FP32 face states (exact conversions).  Only the repair kernels call it, for
// the faces the FP32 solver declined; the step kernels hold no FP64 HLLD code,
// which would raise their register count (a 64-register 2D step kernel went
// to 126) or spill inside their hot loops.  Out of line, states and flux by
// value.
struct HlldFlux32
{
  float f[6];
};
template <int NF>
__device__ __noinline__ HlldFlux32
mhd_hlld_f64_island(float4 l0, float4 l1, float4 r0, float4 r1, float gamma0)
{
  double l[8] = { f2d(l0.x), f2d(l0.y), f2d(l0.z), f2d(l0.w), f2d(l1.x), f2d(l1.y), f2d(l1.z), f2d(l1.w) };
  double r[8] = { f2d(r0.x), f2d(r0.y), f2d(r0.z), f2d(r0.w), f2d(r1.x), f2d(r1.y), f2d(r1.z), f2d(r1.w) };
  double f[NF];
  mhd_hlld<double, NF>(l, r, f, f2d(gamma0));
  HlldFlux32 out;
#pragma unroll
  for (int i = 0; i < 6; ++i)
    out.f[i] = i < NF ? d2f_rn(f[i < NF ? i : 0]) : 0.f;
  return out;
}
template <int NF>
__device__ __forceinline__ void
mhd_hlld_f64_from_f32(const float (&ql)[8], const float (&qr)[8], float (&flux)[NF], float gamma0)
{
  const HlldFlux32 o = mhd_hlld_f64_island<NF>(make_float4(ql[0], ql[1], ql[2], ql[3]), make_float4(ql[4], ql[5], ql[6], ql[7]),
                                               make_float4(qr[0], qr[1], qr[2], qr[3]), make_float4(qr[4], qr[5], qr[6], qr[7]),
                                               gamma0);
#pragma unroll
  for (int i = 0; i < NF; ++i)
    flux[i] = o.f[i];
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

// mag_riemann2d_hlld in FP32 for the mixed form: one reciprocal per corner
// density and per shared denominator, |B| / sqrt(rho*) as reciprocal square
// roots; the reference's branch-free selection of the emf.
__device__ __forceinline__ float
mag_riemann2d_hlld_f32(const EdgeQ<float> & LL, const EdgeQ<float> & RL, const EdgeQ<float> & LR,
                       const EdgeQ<float> & RR, float ELL, float ERL, float ELR, float ERR, float gamma0,
                       float smallc)
{
  // squares of the fast speeds along x and y (before the outer square root:
  // one square root of the largest of the four corners', below)
  auto fast2 = [gamma0](const EdgeQ<float> & q, float & cx, float & cy) {
    const float ir = rcp_a(q.r);
    const float c2 = gamma0 * q.p * ir;
    const float d2 = 0.5f * ((q.a * q.a + q.b * q.b + q.c * q.c) * ir + c2);
    const float dd = d2 * d2, cr = c2 * ir;
    cx = d2 + sqrt_a(dd - cr * q.a * q.a);
    cy = d2 + sqrt_a(dd - cr * q.b * q.b);
  };
  const float rLL = LL.r, pLL = LL.p, uLL = LL.u, vLL = LL.v, aLL = LL.a, bLL = LL.b, cLL = LL.c;
  const float rLR = LR.r, pLR = LR.p, uLR = LR.u, vLR = LR.v, aLR = LR.a, bLR = LR.b, cLR = LR.c;
  const float rRL = RL.r, pRL = RL.p, uRL = RL.u, vRL = RL.v, aRL = RL.a, bRL = RL.b, cRL = RL.c;
  const float rRR = RR.r, pRR = RR.p, uRR = RR.u, vRR = RR.v, aRR = RR.a, bRR = RR.b, cRR = RR.c;
  float cLLx, cLLy, cLRx, cLRy, cRLx, cRLy, cRRx, cRRy;
  fast2(LL, cLLx, cLLy);
  fast2(LR, cLRx, cLRy);
  fast2(RL, cRLx, cRLy);
  fast2(RR, cRRx, cRRy);
  const float cmx = sqrt_a(fmax4(cLLx, cLRx, cRLx, cRRx)), cmy = sqrt_a(fmax4(cLLy, cLRy, cRLy, cRRy));
  const float SL = fmin4(uLL, uLR, uRL, uRR) - cmx;
  const float SR = fmax4(uLL, uLR, uRL, uRR) + cmx;
  const float SB = fmin4(vLL, vLR, vRL, vRR) - cmy;
  const float ST = fmax4(vLL, vLR, vRL, vRR) + cmy;

  const float PtotLL = pLL + 0.5f * (aLL * aLL + bLL * bLL + cLL * cLL);
  const float PtotLR = pLR + 0.5f * (aLR * aLR + bLR * bLR + cLR * cLR);
  const float PtotRL = pRL + 0.5f * (aRL * aRL + bRL * bRL + cRL * cRL);
  const float PtotRR = pRR + 0.5f * (aRR * aRR + bRR * bRR + cRR * cRR);

  const float rcLLx = rLL * (uLL - SL), rcRLx = rRL * (SR - uRL);
  const float rcLRx = rLR * (uLR - SL), rcRRx = rRR * (SR - uRR);
  const float rcLLy = rLL * (vLL - SB), rcLRy = rLR * (ST - vLR);
  const float rcRLy = rRL * (vRL - SB), rcRRy = rRR * (ST - vRR);

  const float ustar = (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) *
                      rcp_a(rcLLx + rcLRx + rcRLx + rcRRx);
  const float vstar = (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) *
                      rcp_a(rcLLy + rcLRy + rcRLy + rcRRy);
  const float iL = rcp_a(SL - ustar), iR = rcp_a(SR - ustar), iB = rcp_a(SB - vstar), iT = rcp_a(ST - vstar);

  // star states of corner (r, u, v, a, b) against the x-side factor fx and y-side factor fy
  const float fxLL = (SL - uLL) * iL, fyLL = (SB - vLL) * iB;
  const float fxLR = (SL - uLR) * iL, fyLR = (ST - vLR) * iT;
  const float fxRL = (SR - uRL) * iR, fyRL = (SB - vRL) * iB;
  const float fxRR = (SR - uRR) * iR, fyRR = (ST - vRR) * iT;

  const float rstarLLx = rLL * fxLL, BstarLL = bLL * fxLL, rstarLLy = rLL * fyLL, AstarLL = aLL * fyLL;
  const float rstarLL = rstarLLx * fyLL;
  const float EstarLLx = ustar * BstarLL - vLL * aLL, EstarLLy = uLL * bLL - vstar * AstarLL;
  const float EstarLL = ustar * BstarLL - vstar * AstarLL;
  const float rstarLRx = rLR * fxLR, BstarLR = bLR * fxLR, rstarLRy = rLR * fyLR, AstarLR = aLR * fyLR;
  const float rstarLR = rstarLRx * fyLR;
  const float EstarLRx = ustar * BstarLR - vLR * aLR, EstarLRy = uLR * bLR - vstar * AstarLR;
  const float EstarLR = ustar * BstarLR - vstar * AstarLR;
  const float rstarRLx = rRL * fxRL, BstarRL = bRL * fxRL, rstarRLy = rRL * fyRL, AstarRL = aRL * fyRL;
  const float rstarRL = rstarRLx * fyRL;
  const float EstarRLx = ustar * BstarRL - vRL * aRL, EstarRLy = uRL * bRL - vstar * AstarRL;
  const float EstarRL = ustar * BstarRL - vstar * AstarRL;
  const float rstarRRx = rRR * fxRR, BstarRR = bRR * fxRR, rstarRRy = rRR * fyRR, AstarRR = aRR * fyRR;
  const float rstarRR = rstarRRx * fyRR;
  const float EstarRRx = ustar * BstarRR - vRR * aRR, EstarRRy = uRR * bRR - vstar * AstarRR;
  const float EstarRR = ustar * BstarRR - vstar * AstarRR;

  const float qLL = rsqrt_a(rstarLL), qLR = rsqrt_a(rstarLR), qRL = rsqrt_a(rstarRL), qRR = rsqrt_a(rstarRR);
  const float calfvenL = fmax5(fabsf(aLR) * rsqrt_a(rstarLRx), fabsf(AstarLR) * qLR,
                               fabsf(aLL) * rsqrt_a(rstarLLx), fabsf(AstarLL) * qLL, smallc);
  const float calfvenR = fmax5(fabsf(aRR) * rsqrt_a(rstarRRx), fabsf(AstarRR) * qRR,
                               fabsf(aRL) * rsqrt_a(rstarRLx), fabsf(AstarRL) * qRL, smallc);
  const float calfvenB = fmax5(fabsf(bLL) * rsqrt_a(rstarLLy), fabsf(BstarLL) * qLL,
                               fabsf(bRL) * rsqrt_a(rstarRLy), fabsf(BstarRL) * qRL, smallc);
  const float calfvenT = fmax5(fabsf(bLR) * rsqrt_a(rstarLRy), fabsf(BstarLR) * qLR,
                               fabsf(bRR) * rsqrt_a(rstarRRy), fabsf(BstarRR) * qRR, smallc);

  const float SAL = fminf(ustar - calfvenL, 0.f);
  const float SAR = fmaxf(ustar + calfvenR, 0.f);
  const float SAB = fminf(vstar - calfvenB, 0.f);
  const float SAT = fmaxf(vstar + calfvenT, 0.f);
  const float iAx = rcp_a(SAR - SAL), iAy = rcp_a(SAT - SAB);

  const float AstarT = (SAR * AstarRR - SAL * AstarLR) * iAx;
  const float AstarB = (SAR * AstarRL - SAL * AstarLL) * iAx;
  const float BstarR = (SAT * BstarRR - SAB * BstarRL) * iAy;
  const float BstarL = (SAT * BstarLR - SAB * BstarLL) * iAy;

  // the reference's sign masks (1 + copysign(1, S)) / 2 as sign-bit tests and
  // its mask-weighted sums as selects: exactly one term of each sum is live
  const bool SBp = !signbit(SB), STp = !signbit(ST), SLp = !signbit(SL), SRp = !signbit(SR);
  float      E = 0.f, tmpE;

  tmpE = (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) * iAx * iAy -
         SAT * SAB * iAy * (AstarT - AstarB) + SAR * SAL * iAx * (BstarR - BstarL);
  E += (!SBp && STp && !SLp && SRp) ? tmpE : 0.f;

  tmpE = (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) * iAx;
  tmpE = SLp ? ELL : (!SRp ? ERL : tmpE);
  E += SBp ? tmpE : 0.f;

  tmpE = (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) * iAx;
  tmpE = SLp ? ELR : (!SRp ? ERR : tmpE);
  E += (!SBp && !STp) ? tmpE : 0.f;

  tmpE = (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) * iAy;
  E += (!SBp && STp && SLp) ? tmpE : 0.f;

  tmpE = (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) * iAy;
  E += (!SBp && STp && !SLp && !SRp) ? tmpE : 0.f;
  return E;
}

// mag_riemann2d_hlld (RiemannSolvers_MHD.h:395-627); corners LL, RL, LR, RR
template <class R>
__device__ __forceinline__ R
mag_riemann2d_hlld(const EdgeQ<R> & LL, const EdgeQ<R> & RL, const EdgeQ<R> & LR,
                   const EdgeQ<R> & RR, R ELL, R ERL, R ELR, R ERR, R gamma0, R smallc)
{
  if constexpr (sizeof(R) == 4)
    return mag_riemann2d_hlld_f32(LL, RL, LR, RR, ELL, ERL, ELR, ERR, gamma0, smallc);
  else
  {
  // fast speed of a corner state along x or y; the FP64 FMA build returns its
  // square (before the outer square root, see mhd_speed_fast_sq) and takes one
  // square root of the largest
  auto fast = [gamma0](const EdgeQ<R> & q, bool ydir) {
    const R b2 = q.a * q.a + q.b * q.b + q.c * q.c;
    const R bn = ydir ? q.b : q.a;
    if constexpr (kShareRecip)
    {
      const R ir = R(1) / q.r;
      const R c2 = gamma0 * q.p * ir;
      const R d2 = R(0.5) * (b2 * ir + c2);
      return d2 + sqrt(d2 * d2 - c2 * bn * bn * ir);
    }
    const R c2 = gamma0 * q.p / q.r;
    const R d2 = R(0.5) * (b2 / q.r + c2);
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

  R cmx = fmax4(cFastLLx, cFastLRx, cFastRLx, cFastRRx), cmy = fmax4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  if constexpr (kShareRecip)
    cmx = sqrt(cmx), cmy = sqrt(cmy);
  const R SL = fmin4(uLL, uLR, uRL, uRR) - cmx;
  const R SR = fmax4(uLL, uLR, uRL, uRR) + cmx;
  const R SB = fmin4(vLL, vLR, vRL, vRR) - cmy;
  const R ST = fmax4(vLL, vLR, vRL, vRR) + cmy;

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

  // quotients by the six shared denominators: divided in the exact build (the
  // reference's expressions), one reciprocal each in the FMA build
  const R dSLu = SL - ustar, dSRu = SR - ustar, dSBv = SB - vstar, dSTv = ST - vstar;
  const R iSLu = kShareRecip ? R(1) / dSLu : R(0), iSRu = kShareRecip ? R(1) / dSRu : R(0);
  const R iSBv = kShareRecip ? R(1) / dSBv : R(0), iSTv = kShareRecip ? R(1) / dSTv : R(0);
  auto q_SLu = [&](R x) { return kShareRecip ? x * iSLu : x / dSLu; };
  auto q_SRu = [&](R x) { return kShareRecip ? x * iSRu : x / dSRu; };
  auto q_SBv = [&](R x) { return kShareRecip ? x * iSBv : x / dSBv; };
  auto q_STv = [&](R x) { return kShareRecip ? x * iSTv : x / dSTv; };
  const R rstarLLx = q_SLu(rLL * (SL - uLL));
  const R BstarLL = q_SLu(bLL * (SL - uLL));
  const R rstarLLy = q_SBv(rLL * (SB - vLL));
  const R AstarLL = q_SBv(aLL * (SB - vLL));
  const R rstarLL = q_SBv(q_SLu(rLL * (SL - uLL)) * (SB - vLL));
  const R EstarLLx = ustar * BstarLL - vLL * aLL;
  const R EstarLLy = uLL * bLL - vstar * AstarLL;
  const R EstarLL = ustar * BstarLL - vstar * AstarLL;

  const R rstarLRx = q_SLu(rLR * (SL - uLR));
  const R BstarLR = q_SLu(bLR * (SL - uLR));
  const R rstarLRy = q_STv(rLR * (ST - vLR));
  const R AstarLR = q_STv(aLR * (ST - vLR));
  const R rstarLR = q_STv(q_SLu(rLR * (SL - uLR)) * (ST - vLR));
  const R EstarLRx = ustar * BstarLR - vLR * aLR;
  const R EstarLRy = uLR * bLR - vstar * AstarLR;
  const R EstarLR = ustar * BstarLR - vstar * AstarLR;

  const R rstarRLx = q_SRu(rRL * (SR - uRL));
  const R BstarRL = q_SRu(bRL * (SR - uRL));
  const R rstarRLy = q_SBv(rRL * (SB - vRL));
  const R AstarRL = q_SBv(aRL * (SB - vRL));
  const R rstarRL = q_SBv(q_SRu(rRL * (SR - uRL)) * (SB - vRL));
  const R EstarRLx = ustar * BstarRL - vRL * aRL;
  const R EstarRLy = uRL * bRL - vstar * AstarRL;
  const R EstarRL = ustar * BstarRL - vstar * AstarRL;

  const R rstarRRx = q_SRu(rRR * (SR - uRR));
  const R BstarRR = q_SRu(bRR * (SR - uRR));
  const R rstarRRy = q_STv(rRR * (ST - vRR));
  const R AstarRR = q_STv(aRR * (ST - vRR));
  const R rstarRR = q_STv(q_SRu(rRR * (SR - uRR)) * (ST - vRR));
  const R EstarRRx = ustar * BstarRR - vRR * aRR;
  const R EstarRRy = uRR * bRR - vstar * AstarRR;
  const R EstarRR = ustar * BstarRR - vstar * AstarRR;

  // |B| / sqrt(rho*): the reference's quotient in the exact build; one
  // reciprocal square root (CUDA's rsqrt) in the FMA build
  auto b_over_sqrt = [](R b, R r) { return kShareRecip ? fabs(b) * rsqrt(r) : fabs(b) / sqrt(r); };
  const R calfvenL = fmax5(b_over_sqrt(aLR, rstarLRx), b_over_sqrt(AstarLR, rstarLR),
                           b_over_sqrt(aLL, rstarLLx), b_over_sqrt(AstarLL, rstarLL), smallc);
  const R calfvenR = fmax5(b_over_sqrt(aRR, rstarRRx), b_over_sqrt(AstarRR, rstarRR),
                           b_over_sqrt(aRL, rstarRLx), b_over_sqrt(AstarRL, rstarRL), smallc);
  const R calfvenB = fmax5(b_over_sqrt(bLL, rstarLLy), b_over_sqrt(BstarLL, rstarLL),
                           b_over_sqrt(bRL, rstarRLy), b_over_sqrt(BstarRL, rstarRL), smallc);
  const R calfvenT = fmax5(b_over_sqrt(bLR, rstarLRy), b_over_sqrt(BstarLR, rstarLR),
                           b_over_sqrt(bRR, rstarRRy), b_over_sqrt(BstarRR, rstarRR), smallc);

  const R SAL = fmin(ustar - calfvenL, R(0));
  const R SAR = fmax(ustar + calfvenR, R(0));
  const R SAB = fmin(vstar - calfvenB, R(0));
  const R SAT = fmax(vstar + calfvenT, R(0));
  const R dA = SAR - SAL, dB = SAT - SAB;
  const R iA = kShareRecip ? R(1) / dA : R(0), iB = kShareRecip ? R(1) / dB : R(0);
  auto q_A = [&](R x) { return kShareRecip ? x * iA : x / dA; };
  auto q_B = [&](R x) { return kShareRecip ? x * iB : x / dB; };

  const R AstarT = q_A(SAR * AstarRR - SAL * AstarLR);
  const R AstarB = q_A(SAR * AstarRL - SAL * AstarLL);
  const R BstarR = q_B(SAT * BstarRR - SAB * BstarRL);
  const R BstarL = q_B(SAT * BstarLR - SAB * BstarLL);

  R       E = 0, tmpE = 0;
  const int SB_pos = (int)(1 + copysign(R(1), SB)) / 2, SB_neg = 1 - SB_pos;
  const int ST_pos = (int)(1 + copysign(R(1), ST)) / 2, ST_neg = 1 - ST_pos;
  const int SL_pos = (int)(1 + copysign(R(1), SL)) / 2, SL_neg = 1 - SL_pos;
  const int SR_pos = (int)(1 + copysign(R(1), SR)) / 2, SR_neg = 1 - SR_pos;

  tmpE = q_B(q_A(SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL)) -
         q_B(SAT * SAB) * (AstarT - AstarB) + q_A(SAR * SAL) * (BstarR - BstarL);
  E += (R)(SB_neg * ST_pos * SL_neg * SR_pos) * tmpE;

  tmpE = q_A(SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL));
  tmpE = (R)SL_pos * ELL + (R)(SL_neg * SR_neg) * ERL + (R)(SL_neg * SR_pos) * tmpE;
  E += (R)SB_pos * tmpE;

  tmpE = q_A(SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR));
  tmpE = (R)SL_pos * ELR + (R)(SL_neg * SR_neg) * ERR + (R)(SL_neg * SR_pos) * tmpE;
  E += (R)(SB_neg * ST_neg) * tmpE;

  tmpE = q_B(SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL));
  E += (R)(SB_neg * ST_pos * SL_pos) * tmpE;

  tmpE = q_B(SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL));
  E += (R)(SB_neg * ST_pos * SL_neg * SR_neg) * tmpE;
  return E;
  }
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

// Accessors of a cell's trace fields: A(f) is field f.
// StrideAcc: field-major storage with stride st (the staged shared-memory
// planes).  QuadAcc: the HBM trace, 16-byte quads of fields per cell (see
// trace_cell); the gathers below read compile-time field indices, so only the
// quads a face or edge state needs are loaded (the others are never used and
// their loads are removed), one vector load per quad.
template <class R>
struct StrideAcc
{
  const R * t;
  int       st;
  __device__ __forceinline__ R
  operator()(int f) const
  {
    return t[f * st];
  }
};
constexpr int kTraceLanes = 32; // cells per block of the HBM trace
template <class R>
using TVec = typename std::conditional<sizeof(R) == 4, float4, double2>::type;
template <class R>
constexpr int kTVecN = 16 / (int)sizeof(R); // fields per quad
template <class R>
constexpr int kTQuads = (T_N + kTVecN<R> - 1) / kTVecN<R>; // quads per cell
template <class R>
struct QuadAcc
{
  TVec<R> v[kTQuads<R>];
  __device__ __forceinline__ explicit QuadAcc(const R * t)
  {
#pragma unroll
    for (int q = 0; q < kTQuads<R>; ++q)
      v[q] = __ldg(reinterpret_cast<const TVec<R> *>(t + q * kTraceLanes * kTVecN<R>));
  }
  __device__ __forceinline__ R
  operator()(int f) const
  {
    const TVec<R> & x = v[f / kTVecN<R>];
    if constexpr (sizeof(R) == 4)
    {
      const int c = f % 4;
      return c == 0 ? x.x : (c == 1 ? x.y : (c == 2 ? x.z : x.w));
    }
    else
      return f % 2 == 0 ? x.x : x.y;
  }
};

// Face state of a cell on its face normal to d (PLUS: the right face, the
// left state of that face), in the face frame the flux functor hands to the
// Riemann solver: normal velocity in IU and normal field in IA, with the
// reference's component swaps for y (IU<->IV, IA<->IB) and z (IU<->IW,
// IA<->IC) faces (trace_unsplit_mhd_3d_simpler, MHDBaseFunctor3D.h:905-955;
// MHDRunFunctors3D.h:1839-1874).
template <class R, bool PLUS, class ACC>
__device__ __forceinline__ void
face_state_acc(const ACC & T, int d, R (&q)[8], R smallr, R smallp)
{
  auto h = [&](int f) {
    const R c = T(f), s = T(t_hslope(d, f));
    return PLUS ? c + s : c - s;
  };
  auto tb = [&](int f) {
    const R c = T(T_A + f), s = T(t_bslope(d, f));
    return PLUS ? c + s : c - s;
  };
  q[ID] = h(T_R);
  q[IP] = h(T_P);
  q[IU] = h(T_U + d);
  q[IV] = h(d == 1 ? T_U : T_V);
  q[IW] = h(d == 2 ? T_U : T_W);
  q[IA] = T(t_bface(d, PLUS ? 1 : 0));
  q[IB] = tb(d == 1 ? 0 : 1);
  q[IC] = tb(d == 2 ? 0 : 2);
  floor_state(q, smallr, smallp);
}
template <class R, bool PLUS>
__device__ __forceinline__ void
face_state_dir(const R * t, int st, int d, R (&q)[8], R smallr, R smallp)
{
  face_state_acc<R, PLUS>(StrideAcc<R>{ t, st }, d, q, smallr, smallp);
}

// One corner of an edge along d (MHDBaseFunctor3D.h:957-1113).  The
// transverse directions are p1 = (d+1)%3 and p2 = (d+2)%3, the order in which
// compute_emf<emfDir> reads them; S1/S2 are the sides (+1 right, -1 left) of
// the corner along p1/p2.  Each sum keeps the reference's operands, so the
// result is bit-identical to the per-direction expressions.
template <class R, int S1, int S2, class ACC>
__device__ __forceinline__ EdgeCorner<R>
edge_corner_acc(const ACC & T, int d, int p1, int p2, R smallr, R smallp)
{
  auto sg1 = [](R x) { return S1 > 0 ? x : -x; };
  auto sg2 = [](R x) { return S2 > 0 ? x : -x; };
  auto hyd = [&](int f) { return T(f) + (sg1(T(t_hslope(p1, f))) + sg2(T(t_hslope(p2, f)))); };
  EdgeCorner<R> e;
  e.r = fmax(smallr, hyd(T_R));
  e.p = fmax(smallp, hyd(T_P));
  e.u = hyd(T_U + p1);
  e.v = hyd(T_U + p2);
  e.a = T(t_bface(p1, S1 > 0)) + sg2(T(t_bfslope(p1, S1 > 0, p2)));
  e.b = T(t_bface(p2, S2 > 0)) + sg1(T(t_bfslope(p2, S2 > 0, p1)));
  e.c = T(T_A + d) + (sg1(T(t_bslope(p1, d))) + sg2(T(t_bslope(p2, d))));
  return e;
}
template <class R, int S1, int S2>
__device__ __forceinline__ EdgeCorner<R>
edge_corner(const R * t, int st, int d, int p1, int p2, R smallr, R smallp)
{
  return edge_corner_acc<R, S1, S2>(StrideAcc<R>{ t, st }, d, p1, p2, smallr, smallp);
}

} // namespace EK_NS
