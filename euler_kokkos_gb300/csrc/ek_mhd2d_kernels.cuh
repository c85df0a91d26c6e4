// MHD 2D (SolverMHDMuscl<2>, implementationVersion 0) on GB300: two kernels
// per step.
//   1. mhd2d_dt_kernel    primitive variables of the boundary-mapped state and
//                         the CFL max-reduction (ConvertToPrimitivesFunctor2D_MHD
//                         + ComputeDtFunctor2D_MHD, MHDRunFunctors2D.h:16-160);
//                         the reference computes dt inside the step, after
//                         the ghost fill (SolverMHDMuscl.cpp:386-392)
//   2. mhd2d_step_kernel  one CTA per TX x TY output tile: face fields and
//                         primitives of the tile halo, the CT trace of the
//                         cells [i0-1, i0+TX] x [j0-1, j0+TY] kept as 30
//                         numbers per cell in shared memory, HLLD fluxes on
//                         the x and y faces, the 2D-HLLD emf on the z edges,
//                         then the hydro, Bz and face-field update
//                         (SolverMHDMuscl.cpp:369-420).
// The state is read from HBM in 1 and 2 and written once in 2.
#pragma once

#include "ek_mhd_kernels.cuh"

namespace EK_NS
{

// Compact 2D trace: trace_unsplit_mhd_2d (MHDBaseFunctor2D.h:775-1114)
// produces 4 face states and 4 edge states per cell, all simple combinations
// of these 30 numbers; the step kernel rebuilds each state from them with the
// reference's own expressions, so the result is bit-identical.
enum : int
{
  V_R = 0, V_P, V_U, V_V, V_W, V_A, V_B, V_C,      // advanced cell state
  V_AL, V_AR, V_BL, V_BR,                          // advanced face fields
  V_DRX, V_DPX, V_DUX, V_DVX, V_DWX, V_DCX, V_DBX, // half slopes along x
  V_DRY, V_DPY, V_DUY, V_DVY, V_DWY, V_DCY, V_DAY, // along y
  V_DALY, V_DBLX, V_DARY, V_DBRX,                  // face-field half slopes
  V_N
};

// 2D floors of the traced states (MHDBaseFunctor2D.h:1022-1113): rho >=
// smallr, p >= smallp * rho
template <class R>
__device__ __forceinline__ void
floor2d(R & r, R & p, R smallr, R smallp)
{
  r = fmax(smallr, r);
  p = fmax(smallp * r, p);
}

// Face state normal to d (0 x, 1 y) of a cell: PLUS is the left state of its
// right face (qm), otherwise the right state of its left face (qp); y states
// come in the face frame (IU<->IV and IA<->IB swapped) as the flux functor
// hands them to the Riemann solver (MHDRunFunctors2D.h:418-466).
template <class R, bool PLUS>
__device__ __forceinline__ void
face2d_state(const R * t, int st, int d, R (&q)[8], R smallr, R smallp)
{
  const int ds = V_DRX + 7 * d;
  auto      h = [&](int f) {
    const R c = t[f * st], s = t[(ds + f) * st];
    return PLUS ? c + s : c - s;
  };
  q[ID] = h(V_R);
  q[IP] = h(V_P);
  q[IU] = h(V_U + d);
  q[IV] = h(d == 1 ? V_U : V_V);
  q[IW] = h(V_W);
  q[IA] = t[(d == 0 ? (PLUS ? V_AR : V_AL) : (PLUS ? V_BR : V_BL)) * st];
  {
    // transverse in-plane field: B +- dBx (x faces), A +- dAy (y faces)
    const R c = t[(d == 0 ? V_B : V_A) * st], s = t[(ds + 6) * st];
    q[IB] = PLUS ? c + s : c - s;
  }
  {
    const R c = t[V_C * st], s = t[(ds + 5) * st];
    q[IC] = PLUS ? c + s : c - s;
  }
  floor2d(q[ID], q[IP], smallr, smallp);
}

// Edge state of a cell at its corner (S1 along x, S2 along y: +1 right/top,
// -1 left/bottom) with the components compute_emf<EMFZ> reads
// (MHDBaseFunctor2D.h:1061-1113).
template <class R, int S1, int S2>
__device__ __forceinline__ EdgeCorner<R>
edge2d_corner(const R * t, int st, R smallr, R smallp)
{
  auto sg1 = [](R x) { return S1 > 0 ? x : -x; };
  auto sg2 = [](R x) { return S2 > 0 ? x : -x; };
  auto hyd = [&](int f) { return t[f * st] + (sg1(t[(V_DRX + f) * st]) + sg2(t[(V_DRY + f) * st])); };
  EdgeCorner<R> e;
  e.r = hyd(V_R);
  e.p = hyd(V_P);
  floor2d(e.r, e.p, smallr, smallp);
  e.u = hyd(V_U);
  e.v = hyd(V_V);
  e.a = t[(S1 > 0 ? V_AR : V_AL) * st] + sg2(t[(S1 > 0 ? V_DARY : V_DALY) * st]);
  e.b = t[(S2 > 0 ? V_BR : V_BL) * st] + sg1(t[(S2 > 0 ? V_DBRX : V_DBLX) * st]);
  e.c = t[V_C * st] + (sg1(t[V_DCX * st]) + sg2(t[V_DCY * st]));
  return e;
}

// hydro variables of a mapped cell (reflect flips applied) and its Bz
template <class S, class R>
__device__ __forceinline__ void
load_mhd2d_cell(const MhdState<S> & m, const KParams & P, const SrcCell & s, R (&u)[5], double & bz)
{
  load_hydro<S, R>(m, P, s, u);
  bz = load_face<S>(m, P, s, 2);
}

// ---------------------------------------------------------------------------
// 1. CFL reduction of the step
// ---------------------------------------------------------------------------
template <class S, class R>
__global__ void __launch_bounds__(256, EK_MINB(R, 5, 2))
mhd2d_dt_kernel(const void * __restrict__ U, KParams P, DevClock * clk, int step,
                unsigned long long * key)
{
  if (clk)
  {
    const int s = step % 3;
    if (clk->sid[s] != step || clk->t[s] >= P.tEnd - 1e-14)
      return;
  }
  const MhdState<S> m = mhd_state<S>(U, P);
  const MhdConst<R> C = mhd_const<R>(P);
  R                 tmax = R(-INFINITY);
  for_interior_rows(P, [&](int i, int j, int) {
    const SrcCell s = src_cell(P, i, j, 0);
    R             u[5];
    double        bz;
    load_mhd2d_cell<S, R>(m, P, s, u, bz);
    const double bl0 = load_face<S>(m, P, s, 0), bl1 = load_face<S>(m, P, s, 1);
    const double br0 = load_face<S>(m, P, src_cell(P, i + 1, j, 0), 0);
    const double br1 = load_face<S>(m, P, src_cell(P, i, j + 1, 0), 1);
    R            bl[3] = { to_r<R>(bl0), to_r<R>(bl1), to_r<R>(bz) };
    R            br[3] = { to_r<R>(br0), to_r<R>(br1), R(0) };
    R            q[8];
    mhd_constoprim<R>(u, bl, br, q, C, [&](double (&a)[3], double (&b)[3]) {
      a[0] = bl0, a[1] = bl1, a[2] = bz;
      b[0] = br0, b[1] = br1, b[2] = 0.0;
    });
    // find_speed_info<TWO_D>: x and y only (mhd_utils.h:319-366)
    const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], cc = q[IC];
    const R b2 = a * a + b * b + cc * cc;
    R       cfx, cfy;
    if constexpr (sizeof(R) == 4)
    {
      const float id = rcp_a(d), c2 = C.gamma0 * p * id;
      const float d2 = 0.5f * (b2 * id + c2), cr = c2 * id;
      cfx = sqrt_a(d2 + sqrt_a(d2 * d2 - cr * a * a));
      cfy = sqrt_a(d2 + sqrt_a(d2 * d2 - cr * b * b));
      tmax = fmax(tmax, (cfx + fabsf(q[IU])) * P.idx + (cfy + fabsf(q[IV])) * P.idy);
    }
    else if constexpr (kShareRecip)
    {
      // FP64 FMA build: one reciprocal of the density, host-prepared 1/dx
      const R id = R(1) / d, c2 = C.gamma0 * p * id;
      const R d2 = R(0.5) * (b2 * id + c2), cr = c2 * id;
      cfx = sqrt(d2 + sqrt(d2 * d2 - cr * a * a));
      cfy = sqrt(d2 + sqrt(d2 * d2 - cr * b * b));
      tmax = fmax(tmax, (cfx + fabs(q[IU])) * P.idxd + (cfy + fabs(q[IV])) * P.idyd);
    }
    else
    {
      const R c2 = C.gamma0 * p / d;
      const R d2 = R(0.5) * (b2 / d + c2);
      cfx = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
      cfy = sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
      tmax = fmax(tmax, (cfx + fabs(q[IU])) / P.dx + (cfy + fabs(q[IV])) / P.dy);
    }
  });
  block_max_commit<256>(cand_key((double)tmax), key ? key : &clk->key[step % 3]);
  if (!key)
    finalize_step(clk, P, step); // dt and its ratios for the step kernel
}

// ---------------------------------------------------------------------------
// 2. fused step
// ---------------------------------------------------------------------------
template <int TX, int TY>
struct Mhd2dTile
{
  static constexpr int BX = TX + 5, BY = TY + 5; // face fields: cells [i0-2, i0+TX+2]
  static constexpr int QX = TX + 4, QY = TY + 4; // primitives:  cells [i0-2, i0+TX+1]
  static constexpr int XE = TX + 2, YE = TY + 2; // trace:       cells [i0-1, i0+TX]
  static constexpr int PL = XE * YE;
  static constexpr int FXS = (TX + 1) * TY, FYS = TX * (TY + 1), EZS = (TX + 1) * (TY + 1);
  // shared memory in elements of R: trace, then B + Q overlaid by fluxes + emf
  static constexpr int TRACE = V_N * PL;
  static constexpr int BQ = 2 * BX * BY + 8 * QX * QY;
  static constexpr int FE = 6 * (FXS + FYS) + EZS;
  static constexpr int TOTAL = TRACE + (BQ > FE ? BQ : FE);
};

template <class R>
constexpr size_t
mhd2d_smem(int TX, int TY)
{
  const int XE = TX + 2, YE = TY + 2, BQ = 2 * (TX + 5) * (TY + 5) + 8 * (TX + 4) * (TY + 4);
  const int FE = 6 * ((TX + 1) * TY + TX * (TY + 1)) + (TX + 1) * (TY + 1);
  return sizeof(R) * (V_N * XE * YE + (BQ > FE ? BQ : FE));
}

// trace_unsplit_mhd_2d (MHDBaseFunctor2D.h:775-1114) of the cell at Q tile
// coordinates (qx, qy) / B tile coordinates (bx, by), written as the compact
// trace with field stride ost.
template <class R, int TX, int TY>
__device__ __forceinline__ void
trace2d_compact(const R * sQ, const R * sB, int qx, int qy, int bx, int by, R dtdx, R dtdy,
                const MhdConst<R> & C, R * out, int ost)
{
  using T = Mhd2dTile<TX, TY>;
  auto Qv = [&](int v, int x, int y) { return sQ[(v * T::QY + y) * T::QX + x]; };
  auto Bv = [&](int c, int x, int y) { return sB[(c * T::BY + y) * T::BX + x]; };

  // edge electric fields around the cell (MHDBaseFunctor2D.h:816-835)
  R Ez[2][2];
#pragma unroll
  for (int di = 0; di < 2; ++di)
#pragma unroll
    for (int dj = 0; dj < 2; ++dj)
    {
      const int x0 = qx + di - 1, y0 = qy + dj - 1;
      const R   u = R(0.25) * (Qv(IU, x0, y0) + Qv(IU, x0, y0 + 1) + Qv(IU, x0 + 1, y0) + Qv(IU, x0 + 1, y0 + 1));
      const R   v = R(0.25) * (Qv(IV, x0, y0) + Qv(IV, x0, y0 + 1) + Qv(IV, x0 + 1, y0) + Qv(IV, x0 + 1, y0 + 1));
      const R   A = R(0.5) * (Bv(0, bx + di, by + dj - 1) + Bv(0, bx + di, by + dj));
      const R   B = R(0.5) * (Bv(1, bx + di - 1, by + dj) + Bv(1, bx + di, by + dj));
      Ez[di][dj] = u * B - v * A;
    }
  const R ELL = Ez[0][0], ELR = Ez[0][1], ERL = Ez[1][0], ERR = Ez[1][1];

  R q[8];
#pragma unroll
  for (int v = 0; v < 8; ++v)
    q[v] = Qv(v, qx, qy);
  R r = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW], A = q[IA], B = q[IB], Cc = q[IC];
  R AL = Bv(0, bx, by), AR = Bv(0, bx + 1, by), BL = Bv(1, bx, by), BR = Bv(1, bx, by + 1);

  // hydro slopes (slope_unsplit_hydro_2d, MHDBaseFunctor2D.h:346-404)
  const R st = C.slope_type;
  R       dqx[8], dqy[8];
#pragma unroll
  for (int vv = 0; vv < 8; ++vv)
  {
    dqx[vv] = slope1<R>(q[vv], Qv(vv, qx + 1, qy), Qv(vv, qx - 1, qy), st);
    dqy[vv] = slope1<R>(q[vv], Qv(vv, qx, qy + 1), Qv(vv, qx, qy - 1), st);
  }
  const R drx = dqx[ID] * R(0.5), dpx = dqx[IP] * R(0.5), dux = dqx[IU] * R(0.5), dvx = dqx[IV] * R(0.5),
          dwx = dqx[IW] * R(0.5), dCx = dqx[IC] * R(0.5), dBx = dqx[IB] * R(0.5);
  const R dry = dqy[ID] * R(0.5), dpy = dqy[IP] * R(0.5), duy = dqy[IU] * R(0.5), dvy = dqy[IV] * R(0.5),
          dwy = dqy[IW] * R(0.5), dCy = dqy[IC] * R(0.5), dAy = dqy[IA] * R(0.5);

  // transverse face-field slopes (slope_unsplit_mhd_2d, MHDBaseFunctor2D.h:455-518)
  const R dALy = R(0.5) * slope1<R>(Bv(0, bx, by), Bv(0, bx, by + 1), Bv(0, bx, by - 1), st);
  const R dBLx = R(0.5) * slope1<R>(Bv(1, bx, by), Bv(1, bx + 1, by), Bv(1, bx - 1, by), st);
  const R dARy = R(0.5) * slope1<R>(Bv(0, bx + 1, by), Bv(0, bx + 1, by + 1), Bv(0, bx + 1, by - 1), st);
  const R dBRx = R(0.5) * slope1<R>(Bv(1, bx, by + 1), Bv(1, bx + 1, by + 1), Bv(1, bx - 1, by + 1), st);

  const R dAx = R(0.5) * (AR - AL);
  const R dBy = R(0.5) * (BR - BL);
  const R gamma = C.gamma0;

  // source terms (MHDBaseFunctor2D.h:969-995)
  R su0, sv0, sw0;
  if constexpr (sizeof(R) == 4)
  {
    const float ir = rcp_a(r);
    su0 = (-u * dux - dpx * ir - B * dBx * ir - Cc * dCx * ir) * dtdx + (-v * duy + B * dAy * ir) * dtdy;
    sv0 = (-u * dvx + A * dBx * ir) * dtdx + (-v * dvy - dpy * ir - A * dAy * ir - Cc * dCy * ir) * dtdy;
    sw0 = (-u * dwx + A * dCx * ir) * dtdx + (-v * dwy + B * dCy * ir) * dtdy;
  }
  else
  {
    su0 = (-u * dux - dpx / r - B * dBx / r - Cc * dCx / r) * dtdx + (-v * duy + B * dAy / r) * dtdy;
    sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - Cc * dCy / r) * dtdy;
    sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy;
  }
  const R sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
  const R sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
  const R sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy;
  const R sB0 = (-u * dBx - B * dux + v * dAx + A * dvx) * dtdx;
  const R sC0 = (w * dAx + A * dwx - u * dCx - Cc * dux) * dtdx + (-v * dCy - Cc * dvy + w * dBy + B * dwy) * dtdy;
  const R sAL0 = +(ELR - ELL) * R(0.5) * dtdy;
  const R sAR0 = +(ERR - ERL) * R(0.5) * dtdy;
  const R sBL0 = -(ERL - ELL) * R(0.5) * dtdx;
  const R sBR0 = -(ERR - ELR) * R(0.5) * dtdx;

  R o[V_N];
  o[V_R] = r + sr0;
  o[V_U] = u + su0;
  o[V_V] = v + sv0;
  o[V_W] = w + sw0;
  o[V_P] = p + sp0;
  o[V_A] = A + sA0;
  o[V_B] = B + sB0;
  o[V_C] = Cc + sC0;
  o[V_AL] = AL + sAL0;
  o[V_AR] = AR + sAR0;
  o[V_BL] = BL + sBL0;
  o[V_BR] = BR + sBR0;
  o[V_DRX] = drx, o[V_DPX] = dpx, o[V_DUX] = dux, o[V_DVX] = dvx, o[V_DWX] = dwx, o[V_DCX] = dCx, o[V_DBX] = dBx;
  o[V_DRY] = dry, o[V_DPY] = dpy, o[V_DUY] = duy, o[V_DVY] = dvy, o[V_DWY] = dwy, o[V_DCY] = dCy, o[V_DAY] = dAy;
  o[V_DALY] = dALy, o[V_DBLX] = dBLx, o[V_DARY] = dARy, o[V_DBRX] = dBRx;
#pragma unroll
  for (int f = 0; f < V_N; ++f)
    out[f * ost] = o[f];
}

// One tile of the step: the cells [i0, i0+TX) x [j0, j0+TY) of tile (bx, by),
// written from the step's input state only.  REPAIR: the faces whose FP32
// HLLD star state is ill-conditioned are solved in FP64 (the repair kernel);
// otherwise such a face lists the tile for that kernel (repair list as in
// the 3D update kernel: [0] count, [1] blocks done, [2..3] tiles repaired,
// [4..] tiles).
template <class S, class R, int TX, int TY, int RS, bool REPAIR>
__device__ __forceinline__ void
mhd2d_tile(const void * __restrict__ Uin, void * __restrict__ Uout, const KParams & P, const StepConsts & sc,
           int bx, int by, int * repair)
{
  using T = Mhd2dTile<TX, TY>;
  constexpr int NT = TX * TY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R * sT = reinterpret_cast<R *>(smem_raw); // [V_N][YE][XE] compact trace
  R * sB = sT + T::TRACE;                   // [2][BY][BX] face fields IA, IB
  R * sQ = sB + 2 * T::BX * T::BY;          // [8][QY][QX] primitives
  R * sFx = sT + T::TRACE;                  // [6][TY][TX+1] x fluxes (over sB/sQ)
  R * sFy = sFx + 6 * T::FXS;               // [6][TY+1][TX]  y fluxes
  R * sE = sFy + 6 * T::FYS;                // [TY+1][TX+1]   z-edge emf

  const R           dtdx = to_r<R>(sc.dtdx), dtdy = to_r<R>(sc.dtdy);
  const double      ddtdx = sc.dtdx, ddtdy = sc.dtdy; // FP64 ratios of the face-field update
  const MhdConst<R> C = mhd_const<R>(P);
  const MhdState<S> m = mhd_state<S>(Uin, P);
  const int         gw = P.gw;
  const int         i0 = gw + bx * TX, j0 = gw + by * TY;

  // A. face fields IA, IB of cells [i0-2, i0+TX+2] x [j0-2, j0+TY+2]
  for (int c = threadIdx.x; c < T::BX * T::BY; c += NT)
  {
    const int     x = c % T::BX, y = c / T::BX;
    const SrcCell s = src_cell(P, i0 - 2 + x, j0 - 2 + y, 0);
    sB[(0 * T::BY + y) * T::BX + x] = to_r<R>(load_face<S>(m, P, s, 0));
    sB[(1 * T::BY + y) * T::BX + x] = to_r<R>(load_face<S>(m, P, s, 1));
  }
  __syncthreads();

  // B. primitives of cells [i0-2, i0+TX+1] x [j0-2, j0+TY+1]
  //    (ConvertToPrimitivesFunctor2D_MHD: right-face fields, zero z neighbour)
  for (int c = threadIdx.x; c < T::QX * T::QY; c += NT)
  {
    const int     x = c % T::QX, y = c / T::QX;
    const int     gi = i0 - 2 + x, gj = j0 - 2 + y;
    const SrcCell s = src_cell(P, gi, gj, 0);
    R             u[5], q[8];
    double        bz;
    load_mhd2d_cell<S, R>(m, P, s, u, bz);
    R bl[3] = { sB[(0 * T::BY + y) * T::BX + x], sB[(1 * T::BY + y) * T::BX + x], to_r<R>(bz) };
    R br[3] = { sB[(0 * T::BY + y) * T::BX + x + 1], sB[(1 * T::BY + y + 1) * T::BX + x], R(0) };
    mhd_constoprim<R>(u, bl, br, q, C, [&](double (&a)[3], double (&b)[3]) {
      a[0] = load_face<S>(m, P, s, 0);
      a[1] = load_face<S>(m, P, s, 1);
      a[2] = bz;
      b[0] = load_face<S>(m, P, src_cell(P, gi + 1, gj, 0), 0);
      b[1] = load_face<S>(m, P, src_cell(P, gi, gj + 1, 0), 1);
      b[2] = 0.0;
    });
#pragma unroll
    for (int v = 0; v < 8; ++v)
      sQ[(v * T::QY + y) * T::QX + x] = q[v];
  }
  __syncthreads();

  // C. compact trace of cells [i0-1, i0+TX] x [j0-1, j0+TY]
  for (int c = threadIdx.x; c < T::PL; c += NT)
  {
    const int x = c % T::XE, y = c / T::XE;
    trace2d_compact<R, TX, TY>(sQ, sB, x + 1, y + 1, x + 1, y + 1, dtdx, dtdy, C, sT + c, T::PL);
  }
  __syncthreads();

  // D. x- and y-face fluxes (padded to whole warps), then z-edge emfs
  //    (ComputeFluxesAndStoreFunctor2D_MHD, ComputeEmfAndStoreFunctor2D)
  const R   sr = C.smallr, sp = C.smallp;
  const int ihi = P.nx + gw, jhi = P.ny + gw;
  auto      TS = [&](int gi, int gj) { return sT + (gj - (j0 - 1)) * T::XE + (gi - (i0 - 1)); };
  constexpr int NF = T::FXS + T::FYS, NFP = (NF + 31) & ~31;
  // mixed HLLD: a face whose FP32 star state is ill-conditioned marks the tile
  constexpr bool kFlag = sizeof(R) == 4 && RS == 4 && !REPAIR;
  __shared__ int s_dirty;
  if (threadIdx.x == 0)
    s_dirty = 0;
  __syncthreads();
  // face work item w (x faces, then y faces)
  auto face = [&](int w) {
    const int d = w < T::FXS ? 0 : 1;
    const int f = d == 0 ? w : w - T::FXS;
    const int ex = TX + (d == 0 ? 1 : 0);
    const int i = i0 + f % ex, j = j0 + f / ex;
    if (i > ihi - (d != 0 ? 1 : 0) || j > jhi - (d != 1 ? 1 : 0))
      return;
    R ql[8], qr[8], fl[6];
    face2d_state<R, true>(TS(i - (d == 0), j - (d == 1)), T::PL, d, ql, sr, sp);
    face2d_state<R, false>(TS(i, j), T::PL, d, qr, sr, sp);
    if (!mhd_riemann<RS, R, 6>(ql, qr, fl, C.gamma0))
    {
      // ill-conditioned star state in FP32 (mixed HLLD only)
      if constexpr (REPAIR)
        mhd_hlld_f64_from_f32<6>(ql, qr, fl, C.gamma0);
      else
      {
        s_dirty = 1;
        return;
      }
    }
    R *       dst = d == 0 ? sFx : sFy;
    const int nd = d == 0 ? T::FXS : T::FYS;
#pragma unroll
    for (int v = 0; v < 6; ++v)
      dst[v * nd + f] = fl[v];
  };
  for (int w = threadIdx.x; w < NFP + T::EZS; w += NT)
  {
    if (w < NFP)
    {
      if (w >= NF)
        continue;
      face(w);
      continue;
    }
    // z edge at the low corner of cell (i,j): RT(i-1,j-1), RB(i-1,j), LT(i,j-1), LB(i,j)
    const int f = w - NFP;
    const int i = i0 + f % (TX + 1), j = j0 + f / (TX + 1);
    if (i > ihi || j > jhi)
      continue;
    const EdgeCorner<R> cRT = edge2d_corner<R, 1, 1>(TS(i - 1, j - 1), T::PL, sr, sp);
    const EdgeCorner<R> cRB = edge2d_corner<R, 1, -1>(TS(i - 1, j), T::PL, sr, sp);
    const EdgeCorner<R> cLT = edge2d_corner<R, -1, 1>(TS(i, j - 1), T::PL, sr, sp);
    const EdgeCorner<R> cLB = edge2d_corner<R, -1, -1>(TS(i, j), T::PL, sr, sp);
    sE[f] = mhd_emf_corners<R>(cRT, cRB, cLT, cLB, C.gamma0, C.smallc);
  }
  __syncthreads();
  // E. update (UpdateFunctor2D_MHD then UpdateEmfFunctor2D,
  //    MHDRunFunctors2D.h:1572-1700), in the reference's order per variable
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int gi = i0 + tx, gj = j0 + ty;
  if (gi < ihi && gj < jhi)
  {
    const long long st = P.vstride;
    const long long off = (long long)gj * P.isize + gi;
    const int       fx0 = ty * (TX + 1) + tx, fy0 = ty * TX + tx, e0 = ty * (TX + 1) + tx;
    R               u[5];
#pragma unroll
    for (int v = 0; v < 5; ++v)
      u[v] = (R)ldg(m.h + v * st + off);
    // flux components 0..4 = ID, IP, IU, IV, IW of the face frame, 5 = Bz
#pragma unroll
    for (int v = 0; v < 5; ++v)
      u[v] += sFx[v * T::FXS + fx0] * dtdx;
#pragma unroll
    for (int v = 0; v < 5; ++v)
      u[v] -= sFx[v * T::FXS + fx0 + 1] * dtdx;
    u[ID] += sFy[ID * T::FYS + fy0] * dtdy;
    u[IP] += sFy[IP * T::FYS + fy0] * dtdy;
    u[IU] += sFy[IV * T::FYS + fy0] * dtdy;
    u[IV] += sFy[IU * T::FYS + fy0] * dtdy;
    u[IW] += sFy[IW * T::FYS + fy0] * dtdy;
    u[ID] -= sFy[ID * T::FYS + fy0 + TX] * dtdy;
    u[IP] -= sFy[IP * T::FYS + fy0 + TX] * dtdy;
    u[IU] -= sFy[IV * T::FYS + fy0 + TX] * dtdy;
    u[IV] -= sFy[IU * T::FYS + fy0 + TX] * dtdy;
    u[IW] -= sFy[IW * T::FYS + fy0 + TX] * dtdy;
    S * hout = (S *)Uout;
#pragma unroll
    for (int v = 0; v < 5; ++v)
      hout[v * st + off] = (S)u[v];

    double * bout = sizeof(S) == 8 ? (double *)Uout + 5 * P.vstride : mixed_bfield(Uout, P);
    double   bx = m.b[0 * st + off], by = m.b[1 * st + off], bz = m.b[2 * st + off];
    const R  e00 = sE[e0], e01 = sE[e0 + TX + 1], e10 = sE[e0 + 1];
    if constexpr (sizeof(R) == 8)
    {
      bz += sFx[5 * T::FXS + fx0] * dtdx;
      bz -= sFx[5 * T::FXS + fx0 + 1] * dtdx;
      bz += sFy[5 * T::FYS + fy0] * dtdy;
      bz -= sFy[5 * T::FYS + fy0 + TX] * dtdy;
      bx += (e01 - e00) * dtdy;
      by -= (e10 - e00) * dtdx;
    }
    else
    {
      // FP64 island: the face fields (CT) accumulate in FP64 so div B stays at
      // FP64 round-off (one subtraction and one fused multiply-add each).  Bz
      // (cell-centred in 2D, outside div B) is advanced in FP32 like the
      // hydro variables; its storage stays FP64.
      float bzf = to_r<float>(bz);
      bzf += sFx[5 * T::FXS + fx0] * dtdx;
      bzf -= sFx[5 * T::FXS + fx0 + 1] * dtdx;
      bzf += sFy[5 * T::FYS + fy0] * dtdy;
      bzf -= sFy[5 * T::FYS + fy0 + TX] * dtdy;
      bz = f2d(bzf);
      bx = fma(f2d(e01) - f2d(e00), ddtdy, bx);
      by = fma(f2d(e00) - f2d(e10), ddtdx, by);
    }
    bout[0 * st + off] = bx;
    bout[1 * st + off] = by;
    bout[2 * st + off] = bz;
  }
  // s_dirty was last written before the barrier that ends phase D
  if (kFlag && threadIdx.x == 0 && s_dirty)
    repair[kRepairHead + atomicAdd(&repair[0], 1)] = by * ((P.nx + TX - 1) / TX) + bx;
}

// One launch per step: the tiles of the grid.  repair: the tile list of the
// mixed HLLD form (null otherwise), for the repair kernel that follows.
template <class S, class R, int TX, int TY, int RS>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_M2_MINB_F32, EK_M2_MINB_F64))
mhd2d_step_kernel(const void * __restrict__ Uin, void * __restrict__ Uout, KParams P, DevClock * clk,
                  int step, int * repair)
{
  StepConsts sc;
  if (!step_consts(clk, step, sc))
    return;
  mhd2d_tile<S, R, TX, TY, RS, false>(Uin, Uout, P, sc, blockIdx.x, blockIdx.y, repair);
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0)
    step_commit(clk, step, sc.t, sc.dt);
}

// After the step kernel of the mixed HLLD form: recomputes the tiles it
// listed with the ill-conditioned faces solved in FP64 (tiles are independent
// within a step, so this replaces their output), then clears the list.
template <class S, class R, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_M2_MINB_F32, EK_M2_MINB_F64))
mhd2d_repair_kernel(const void * __restrict__ Uin, void * __restrict__ Uout, KParams P, DevClock * clk,
                    int step, int * repair)
{
  StepConsts sc;
  if (!step_consts(clk, step, sc))
    return;
  const int n = repair[0];
  const int gx = (P.nx + TX - 1) / TX;
  for (int e = blockIdx.x; e < n; e += gridDim.x)
  {
    const int tile = repair[kRepairHead + e];
    mhd2d_tile<S, R, TX, TY, 4, true>(Uin, Uout, P, sc, tile % gx, tile / gx, repair);
    __syncthreads(); // shared memory of the next tile
  }
  repair_list_release(repair);
}

constexpr int M2_TX = EK_M2_TX, M2_TY = EK_M2_TY;

inline long long
mhd2d_tiles(const KParams & P)
{
  return (long long)((P.nx + M2_TX - 1) / M2_TX) * ((P.ny + M2_TY - 1) / M2_TY);
}

template <class S, class R>
cudaError_t
mhd2d_step_t(int phase, const void * Uin, void * Uout, void * work, const KParams & P, DevClock * clk,
             int step, cudaStream_t st)
{
  if (phase == 0)
  {
    mhd2d_dt_kernel<S, R><<<row_blocks(P), 256, 0, st>>>(Uin, P, clk, step, nullptr);
    return cudaGetLastError();
  }
  // the repair pass of the mixed HLLD form (after phase 1)
  if (phase == 2)
  {
    if constexpr (sizeof(R) == 8)
      return cudaErrorNotSupported;
    else
    {
      if (P.riemann != 4)
        return cudaErrorNotSupported;
      auto        k = mhd2d_repair_kernel<S, R, M2_TX, M2_TY>;
      const int   sm = (int)mhd2d_smem<R>(M2_TX, M2_TY);
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      if (e != cudaSuccess)
        return e;
      k<<<repair_grid(mhd2d_tiles(P)), M2_TX * M2_TY, sm, st>>>(Uin, Uout, P, clk, step, (int *)work);
      return cudaGetLastError();
    }
  }
  auto k = P.riemann == 1   ? mhd2d_step_kernel<S, R, M2_TX, M2_TY, 1>
           : P.riemann == 2 ? mhd2d_step_kernel<S, R, M2_TX, M2_TY, 2>
                            : mhd2d_step_kernel<S, R, M2_TX, M2_TY, 4>;
  const int   sm = (int)mhd2d_smem<R>(M2_TX, M2_TY);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
  if (e != cudaSuccess)
    return e;
  dim3  grid((P.nx + M2_TX - 1) / M2_TX, (P.ny + M2_TY - 1) / M2_TY, 1);
  int * repair = sizeof(R) == 4 && P.riemann == 4 ? (int *)work : nullptr;
  k<<<grid, M2_TX * M2_TY, sm, st>>>(Uin, Uout, P, clk, step, repair);
  return cudaGetLastError();
}

// the repair pass's tile list of the mixed form (cleared by the caller before
// the first step)
size_t
mhd2d_work_bytes(int prec, const KParams & P)
{
  return prec == 0 ? 0 : sizeof(int) * (size_t)(kRepairHead + mhd2d_tiles(P));
}

// one MHD 2D step = phase 0 (CFL), 1 (fused trace, fluxes, emf, update),
// 2 (the repair pass, mixed HLLD form)
cudaError_t
mhd2d_step(int prec, int phase, const void * Uin, void * Uout, void * work, const KParams & P, DevClock * clk,
           int step, cudaStream_t st)
{
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  return mhd2d_step_t<double, double>(phase, Uin, Uout, work, P, clk, step, st);
#else
  if (prec == 0)
    return mhd2d_step_t<double, double>(phase, Uin, Uout, work, P, clk, step, st);
  return mhd2d_step_t<float, float>(phase, Uin, Uout, work, P, clk, step, st);
#endif
}

cudaError_t
mhd2d_dt(int prec, const void * U, const KParams & P, unsigned long long * key, cudaStream_t st)
{
  const int blocks = row_blocks(P);
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  mhd2d_dt_kernel<double, double><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
#else
  if (prec == 0)
    mhd2d_dt_kernel<double, double><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
  else
    mhd2d_dt_kernel<float, float><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
#endif
  return cudaGetLastError();
}

} // namespace EK_NS
