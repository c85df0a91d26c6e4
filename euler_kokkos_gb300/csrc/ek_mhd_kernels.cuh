// CT-MHD 3D step (SolverMHDMuscl<3>::godunov_unsplit_impl v0,
// SolverMHDMuscl.cpp:461-505) in two launches, plus the CFL kernel before
// the first step:
//   1. mhd_dt_kernel     primitive variables of the boundary-mapped state and
//                        the CFL max-reduction (ComputeDtFunctor3D_MHD); the
//                        reference computes MHD dt inside the step, after the
//                        ghost fill (SolverMHDMuscl.cpp:479-484).  Launched for
//                        the first step only: every update kernel computes the
//                        next step's CFL from the cells it has just updated
//   2. mhd_trace_kernel  z-marching: face-field planes, primitive planes and
//                        edge electric fields in shared memory, limited
//                        slopes, CT half-step trace -> 47 numbers per cell
//   3. mhd_update_kernel z-marching: HLLD fluxes (3 faces), 2D-HLLD emfs
//                        (3 edges), conservative update and CT update of the
//                        face fields, all from the compact trace; then the
//                        CFL candidates of the updated cells (their high
//                        faces at tile edges and domain ends are updated
//                        redundantly, or follow the boundary condition as the
//                        next step's ghost fill would) and the next step's dt
// The state is read from HBM in 2 and 3 and written once in 3.
#pragma once

#include "ek_mhd.cuh"
#include "ek_worklist.h"

namespace EK_NS
{

template <class R>
__device__ __forceinline__ MhdConst<R>
mhd_const(const KParams & P)
{
  MhdConst<R> C;
  if constexpr (sizeof(R) == 8)
  {
    C.gamma0 = P.gamma0;
    C.smallr = P.smallr;
    C.smallp = P.smallp;
    C.smallc = P.smallc;
    C.slope_type = P.slope_type;
  }
  else
  {
    C.gamma0 = P.gamma0f;
    C.smallr = P.smallrf;
    C.smallp = P.smallpf;
    C.smallc = P.smallcf;
    C.slope_type = P.slopef;
  }
  return C;
}

// Compact trace in HBM, blocked by 32 cells along x: the trace cells are
// [gw-1, n+gw] in each direction (trace-local it, jt, kt from 0); a block holds
// 32 consecutive cells of one row as 16-byte quads of fields, quad after quad
// ([quad][32 cells][4 floats or 2 doubles]), and blocks follow in
// (it / 32, jt, kt) order.  A cell's fields therefore sit at compile-time
// offsets from the cell's own address, four (two) per 16-byte vector load:
// gathering a face or edge state costs one address computation per cell and
// one load per quad (a field-major layout over the whole grid needs a 64-bit
// product per field).  A warp reading one quad of 32 consecutive cells reads
// 512 contiguous bytes.
struct TraceGrid
{
  int nb; // blocks per row: ceil((nx + 2) / 32)
  int nj; // rows per plane: ny + 2
};
__host__ __device__ inline TraceGrid
trace_grid(const KParams & P)
{
  return TraceGrid{ (P.nx + 2 + kTraceLanes - 1) / kTraceLanes, P.ny + 2 };
}
// address of the first field of the cell with global indices (i, j, k)
// elements of one 32-cell block (the same for FP32 and FP64: 48 fields)
template <class R>
constexpr int kTraceBlock = kTQuads<R> * kTraceLanes * kTVecN<R>;
template <class R>
__device__ __forceinline__ R *
trace_cell(R * trace, const TraceGrid & g, int gw, int i, int j, int k)
{
  // trace-local indices are never negative: unsigned division and remainder
  // by 32 are a shift and a mask
  const unsigned it = (unsigned)(i - (gw - 1)), jt = (unsigned)(j - (gw - 1)), kt = (unsigned)(k - (gw - 1));
  const long long b = ((long long)kt * g.nj + jt) * g.nb + (it / kTraceLanes);
  return trace + b * kTraceBlock<R> + (it % kTraceLanes) * kTVecN<R>;
}
// element offset of field f from its cell's address
template <class R>
__host__ __device__ constexpr int
trace_field(int f)
{
  return (f / kTVecN<R>) * (kTraceLanes * kTVecN<R>) + f % kTVecN<R>;
}

// a direction as a type (compile-time specialisation of a gather)
template <int V>
struct DirC
{
  static constexpr int value = V;
};

// state accessors: hydro planes of type S, face-field planes always FP64
template <class S>
struct MhdState
{
  const S *      h; // 5 hydro planes
  const double * b; // 3 face-field planes
};
template <class S>
__device__ __forceinline__ MhdState<S>
mhd_state(const void * U, const KParams & P)
{
  MhdState<S> m;
  m.h = (const S *)U;
  if constexpr (sizeof(S) == 8)
    m.b = (const double *)U + 5 * P.vstride;
  else
    m.b = mixed_bfield(U, P);
  return m;
}

// hydro variables of a (mapped) cell, reflect flips applied
template <class S, class R>
__device__ __forceinline__ void
load_hydro(const MhdState<S> & m, const KParams & P, const SrcCell & s, R (&u)[5])
{
#pragma unroll
  for (int v = 0; v < 5; ++v)
  {
    u[v] = neg_if((R)ldg(m.h + v * P.vstride + s.off), flips(s, v, 1));
  }
}
template <class S>
__device__ __forceinline__ double
load_face(const MhdState<S> & m, const KParams & P, const SrcCell & s, int comp)
{
  return neg_if(ldg(m.b + comp * P.vstride + s.off), flips(s, IA + comp, 1));
}

// primitive state of cell (gi,gj,gk): constoprim with the face fields of the
// cell and of its +1 neighbours (ConvertToPrimitivesFunctor3D_MHD)
template <class S, class R>
__device__ __forceinline__ void
cell_prims_global(const MhdState<S> & m, const KParams & P, const MhdConst<R> & C, int gi, int gj,
                  int gk, R (&q)[8])
{
  const SrcCell s = src_cell(P, gi, gj, gk);
  R             u[5];
  load_hydro<S, R>(m, P, s, u);
  double bl[3], br[3];
  bl[0] = load_face<S>(m, P, s, 0);
  bl[1] = load_face<S>(m, P, s, 1);
  bl[2] = load_face<S>(m, P, s, 2);
  br[0] = load_face<S>(m, P, src_cell(P, gi + 1, gj, gk), 0);
  br[1] = load_face<S>(m, P, src_cell(P, gi, gj + 1, gk), 1);
  br[2] = load_face<S>(m, P, src_cell(P, gi, gj, gk + 1), 2);
  R blr[3], brr[3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
  {
    blr[c] = to_r<R>(bl[c]);
    brr[c] = to_r<R>(br[c]);
  }
  mhd_constoprim<R>(u, blr, brr, q, C, [&](double (&a)[3], double (&b)[3]) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      a[c] = bl[c];
      b[c] = br[c];
    }
  });
}

// ---------------------------------------------------------------------------
// 1. CFL reduction of the step (on the primitive variables of the input)
// ---------------------------------------------------------------------------
template <class S, class R>
__global__ void __launch_bounds__(256, EK_MINB(R, 5, 2))
mhd_dt_kernel(const void * __restrict__ U, KParams P, DevClock * clk, int step,
              unsigned long long * key)
{
  if (clk)
  {
    // a step that must not run (finished, or an earlier one did not run)
    const int s = step % 3;
    if (clk->sid[s] != step || clk->t[s] >= P.tEnd - 1e-14)
      return;
  }
  const MhdState<S> m = mhd_state<S>(U, P);
  const MhdConst<R> C = mhd_const<R>(P);
  R                 tmax = R(-INFINITY);
  for_interior_rows(P, [&](int i, int j, int k) {
    R q[8];
    cell_prims_global<S, R>(m, P, C, i, j, k, q);
    tmax = fmax(tmax, mhd_invdt<R>(q, C.gamma0, P.dx, P.dy, P.dz, P.idx, P.idy, P.idz, P.idxd, P.idyd, P.idzd));
  });
  block_max_commit<256>(cand_key((double)tmax), key ? key : &clk->key[step % 3]);
  if (!key)
    finalize_step(clk, P, step); // dt and its ratios for the trace and update kernels
}

// ---------------------------------------------------------------------------
// 2. trace kernel
// ---------------------------------------------------------------------------
// Tile of trace cells [c0, c0+TX) x [d0, d0+TY) (global indices), marching
// over planes [k0, k1).  Shared planes (x extent / y extent):
//   sB  face fields, 4 planes (k-1..k+2), x in [c0-1, c0+TX+1], y in [d0-1, d0+TY+1]
//   sQ  primitives,  3 planes (k-1..k+1), x in [c0-1, c0+TX],   y in [d0-1, d0+TY]
//   sE  edge fields, 2 planes (k, k+1),   x in [c0,   c0+TX],   y in [d0,   d0+TY]
template <int TX, int TY>
struct TraceTile
{
  static constexpr int BX = TX + 3, BY = TY + 3, BP = 3 * BX * BY;
  static constexpr int QX = TX + 2, QY = TY + 2, QP = 8 * QX * QY;
  static constexpr int EX = TX + 1, EY = TY + 1, EP = 3 * EX * EY;
};

template <class R, int TX, int TY>
__device__ __forceinline__ void
trace_cell_compact(const R * sB, int bslot[4], const R * sQ, int qslot[3], const R * sE,
                   int eslot[2], int tx, int ty, R dtdx, R dtdy, R dtdz, const MhdConst<R> & C,
                   R * out)
{
  using T = TraceTile<TX, TY>;
  // local tile coordinates of the cell in each buffer
  const int qx = tx + 1, qy = ty + 1; // sQ
  const int bx = tx + 1, by = ty + 1; // sB
  const int ex = tx, ey = ty;         // sE
  const R * Q0 = sQ + qslot[1] * T::QP;
  const R * Qm = sQ + qslot[0] * T::QP;
  const R * Qp = sQ + qslot[2] * T::QP;
  auto Qv = [&](const R * pl, int v, int x, int y) { return pl[(v * T::QY + y) * T::QX + x]; };
  auto Bv = [&](int slot, int comp, int x, int y) {
    return sB[bslot[slot] * T::BP + (comp * T::BY + y) * T::BX + x];
  };
  auto Ev = [&](int slot, int comp, int x, int y) {
    return sE[eslot[slot] * T::EP + (comp * T::EY + y) * T::EX + x];
  };

  // hydro slopes (slope_unsplit_hydro_3d, MHDBaseFunctor3D.h:340-470); the
  // z-slope of IC uses qMinusY as the reference does (unused by the trace)
  R q[8], dq[3][8];
#pragma unroll
  for (int v = 0; v < 8; ++v)
    q[v] = Qv(Q0, v, qx, qy);
  if (C.slope_type == R(1) || C.slope_type == R(2))
  {
#pragma unroll
    for (int v = 0; v < 8; ++v)
    {
      dq[0][v] = slope1<R>(q[v], Qv(Q0, v, qx + 1, qy), Qv(Q0, v, qx - 1, qy), C.slope_type);
      dq[1][v] = slope1<R>(q[v], Qv(Q0, v, qx, qy + 1), Qv(Q0, v, qx, qy - 1), C.slope_type);
      dq[2][v] = slope1<R>(q[v], Qv(Qp, v, qx, qy), v == IC ? Qv(Q0, v, qx, qy - 1) : Qv(Qm, v, qx, qy),
                           C.slope_type);
    }
  }
  else
  {
#pragma unroll
    for (int v = 0; v < 8; ++v)
      dq[0][v] = dq[1][v] = dq[2][v] = R(0);
  }
  // face fields of the cell (bfNb, MHDRunFunctors3D.h:790-795); planes: 0 k-1, 1 k, 2 k+1
  const R AL = (R)Bv(1, 0, bx, by), AR = (R)Bv(1, 0, bx + 1, by);
  const R BL = (R)Bv(1, 1, bx, by), BR = (R)Bv(1, 1, bx, by + 1);
  const R CL = (R)Bv(1, 2, bx, by), CR = (R)Bv(2, 2, bx, by);
  // transverse face-field slopes (slope_unsplit_mhd_3d, MHDBaseFunctor3D.h:563-668)
  const R xst = fmin(C.slope_type, R(2.0));
  auto    sA = [&](int x, int y, bool zdir) {
    const R b = (R)Bv(1, 0, x, y);
    return zdir ? slope1<R>(b, (R)Bv(2, 0, x, y), (R)Bv(0, 0, x, y), xst)
                   : slope1<R>(b, (R)Bv(1, 0, x, y + 1), (R)Bv(1, 0, x, y - 1), xst);
  };
  auto sBf = [&](int x, int y, bool zdir) {
    const R b = (R)Bv(1, 1, x, y);
    return zdir ? slope1<R>(b, (R)Bv(2, 1, x, y), (R)Bv(0, 1, x, y), xst)
                : slope1<R>(b, (R)Bv(1, 1, x + 1, y), (R)Bv(1, 1, x - 1, y), xst);
  };
  auto sC = [&](int slot, int x, int y, bool ydir) {
    const R b = (R)Bv(slot, 2, x, y);
    return ydir ? slope1<R>(b, (R)Bv(slot, 2, x, y + 1), (R)Bv(slot, 2, x, y - 1), xst)
                : slope1<R>(b, (R)Bv(slot, 2, x + 1, y), (R)Bv(slot, 2, x - 1, y), xst);
  };
  R dbf[12];
  dbf[0] = sA(bx, by, false);      // DeltaA(i,j,k).y
  dbf[1] = sA(bx, by, true);       // DeltaA(i,j,k).z
  dbf[2] = sBf(bx, by, false);     // DeltaB(i,j,k).x
  dbf[3] = sBf(bx, by, true);      // DeltaB(i,j,k).z
  dbf[4] = sC(1, bx, by, false);   // DeltaC(i,j,k).x
  dbf[5] = sC(1, bx, by, true);    // DeltaC(i,j,k).y
  dbf[6] = sA(bx + 1, by, false);  // DeltaA(i+1,j,k).y
  dbf[7] = sA(bx + 1, by, true);   // DeltaA(i+1,j,k).z
  dbf[8] = sBf(bx, by + 1, false); // DeltaB(i,j+1,k).x
  dbf[9] = sBf(bx, by + 1, true);  // DeltaB(i,j+1,k).z
  dbf[10] = sC(2, bx, by, false);  // DeltaC(i,j,k+1).x
  dbf[11] = sC(2, bx, by, true);   // DeltaC(i,j,k+1).y
  // edge electric fields around the cell (MHDRunFunctors3D.h:808-823)
  const R ELL = Ev(0, 0, ex, ey), ELR = Ev(1, 0, ex, ey), ERL = Ev(0, 0, ex, ey + 1),
          ERR = Ev(1, 0, ex, ey + 1);
  const R FLL = Ev(0, 1, ex, ey), FLR = Ev(1, 1, ex, ey), FRL = Ev(0, 1, ex + 1, ey),
          FRR = Ev(1, 1, ex + 1, ey);
  const R GLL = Ev(0, 2, ex, ey), GLR = Ev(0, 2, ex, ey + 1), GRL = Ev(0, 2, ex + 1, ey),
          GRR = Ev(0, 2, ex + 1, ey + 1);

  // trace_unsplit_mhd_3d_simpler (MHDBaseFunctor3D.h:751-917), Omega0 = 0
  R r = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW], A = q[IA], B = q[IB], Cc = q[IC];
  const R drx = dq[0][ID] * R(0.5), dpx = dq[0][IP] * R(0.5), dux = dq[0][IU] * R(0.5),
          dvx = dq[0][IV] * R(0.5), dwx = dq[0][IW] * R(0.5), dCx = dq[0][IC] * R(0.5),
          dBx = dq[0][IB] * R(0.5);
  const R dry = dq[1][ID] * R(0.5), dpy = dq[1][IP] * R(0.5), duy = dq[1][IU] * R(0.5),
          dvy = dq[1][IV] * R(0.5), dwy = dq[1][IW] * R(0.5), dCy = dq[1][IC] * R(0.5),
          dAy = dq[1][IA] * R(0.5);
  const R drz = dq[2][ID] * R(0.5), dpz = dq[2][IP] * R(0.5), duz = dq[2][IU] * R(0.5),
          dvz = dq[2][IV] * R(0.5), dwz = dq[2][IW] * R(0.5), dAz = dq[2][IA] * R(0.5),
          dBz = dq[2][IB] * R(0.5);
  const R dALy = R(0.5) * dbf[0], dALz = R(0.5) * dbf[1], dBLx = R(0.5) * dbf[2],
          dBLz = R(0.5) * dbf[3], dCLx = R(0.5) * dbf[4], dCLy = R(0.5) * dbf[5];
  const R dARy = R(0.5) * dbf[6], dARz = R(0.5) * dbf[7], dBRx = R(0.5) * dbf[8],
          dBRz = R(0.5) * dbf[9], dCRx = R(0.5) * dbf[10], dCRy = R(0.5) * dbf[11];
  const R dAx = R(0.5) * (AR - AL);
  const R dBy = R(0.5) * (BR - BL);
  const R dCz = R(0.5) * (CR - CL);
  const R gamma = C.gamma0;
  const R C_ = Cc;
  const R sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
  R su0, sv0, sw0;
  if constexpr (sizeof(R) == 4 || kShareRecip)
  {
    // one reciprocal of the density (FP32: approximate; FP64 FMA build: exact
    // reciprocal, then products); the exact build divides below
    R ir;
    if constexpr (sizeof(R) == 4)
      ir = rcp_a(r);
    else
      ir = R(1) / r;
    su0 = (-u * dux - (dpx + B * dBx + C_ * dCx) * ir) * dtdx + (-v * duy + B * dAy * ir) * dtdy +
          (-w * duz + C_ * dAz * ir) * dtdz;
    sv0 = (-u * dvx + A * dBx * ir) * dtdx + (-v * dvy - (dpy + A * dAy + C_ * dCy) * ir) * dtdy +
          (-w * dvz + C_ * dBz * ir) * dtdz;
    sw0 = (-u * dwx + A * dCx * ir) * dtdx + (-v * dwy + B * dCy * ir) * dtdy +
          (-w * dwz - (dpz + A * dAz + B * dBz) * ir) * dtdz;
  }
  else
  {
    su0 = (-u * dux - (dpx + B * dBx + C_ * dCx) / r) * dtdx + (-v * duy + B * dAy / r) * dtdy +
          (-w * duz + C_ * dAz / r) * dtdz;
    sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + C_ * dCy) / r) * dtdy +
          (-w * dvz + C_ * dBz / r) * dtdz;
    sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
          (-w * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
  }
  const R sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
                (-w * dpz - dwz * gamma * p) * dtdz;
  const R sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy + (u * dCz + C_ * duz - w * dAz - A * dwz) * dtdz;
  const R sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx + (v * dCz + C_ * dvz - w * dBz - B * dwz) * dtdz;
  const R sC0 = (w * dAx + A * dwx - u * dCx - C_ * dux) * dtdx + (w * dBy + B * dwy - v * dCy - C_ * dvy) * dtdy;
  const R sAL0 = +(GLR - GLL) * dtdy * R(0.5) - (FLR - FLL) * dtdz * R(0.5);
  const R sAR0 = +(GRR - GRL) * dtdy * R(0.5) - (FRR - FRL) * dtdz * R(0.5);
  const R sBL0 = -(GRL - GLL) * dtdx * R(0.5) + (ELR - ELL) * dtdz * R(0.5);
  const R sBR0 = -(GRR - GLR) * dtdx * R(0.5) + (ERR - ERL) * dtdz * R(0.5);
  const R sCL0 = +(FRL - FLL) * dtdx * R(0.5) - (ERL - ELL) * dtdy * R(0.5);
  const R sCR0 = +(FRR - FLR) * dtdx * R(0.5) - (ERR - ELR) * dtdy * R(0.5);

  R o[T_N];
  o[T_R] = r + sr0;
  o[T_U] = u + su0;
  o[T_V] = v + sv0;
  o[T_W] = w + sw0;
  o[T_P] = p + sp0;
  o[T_A] = A + sA0;
  o[T_B] = B + sB0;
  o[T_C] = C_ + sC0;
  o[T_AL] = AL + sAL0;
  o[T_AR] = AR + sAR0;
  o[T_BL] = BL + sBL0;
  o[T_BR] = BR + sBR0;
  o[T_CL] = CL + sCL0;
  o[T_CR] = CR + sCR0;
  o[T_DRX] = drx, o[T_DPX] = dpx, o[T_DUX] = dux, o[T_DVX] = dvx, o[T_DWX] = dwx, o[T_DBX] = dBx,
  o[T_DCX] = dCx;
  o[T_DRY] = dry, o[T_DPY] = dpy, o[T_DUY] = duy, o[T_DVY] = dvy, o[T_DWY] = dwy, o[T_DAY] = dAy,
  o[T_DCY] = dCy;
  o[T_DRZ] = drz, o[T_DPZ] = dpz, o[T_DUZ] = duz, o[T_DVZ] = dvz, o[T_DWZ] = dwz, o[T_DAZ] = dAz,
  o[T_DBZ] = dBz;
  o[T_DALY] = dALy, o[T_DALZ] = dALz, o[T_DBLX] = dBLx, o[T_DBLZ] = dBLz, o[T_DCLX] = dCLx,
  o[T_DCLY] = dCLy;
  o[T_DARY] = dARy, o[T_DARZ] = dARz, o[T_DBRX] = dBRx, o[T_DBRZ] = dBRz, o[T_DCRX] = dCRx,
  o[T_DCRY] = dCRy;
  // one 16-byte store per quad (the last quad's spare fields are zero)
#pragma unroll
  for (int q = 0; q < kTQuads<R>; ++q)
  {
    R w[kTVecN<R>];
#pragma unroll
    for (int c = 0; c < kTVecN<R>; ++c)
      w[c] = q * kTVecN<R> + c < T_N ? o[q * kTVecN<R> + c] : R(0);
    TVec<R> x;
    if constexpr (sizeof(R) == 4)
      x = make_float4(w[0], w[1], w[2], w[3]);
    else
      x = make_double2(w[0], w[1]);
    *reinterpret_cast<TVec<R> *>(out + q * kTraceLanes * kTVecN<R>) = x;
  }
}

template <class S, class R, int TX, int TY>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_MT_MINB_F32, EK_MT_MINB_F64))
mhd_trace_kernel(const void * __restrict__ U, R * __restrict__ trace, KParams P, DevClock * clk,
                 int step)
{
  using T = TraceTile<TX, TY>;
  constexpr int NT = TX * TY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // raw copies of the next face-field plane (FP64) and hydro plane (storage
  // type S), landed by asynchronous copies one plane ahead
  double * rawB = reinterpret_cast<double *>(smem_raw); // [3][BY][BX]
  S *      rawU = reinterpret_cast<S *>(rawB + T::BP);  // [5][QY][QX]
  R * sB = reinterpret_cast<R *>(rawU + 5 * T::QX * T::QY); // [4][3][BY][BX] face fields (storage precision R)
  R * sQ = sB + 4 * T::BP;                  // [3][8][QY][QX]
  R *      sE = sQ + 3 * T::QP;                                // [2][3][EY][EX]

  StepConsts sc;
  if (!step_consts(clk, step, sc))
    return;
  const R           dtdx = to_r<R>(sc.dtdx), dtdy = to_r<R>(sc.dtdy), dtdz = to_r<R>(sc.dtdz);
  const MhdConst<R> C = mhd_const<R>(P);
  const MhdState<S> m = mhd_state<S>(U, P);
  const int gw = P.gw;
  // trace cells span global [gw-1, n+gw] in each direction
  const int c0 = gw - 1 + blockIdx.x * TX, d0 = gw - 1 + blockIdx.y * TY;
  const int k0 = gw - 1 + blockIdx.z * P.kchunk;
  const int k1 = min(k0 + P.kchunk, P.nz + gw + 1);
  const int nti = P.nx + 2, ntj = P.ny + 2; // trace cells per row / column
  // planes whose gathered x/y window [c0-1, c0+TX+1] x [d0-1, d0+TY+1] lies in
  // the interior need no boundary mapping: plain offsets, no sign flips
  const bool xy_in = c0 - 1 >= gw && c0 + TX + 1 < P.nx + gw && d0 - 1 >= gw && d0 + TY + 1 < P.ny + gw;
  auto src = [&](int gi, int gj, int gk) -> SrcCell {
    if (xy_in && gk >= gw && gk < P.nz + gw)
    {
      SrcCell s;
      s.off = (long long)gk * P.plane + (long long)gj * P.isize + gi;
      s.fx = s.fy = s.fz = false;
      return s;
    }
    return src_cell(P, gi, gj, gk);
  };

  auto load_B = [&](int gk, int slot) {
    R * dst = sB + slot * T::BP;
    for (int c = threadIdx.x; c < T::BX * T::BY; c += NT)
    {
      const int     x = c % T::BX, y = c / T::BX;
      const SrcCell s = src(c0 - 1 + x, d0 - 1 + y, gk);
#pragma unroll
      for (int comp = 0; comp < 3; ++comp)
        dst[(comp * T::BY + y) * T::BX + x] = to_r<R>(load_face<S>(m, P, s, comp));
    }
  };
  // the same plane through rawB: issue the copies, then (after this thread's
  // cp.async.wait_all) convert the cells this thread copied
  auto issue_B = [&](int gk) {
    for (int c = threadIdx.x; c < T::BX * T::BY; c += NT)
    {
      const int     x = c % T::BX, y = c / T::BX;
      const SrcCell s = src(c0 - 1 + x, d0 - 1 + y, gk);
#pragma unroll
      for (int comp = 0; comp < 3; ++comp)
        cp_async<8>(rawB + (comp * T::BY + y) * T::BX + x, m.b + comp * P.vstride + s.off);
    }
  };
  auto convert_B = [&](int gk, int slot) {
    R * dst = sB + slot * T::BP;
    for (int c = threadIdx.x; c < T::BX * T::BY; c += NT)
    {
      const int     x = c % T::BX, y = c / T::BX;
      const SrcCell s = src(c0 - 1 + x, d0 - 1 + y, gk);
#pragma unroll
      for (int comp = 0; comp < 3; ++comp)
      {
        const int i = (comp * T::BY + y) * T::BX + x;
        dst[i] = to_r<R>(neg_if(rawB[i], flips(s, IA + comp, 1)));
      }
    }
  };
  auto issue_U = [&](int gk) {
    for (int c = threadIdx.x; c < T::QX * T::QY; c += NT)
    {
      const int     x = c % T::QX, y = c / T::QX;
      const SrcCell s = src(c0 - 1 + x, d0 - 1 + y, gk);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        cp_async<sizeof(S)>(rawU + (v * T::QY + y) * T::QX + x, m.h + v * P.vstride + s.off);
    }
  };
  // primitives of plane gk from the hydro variables (global memory, or rawU
  // when from_raw) and the face planes bslot (gk) and bslot1 (gk+1)
  auto load_Q = [&](int gk, int slot, int bs0, int bs1, bool from_raw) {
    R *       dst = sQ + slot * T::QP;
    const R * B0 = sB + bs0 * T::BP;
    const R * B1 = sB + bs1 * T::BP;
    for (int c = threadIdx.x; c < T::QX * T::QY; c += NT)
    {
      const int     x = c % T::QX, y = c / T::QX;
      const SrcCell s = src(c0 - 1 + x, d0 - 1 + y, gk);
      R             u[5], q[8];
      if (from_raw)
      {
#pragma unroll
        for (int v = 0; v < 5; ++v)
          u[v] = neg_if((R)rawU[(v * T::QY + y) * T::QX + x], flips(s, v, 1));
      }
      else
        load_hydro<S, R>(m, P, s, u);
      R bl[3], br[3];
      // sB x index = global - (c0-1): the Q cell at x has B index x
      bl[0] = B0[(0 * T::BY + y) * T::BX + x];
      bl[1] = B0[(1 * T::BY + y) * T::BX + x];
      bl[2] = B0[(2 * T::BY + y) * T::BX + x];
      br[0] = B0[(0 * T::BY + y) * T::BX + x + 1];
      br[1] = B0[(1 * T::BY + y + 1) * T::BX + x];
      br[2] = B1[(2 * T::BY + y) * T::BX + x];
      const int gi = c0 - 1 + x, gj = d0 - 1 + y;
      mhd_constoprim<R>(u, bl, br, q, C, [&](double (&a)[3], double (&b)[3]) {
        // FP64 copies of the face fields for the cancellation island
        a[0] = load_face<S>(m, P, s, 0);
        a[1] = load_face<S>(m, P, s, 1);
        a[2] = load_face<S>(m, P, s, 2);
        b[0] = load_face<S>(m, P, src(gi + 1, gj, gk), 0);
        b[1] = load_face<S>(m, P, src(gi, gj + 1, gk), 1);
        b[2] = load_face<S>(m, P, src(gi, gj, gk + 1), 2);
      });
#pragma unroll
      for (int v = 0; v < 8; ++v)
        dst[(v * T::QY + y) * T::QX + x] = q[v];
    }
  };
  // edge electric fields of plane gk (ComputeElecFieldFunctor3D,
  // MHDRunFunctors3D.h:318-356) from Q planes gk-1 (qs0), gk (qs1) and face
  // planes gk-1 (bs0), gk (bs1)
  auto compute_E = [&](int slot, int qs0, int qs1, int bs0, int bs1) {
    R *            dst = sE + slot * T::EP;
    const R *      Qa = sQ + qs0 * T::QP; // k-1
    const R *      Qb = sQ + qs1 * T::QP; // k
    const R * Ba = sB + bs0 * T::BP;
    const R * Bb = sB + bs1 * T::BP;
    for (int c = threadIdx.x; c < T::EX * T::EY; c += NT)
    {
      const int x = c % T::EX, y = c / T::EX; // E cell global = c0 + x
      const int qx = x + 1, qy = y + 1;       // sQ index of the same cell
      const int bx = x + 1, by = y + 1;       // sB index of the same cell
      auto      Q = [&](const R * pl, int v, int xx, int yy) { return pl[(v * T::QY + yy) * T::QX + xx]; };
      auto      Bf = [&](const R * pl, int comp, int xx, int yy) {
        return (R)pl[(comp * T::BY + yy) * T::BX + xx];
      };
      R uu, vv, ww, A, B, Cc;
      vv = R(0.25) * (Q(Qa, IV, qx, qy - 1) + Q(Qb, IV, qx, qy - 1) + Q(Qa, IV, qx, qy) + Q(Qb, IV, qx, qy));
      ww = R(0.25) * (Q(Qa, IW, qx, qy - 1) + Q(Qb, IW, qx, qy - 1) + Q(Qa, IW, qx, qy) + Q(Qb, IW, qx, qy));
      B = R(0.5) * (Bf(Ba, 1, bx, by) + Bf(Bb, 1, bx, by));
      Cc = R(0.5) * (Bf(Bb, 2, bx, by - 1) + Bf(Bb, 2, bx, by));
      dst[(0 * T::EY + y) * T::EX + x] = vv * Cc - ww * B;
      uu = R(0.25) * (Q(Qa, IU, qx - 1, qy) + Q(Qb, IU, qx - 1, qy) + Q(Qa, IU, qx, qy) + Q(Qb, IU, qx, qy));
      ww = R(0.25) * (Q(Qa, IW, qx - 1, qy) + Q(Qb, IW, qx - 1, qy) + Q(Qa, IW, qx, qy) + Q(Qb, IW, qx, qy));
      A = R(0.5) * (Bf(Ba, 0, bx, by) + Bf(Bb, 0, bx, by));
      Cc = R(0.5) * (Bf(Bb, 2, bx - 1, by) + Bf(Bb, 2, bx, by));
      dst[(1 * T::EY + y) * T::EX + x] = ww * A - uu * Cc;
      uu = R(0.25) * (Q(Qb, IU, qx - 1, qy - 1) + Q(Qb, IU, qx - 1, qy) + Q(Qb, IU, qx, qy - 1) + Q(Qb, IU, qx, qy));
      vv = R(0.25) * (Q(Qb, IV, qx - 1, qy - 1) + Q(Qb, IV, qx - 1, qy) + Q(Qb, IV, qx, qy - 1) + Q(Qb, IV, qx, qy));
      A = R(0.5) * (Bf(Bb, 0, bx, by - 1) + Bf(Bb, 0, bx, by));
      B = R(0.5) * (Bf(Bb, 1, bx - 1, by) + Bf(Bb, 1, bx, by));
      dst[(2 * T::EY + y) * T::EX + x] = uu * B - vv * A;
    }
  };

  // ring slots: face planes by global k modulo 4, Q by k modulo 3, E by k modulo 2
  auto bsl = [](int k) { return (k + 8) % 4; };
  auto qsl = [](int k) { return (k + 6) % 3; };
  auto esl = [](int k) { return (k + 4) % 2; };

  // prologue: face planes k0-1..k0+1, Q(k0-1), Q(k0), E(k0); the copies of
  // face plane k0+2 and hydro plane k0+1 start here
  load_B(k0 - 1, bsl(k0 - 1));
  load_B(k0, bsl(k0));
  load_B(k0 + 1, bsl(k0 + 1));
  issue_B(k0 + 2);
  issue_U(k0 + 1);
  cp_async_commit();
  __syncthreads();
  load_Q(k0 - 1, qsl(k0 - 1), bsl(k0 - 1), bsl(k0), false);
  load_Q(k0, qsl(k0), bsl(k0), bsl(k0 + 1), false);
  __syncthreads();
  compute_E(esl(k0), qsl(k0 - 1), qsl(k0), bsl(k0 - 1), bsl(k0));

  const int       tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const bool      own = (c0 + tx) <= P.nx + gw && (d0 + ty) <= P.ny + gw && (c0 - (gw - 1) + tx) < nti &&
                   (d0 - (gw - 1) + ty) < ntj;
  const TraceGrid tg = trace_grid(P);
  for (int k = k0; k < k1; ++k)
  {
    // face plane k+2 and hydro plane k+1 were copied during the previous
    // plane's work: convert them, then start the next plane's copies
    cp_async_wait_all();
    convert_B(k + 2, bsl(k + 2));
    __syncthreads();
    load_Q(k + 1, qsl(k + 1), bsl(k + 1), bsl(k + 2), true);
    __syncthreads();
    if (k + 1 < k1)
    {
      issue_B(k + 3);
      issue_U(k + 2);
      cp_async_commit();
    }
    compute_E(esl(k + 1), qsl(k), qsl(k + 1), bsl(k), bsl(k + 1));
    __syncthreads();
    if (own)
    {
      int bslot[4] = { bsl(k - 1), bsl(k), bsl(k + 1), bsl(k + 2) };
      int qslot[3] = { qsl(k - 1), qsl(k), qsl(k + 1) };
      int eslot[2] = { esl(k), esl(k + 1) };
      trace_cell_compact<R, TX, TY>(sB, bslot, sQ, qslot, sE, eslot, tx, ty, dtdx, dtdy, dtdz, C,
                                    trace_cell(trace, tg, gw, c0 + tx, d0 + ty, k));
    }
    __syncthreads();
  }
  cp_async_wait_all(); // no copy may land after the block has left
}

// ---------------------------------------------------------------------------
// 3. fluxes, emfs and update
// ---------------------------------------------------------------------------
// Output tile [i0, i0+TX) x [j0, j0+TY) marching over planes [k0, k1).  The
// compact trace of the cells [i0-1, i0+TX] x [j0-1, j0+TY] of planes k-1 and k
// is read through L1, or staged in shared memory (STAGE).  Per plane, the
// faces and edges the tile needs form one work list ordered by rows
// (UpdTile::item): one code path for the faces of the three directions (the
// HLLD solver) and one for the edges (the 2D HLLD emf), so the kernel holds
// one copy of each solver.
using ekc::UpdTile; // the tile's work items (ek_worklist.h)

// The tile list of the HLLD repair pass, at the start of the mixed form's
// work buffer (the trace follows): [0] tiles listed this step, [1] repair
// blocks done, [2..3] tiles repaired since the list was cleared (64-bit),
// [4..] the tile indices.
constexpr int kRepairHead = 4;
__host__ __device__ inline long long
repair_tiles(const KParams & P, int TX, int TY)
{
  return (long long)((P.nx + TX - 1) / TX) * ((P.ny + TY - 1) / TY) * ((P.nz + P.kchunk - 1) / P.kchunk);
}

// One tile column of the step: the cells [i0, i0+TX) x [j0, j0+TY) x [k0, k1)
// of tile (bx, by, bz).  A tile writes only its own cells, from the step's
// input state and trace.  REPAIR: the faces whose FP32 HLLD star state is
// ill-conditioned are solved in FP64 (the repair kernel); otherwise such a
// face lists the tile for that kernel and the tile commits no CFL candidate.
template <class S, class R, int TX, int TY, bool STAGE, int RS, bool REPAIR>
__device__ __forceinline__ void
mhd_update_tile(const void * __restrict__ Uin, void * __restrict__ Uout, const R * __restrict__ trace,
                const KParams & P, DevClock * clk, int step, int cfl_next, const StepConsts & sc, int bx, int by,
                int bz, int * repair)
{
  using T = UpdTile<TX, TY>;
  constexpr int NT = TX * TY;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // next step's CFL (cfl_next): the final face fields of the cells of the
  // last two finished planes (x / y faces by plane parity, the tile's +1
  // column / row beside them), and the final hydro variables and z face of
  // each thread's own cell of the last finished plane
  double * sBxL = reinterpret_cast<double *>(smem_raw); // [2][TY][TX]
  double * sByL = sBxL + 2 * TX * TY;                  // [2][TY][TX]
  double * sBxE = sByL + 2 * TX * TY;                  // [2][TY]  Bx(i0 + TX)
  double * sByE = sBxE + 2 * TY;                       // [2][TX]  By(j0 + TY)
  double * sBzF = sByE + 2 * TX;                       // [TY][TX]
  R *      sFinU = reinterpret_cast<R *>(sBzF + TX * TY); // [5][TY][TX]
  R *      sT = sFinU + 5 * TX * TY;                   // [2][T_N][YE][XE] trace planes (STAGE)
  R * sFx = sT + (STAGE ? 2 * T_N * T::PL : 0); // [5][TY][TX+1]
  R * sFy = sFx + 5 * T::FXS;               // [5][TY+1][TX]
  R * sFz = sFy + 5 * T::FYS;               // [5][TY][TX]
  R * sEz = sFz + 5 * T::FZS;               // [2][TY+1][TX+1]
  R * sEy = sEz + 2 * T::EZS;               // [2][TY][TX+1]
  R * sEx = sEy + 2 * T::EYS;               // [2][TY+1][TX]

  const R           dtdx = to_r<R>(sc.dtdx), dtdy = to_r<R>(sc.dtdy), dtdz = to_r<R>(sc.dtdz);
  const double      ddtdx = sc.dtdx, ddtdy = sc.dtdy, ddtdz = sc.dtdz; // FP64 ratios of the CT update
  const MhdConst<R> C = mhd_const<R>(P);
  const int         gw = P.gw;
  const int         i0 = gw + bx * TX, j0 = gw + by * TY;
  const int         k0 = gw + bz * P.kchunk;
  const int         k1 = min(k0 + P.kchunk, P.nz + gw);
  const int         tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int         gi = i0 + tx, gj = j0 + ty;
  const bool        own = gi < P.nx + gw && gj < P.ny + gw;
  const long long   st = P.vstride;
  const MhdState<S> mi = mhd_state<S>(Uin, P);
  S *               hout = (S *)Uout;
  double *          bout = sizeof(S) == 8 ? (double *)Uout + 5 * P.vstride : mixed_bfield(Uout, P);
  const R           sr = C.smallr, sp = C.smallp;
  // the trace buffer holds cells [gw-1, n+gw] in each direction
  const int ihi = P.nx + gw, jhi = P.ny + gw;

  const TraceGrid tg = trace_grid(P);
  auto load_plane = [&](int k) {
    if (!STAGE)
      return;
    R * dst = sT + (k & 1) * T_N * T::PL;
    for (int c = threadIdx.x; c < T_N * T::PL; c += NT)
    {
      const int f = c / T::PL, r = c - f * T::PL;
      const int x = r % T::XE, y = r / T::XE;
      const int i = min(i0 - 1 + x, ihi), j = min(j0 - 1 + y, jhi);
      dst[c] = ldg(trace_cell(trace, tg, gw, i, j, k) + trace_field<R>(f));
    }
  };
  // trace pointer of cell (i, j) (global indices) of plane k: shared memory
  // (STAGE) or the trace buffer itself (read through L1)
  auto TS = [&](int i, int j, int k) -> const R * {
    if (STAGE)
      return sT + (k & 1) * T_N * T::PL + (j - (j0 - 1)) * T::XE + (i - (i0 - 1));
    return trace_cell(trace, tg, gw, i, j, k);
  };
  constexpr int tst = T::PL; // field stride of the staged planes

  R acc[5];
  R tmax = R(-INFINITY);
  // the CFL candidate of the updated cell (gi, gj, kc) from its final
  // hydro variables u and the final face fields on its low (bl) and high
  // (br) faces (ConvertToPrimitivesFunctor3D_MHD + ComputeDtFunctor3D_MHD on
  // the next step's state, as mhd_dt_kernel computes them)
  auto cfl_cell = [&](const R (&u)[5], const double (&bl)[3], const double (&br)[3]) {
    R blr[3], brr[3], q[8];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      blr[c] = to_r<R>(bl[c]);
      brr[c] = to_r<R>(br[c]);
    }
    mhd_constoprim<R>(u, blr, brr, q, C, [&](double (&a)[3], double (&b)[3]) {
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        a[c] = bl[c];
        b[c] = br[c];
      }
    });
    tmax = fmax(tmax, mhd_invdt<R>(q, C.gamma0, P.dx, P.dy, P.dz, P.idx, P.idy, P.idz, P.idxd, P.idyd, P.idzd));
  };
  // the face field beyond the domain's high end along one axis, as the
  // next step's ghost fill leaves it: outflow copies the last interior face,
  // a reflecting wall negates it, periodic takes the CT update there (equal
  // to the update of the first interior face: same inputs by the mapping)
  auto high_face = [&](int bc, double own, double ct) {
    return bc == BC_PERIODIC ? ct : (bc == BC_DIRICHLET ? -own : own);
  };
  // CT increments of the face fields, in the expressions of the update below
  auto ct_add = [&](double b, R ep, R em, R ratio, double dratio) {
    if constexpr (sizeof(R) == 8)
      return b + (ep - em) * ratio;
    else
      return fma(f2d(ep) - f2d(em), dratio, b);
  };
  auto ct_sub = [&](double b, R ep, R em, R ratio, double dratio) {
    if constexpr (sizeof(R) == 8)
      return b - (ep - em) * ratio;
    else
      return fma(f2d(em) - f2d(ep), dratio, b);
  };
  // mixed HLLD: a face whose FP32 star state is ill-conditioned marks the tile
  constexpr bool kFlag = sizeof(R) == 4 && RS == 4 && !REPAIR;
  __shared__ int s_dirty;
  if (threadIdx.x == 0)
    s_dirty = 0;

  load_plane(k0 - 1);
  for (int k = k0; k <= k1; ++k)
  {
    const bool plane = k < k1; // cells of plane k get their in-plane fluxes this iteration
    load_plane(k);
    __syncthreads();
    R * Ez = sEz + (k & 1) * T::EZS;
    R * Ey = sEy + (k & 1) * T::EYS;
    R * Ex = sEx + (k & 1) * T::EXS;
    // Work items (faces and edges).  Mixed form: ordered by rows (UpdTile::
    // item), so the items that gather a cell's trace run close together and
    // the repeated gathers hit L1 (four CTAs share an SM's L1).  FP64: all
    // faces of the plane, then all edges (UpdTile::item_by_kind): one CTA
    // per SM, bound by the FP64 pipe, and the warps' shares of the two kinds
    // stay equal (an edge costs about twice a face).  Plane k1 only needs its
    // z-faces and its y- and x-edges.
    for (int w = threadIdx.x; w < (sizeof(R) == 4 ? T::NITEMS : T::NITEMS_K); w += NT)
    {
      int kind, li, lj; // kind 0..5: z-, x-, y-face, y-, x-, z-edge
      if (!(sizeof(R) == 4 ? T::item(w, kind, li, lj) : T::item_by_kind(w, kind, li, lj)))
        continue;
      if (!plane && (kind == 1 || kind == 2 || kind == 5))
        continue;
      if (kind < 3)
      {
        // face normal to d between cell (i,j,k) - e_d and cell (i,j,k)
        // (MHDRunFunctors3D.h:1839-1874); flux index f in rows of TX + 1
        // x-faces or TX faces
        const int d = kind == 0 ? 2 : kind - 1;
        const int f = d == 0 ? lj * (TX + 1) + li : lj * TX + li;
        const int i = i0 + li, j = j0 + lj;
        if (i > ihi - (d != 0 ? 1 : 0) || j > jhi - (d != 1 ? 1 : 0))
          continue;
        R ql[8], qr[8], fl[5];
        // the two face states, gathered with the direction fixed at compile
        // time (every trace field at a constant offset); one solver call
        auto gather = [&](auto dc) {
          constexpr int D = decltype(dc)::value;
          const R * tl = TS(i - (D == 0), j - (D == 1), k - (D == 2));
          const R * tr = TS(i, j, k);
          if constexpr (STAGE)
          {
            face_state_dir<R, true>(tl, tst, D, ql, sr, sp);
            face_state_dir<R, false>(tr, tst, D, qr, sr, sp);
          }
          else
          {
            face_state_acc<R, true>(QuadAcc<R>(tl), D, ql, sr, sp);
            face_state_acc<R, false>(QuadAcc<R>(tr), D, qr, sr, sp);
          }
        };
        if (d == 0)
          gather(DirC<0>());
        else if (d == 1)
          gather(DirC<1>());
        else
          gather(DirC<2>());
        if (!mhd_riemann<RS, R, 5>(ql, qr, fl, C.gamma0))
        {
          // ill-conditioned star state in FP32 (mixed HLLD only)
          if constexpr (REPAIR)
            mhd_hlld_f64_from_f32<5>(ql, qr, fl, C.gamma0);
          else
          {
            s_dirty = 1;
            continue;
          }
        }
        R *       dst = d == 0 ? sFx : (d == 1 ? sFy : sFz);
        const int nd = d == 0 ? T::FXS : (d == 1 ? T::FYS : T::FZS);
#pragma unroll
        for (int v = 0; v < 5; ++v)
          dst[v * nd + f] = fl[v];
        continue;
      }
      // edge along d at the low corner of cell (i,j,k); corners RT, RB, LT, LB
      // lie at -1 along (p1,p2), p1, p2 and nowhere (z-edge: RT(i-1,j-1),
      // RB(i-1,j), LT(i,j-1), LB(i,j); MHDRunFunctors3D.h:2180-2230); emf
      // index f in rows of TX x-edges or TX + 1 edges
      const int d = kind == 3 ? 1 : (kind == 4 ? 0 : 2);
      const int f = d == 0 ? lj * TX + li : lj * (TX + 1) + li;
      const int i = i0 + li, j = j0 + lj;
      if (i > ihi - (d == 0 ? 1 : 0) || j > jhi - (d == 1 ? 1 : 0))
        continue;
      EdgeCorner<R> cRT, cRB, cLT, cLB;
      // the four corner states, gathered with the direction fixed at compile
      // time; one emf solver call
      auto gather = [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        constexpr int p1 = D == 2 ? 0 : D + 1, p2 = D == 0 ? 2 : D - 1;
        constexpr int i1 = p1 == 0, j1 = p1 == 1, k1s = p1 == 2;
        constexpr int i2 = p2 == 0, j2 = p2 == 1, k2s = p2 == 2;
        const R * tRT = TS(i - i1 - i2, j - j1 - j2, k - k1s - k2s);
        const R * tRB = TS(i - i1, j - j1, k - k1s);
        const R * tLT = TS(i - i2, j - j2, k - k2s);
        const R * tLB = TS(i, j, k);
        if constexpr (STAGE)
        {
          cRT = edge_corner<R, 1, 1>(tRT, tst, D, p1, p2, sr, sp);
          cRB = edge_corner<R, 1, -1>(tRB, tst, D, p1, p2, sr, sp);
          cLT = edge_corner<R, -1, 1>(tLT, tst, D, p1, p2, sr, sp);
          cLB = edge_corner<R, -1, -1>(tLB, tst, D, p1, p2, sr, sp);
        }
        else
        {
          cRT = edge_corner_acc<R, 1, 1>(QuadAcc<R>(tRT), D, p1, p2, sr, sp);
          cRB = edge_corner_acc<R, 1, -1>(QuadAcc<R>(tRB), D, p1, p2, sr, sp);
          cLT = edge_corner_acc<R, -1, 1>(QuadAcc<R>(tLT), D, p1, p2, sr, sp);
          cLB = edge_corner_acc<R, -1, -1>(QuadAcc<R>(tLB), D, p1, p2, sr, sp);
        }
      };
      if (d == 0)
        gather(DirC<0>());
      else if (d == 1)
        gather(DirC<1>());
      else
        gather(DirC<2>());
      const R e = mhd_emf_corners<R>(cRT, cRB, cLT, cLB, C.gamma0, C.smallc);
      (d == 0 ? Ex : (d == 1 ? Ey : Ez))[f] = e;
    }
    __syncthreads();
    const int fz0 = ty * TX + tx;
    if (own && k > k0)
    {
      // finish cell k-1: hydro (UpdateFunctor3D_MHD, MHDRunFunctors3D.h:2488-2527)
      const long long off = (long long)(k - 1) * P.plane + (long long)gj * P.isize + gi;
      acc[ID] -= sFz[ID * T::FZS + fz0] * dtdz;
      acc[IP] -= sFz[IP * T::FZS + fz0] * dtdz;
      acc[IU] -= sFz[IW * T::FZS + fz0] * dtdz;
      acc[IV] -= sFz[IV * T::FZS + fz0] * dtdz;
      acc[IW] -= sFz[IU * T::FZS + fz0] * dtdz;
#pragma unroll
      for (int v = 0; v < 5; ++v)
        hout[v * st + off] = (S)acc[v];
      // CT update of the face fields (UpdateEmfFunctor3D, MHDRunFunctors3D.h:2590-2613)
      const R * Ezp = sEz + ((k - 1) & 1) * T::EZS;
      const R * Eyp = sEy + ((k - 1) & 1) * T::EYS;
      const R * Exp = sEx + ((k - 1) & 1) * T::EXS;
      const int ezi = ty * (TX + 1) + tx, eyi = ty * (TX + 1) + tx, exi = ty * TX + tx;
      double    bx = mi.b[0 * st + off], by = mi.b[1 * st + off], bz = mi.b[2 * st + off];
      if constexpr (sizeof(R) == 8)
      {
        bx += (Ezp[ezi + (TX + 1)] - Ezp[ezi]) * dtdy;
        by -= (Ezp[ezi + 1] - Ezp[ezi]) * dtdx;
        bx -= (Ey[eyi] - Eyp[eyi]) * dtdz;
        by += (Ex[exi] - Exp[exi]) * dtdz;
        bz += (Eyp[eyi + 1] - Eyp[eyi]) * dtdx;
        bz -= (Exp[exi + TX] - Exp[exi]) * dtdy;
      }
      else
      {
        // FP64 island: the CT update keeps div B at FP64 round-off (one
        // subtraction and one fused multiply-add per term)
        bx = fma(f2d(Ezp[ezi + (TX + 1)]) - f2d(Ezp[ezi]), ddtdy, bx);
        by = fma(f2d(Ezp[ezi]) - f2d(Ezp[ezi + 1]), ddtdx, by);
        bx = fma(f2d(Eyp[eyi]) - f2d(Ey[eyi]), ddtdz, bx);
        by = fma(f2d(Ex[exi]) - f2d(Exp[exi]), ddtdz, by);
        bz = fma(f2d(Eyp[eyi + 1]) - f2d(Eyp[eyi]), ddtdx, bz);
        bz = fma(f2d(Exp[exi]) - f2d(Exp[exi + TX]), ddtdy, bz);
      }
      bout[0 * st + off] = bx;
      bout[1 * st + off] = by;
      bout[2 * st + off] = bz;
      if (cfl_next)
      {
        const int c = ty * TX + tx;
        if (k > k0 + 1)
        {
          // cell k-2 is complete now that its high z face (this cell's bz)
          // is final
          const int par = (k - 2) & 1;
          R         u[5];
#pragma unroll
          for (int v = 0; v < 5; ++v)
            u[v] = sFinU[v * TX * TY + c];
          const double bl[3] = { sBxL[par * TX * TY + c], sByL[par * TX * TY + c], sBzF[c] };
          const double br[3] = { tx + 1 < TX && gi + 1 < P.nx + gw ? sBxL[par * TX * TY + c + 1] : sBxE[par * TY + ty],
                                 ty + 1 < TY && gj + 1 < P.ny + gw ? sByL[par * TX * TY + c + TX] : sByE[par * TX + tx],
                                 bz };
          cfl_cell(u, bl, br);
        }
        // this cell's final state for the CFL at the next plane
        const int par = (k - 1) & 1;
#pragma unroll
        for (int v = 0; v < 5; ++v)
          sFinU[v * TX * TY + c] = (R)(S)acc[v];
        sBxL[par * TX * TY + c] = bx;
        sByL[par * TX * TY + c] = by;
        sBzF[c] = bz;
        if (tx == TX - 1 || gi + 1 == P.nx + gw)
        {
          // Bx on the cell's high x face: the tile's edge or the domain's end
          double b1 = gi + 1 == P.nx + gw ? load_face<S>(mi, P, src_cell(P, gi + 1, gj, k - 1), 0)
                                          : ldg(mi.b + 0 * st + off + 1);
          b1 = ct_add(b1, Ezp[ezi + 1 + (TX + 1)], Ezp[ezi + 1], dtdy, ddtdy);
          b1 = ct_sub(b1, Ey[eyi + 1], Eyp[eyi + 1], dtdz, ddtdz);
          sBxE[par * TY + ty] = gi + 1 == P.nx + gw ? high_face(P.bc[1], bx, b1) : b1;
        }
        if (ty == TY - 1 || gj + 1 == P.ny + gw)
        {
          double b1 = gj + 1 == P.ny + gw ? load_face<S>(mi, P, src_cell(P, gi, gj + 1, k - 1), 1)
                                          : ldg(mi.b + 1 * st + off + P.isize);
          b1 = ct_sub(b1, Ezp[ezi + (TX + 1) + 1], Ezp[ezi + (TX + 1)], dtdx, ddtdx);
          b1 = ct_add(b1, Ex[exi + TX], Exp[exi + TX], dtdz, ddtdz);
          sByE[par * TX + tx] = gj + 1 == P.ny + gw ? high_face(P.bc[3], by, b1) : b1;
        }
      }
    }
    if (own && plane)
    {
      // partial update of cell k: U + Fx(i) - Fx(i+1) + Fy(j) - Fy(j+1) + Fz(k)
      const long long off = (long long)k * P.plane + (long long)gj * P.isize + gi;
      R               u[5];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        u[v] = (R)ldg(mi.h + v * st + off);
      const int fx0 = ty * (TX + 1) + tx, fy0 = ty * TX + tx;
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
      u[ID] += sFz[ID * T::FZS + fz0] * dtdz;
      u[IP] += sFz[IP * T::FZS + fz0] * dtdz;
      u[IU] += sFz[IW * T::FZS + fz0] * dtdz;
      u[IV] += sFz[IV * T::FZS + fz0] * dtdz;
      u[IW] += sFz[IU * T::FZS + fz0] * dtdz;
#pragma unroll
      for (int v = 0; v < 5; ++v)
        acc[v] = u[v];
    }
    __syncthreads(); // trace slot, flux buffers and the older emf planes are reused
  }
  // block-uniform: the plane loop ended with a barrier
  const bool dirty = kFlag && s_dirty != 0;
  if (cfl_next)
  {
    if (own && k1 > k0)
    {
      // the chunk's last cell (k1-1): its high z face is the next chunk's
      // first face, updated here from the emfs of plane k1
      const int       c = ty * TX + tx, par = (k1 - 1) & 1;
      const long long off = (long long)k1 * P.plane + (long long)gj * P.isize + gi;
      const R *       Ex1 = sEx + (k1 & 1) * T::EXS;
      const R *       Ey1 = sEy + (k1 & 1) * T::EYS;
      const int       eyi = ty * (TX + 1) + tx, exi = ty * TX + tx;
      double          bz1 = k1 == P.nz + gw ? load_face<S>(mi, P, src_cell(P, gi, gj, k1), 2) : ldg(mi.b + 2 * st + off);
      bz1 = ct_add(bz1, Ey1[eyi + 1], Ey1[eyi], dtdx, ddtdx);
      bz1 = ct_sub(bz1, Ex1[exi + TX], Ex1[exi], dtdy, ddtdy);
      if (k1 == P.nz + gw)
        bz1 = high_face(P.bc[5], sBzF[c], bz1);
      R u[5];
#pragma unroll
      for (int v = 0; v < 5; ++v)
        u[v] = sFinU[v * TX * TY + c];
      const double bl[3] = { sBxL[par * TX * TY + c], sByL[par * TX * TY + c], sBzF[c] };
      const double br[3] = { tx + 1 < TX && gi + 1 < P.nx + gw ? sBxL[par * TX * TY + c + 1] : sBxE[par * TY + ty],
                             ty + 1 < TY && gj + 1 < P.ny + gw ? sByL[par * TX * TY + c + TX] : sByE[par * TX + tx],
                             bz1 };
      cfl_cell(u, bl, br);
    }
    if (!dirty)
      block_max_commit<NT>(cand_key((double)tmax), &clk->key[(step + 1) % 3]);
  }
  if (dirty && threadIdx.x == 0)
  {
    const int gx = (P.nx + TX - 1) / TX, gy = (P.ny + TY - 1) / TY;
    repair[kRepairHead + atomicAdd(&repair[0], 1)] = (bz * gy + by) * gx + bx;
  }
}

// One launch per step: the tile columns of the grid.  repair: the tile list
// of the mixed HLLD form (null otherwise), whose repair kernel then completes
// the next step's CFL key.
template <class S, class R, int TX, int TY, bool STAGE, int RS>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_MU_MINB_F32, EK_MU_MINB_F64))
mhd_update_kernel(const void * __restrict__ Uin, void * __restrict__ Uout, const R * __restrict__ trace,
                  KParams P, DevClock * clk, int step, int cfl_next, int * repair)
{
  StepConsts sc;
  if (!step_consts(clk, step, sc))
    return;
  mhd_update_tile<S, R, TX, TY, STAGE, RS, false>(Uin, Uout, trace, P, clk, step, cfl_next, sc, blockIdx.x,
                                                   blockIdx.y, blockIdx.z, repair);
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0)
    step_commit(clk, step, sc.t, sc.dt);
  if (cfl_next && !repair)
    finalize_step(clk, P, step + 1); // the next step's dt, once its CFL key is complete
}

// The last block of a launch of the repair kernel: true once, after every block
// has read the tile count; it then clears the list for the next step.
__device__ __forceinline__ void
repair_list_release(int * repair)
{
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    __threadfence();
    last = atomicAdd(&repair[1], 1) == (int)(gridDim.x * gridDim.y * gridDim.z) - 1;
  }
  __syncthreads();
  if (last && threadIdx.x == 0)
  {
    __threadfence();
    atomicAdd(reinterpret_cast<unsigned long long *>(repair + 2), (unsigned long long)repair[0]);
    repair[0] = 0;
    repair[1] = 0;
  }
}

// After the update kernel of the mixed HLLD form: recomputes the tiles it
// listed, with the faces whose FP32 star state is ill-conditioned solved in
// FP64 (the rest as in the update kernel, so a tile's other cells are
// unchanged).  Recomputing a tile replaces its output, as tiles are
// independent within a step.  Then the next step's CFL key is complete.
template <class S, class R, int TX, int TY, bool STAGE>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_MU_MINB_F32, EK_MU_MINB_F64))
mhd_repair_kernel(const void * __restrict__ Uin, void * __restrict__ Uout, const R * __restrict__ trace,
                  KParams P, DevClock * clk, int step, int cfl_next, int * repair)
{
  StepConsts sc;
  if (!step_consts(clk, step, sc))
    return;
  const int n = repair[0];
  const int gx = (P.nx + TX - 1) / TX, gy = (P.ny + TY - 1) / TY;
  for (int e = blockIdx.x; e < n; e += gridDim.x)
  {
    const int tile = repair[kRepairHead + e];
    mhd_update_tile<S, R, TX, TY, STAGE, 4, true>(Uin, Uout, trace, P, clk, step, cfl_next, sc, tile % gx,
                                                   (tile / gx) % gy, tile / (gx * gy), repair);
    __syncthreads(); // shared memory of the next tile
  }
  repair_list_release(repair);
  if (cfl_next)
    finalize_step(clk, P, step + 1);
}

// max |div B| over the interior, face differences with dx normalisation
template <class S>
__global__ void
mhd_divb_kernel(const void * __restrict__ U, KParams P, unsigned long long * key)
{
  const MhdState<S> m = mhd_state<S>(U, P);
  unsigned long long kmax = 0ull;
  for_interior_rows(P, [&](int i, int j, int k) {
    const SrcCell   s0 = src_cell(P, i, j, k);
    double          d = (load_face<S>(m, P, src_cell(P, i + 1, j, k), 0) - load_face<S>(m, P, s0, 0)) / P.dx +
                     (load_face<S>(m, P, src_cell(P, i, j + 1, k), 1) - load_face<S>(m, P, s0, 1)) / P.dy;
    // 2D: Bz is not a face field (no z derivative)
    if (P.ksize > 1)
      d += (load_face<S>(m, P, src_cell(P, i, j, k + 1), 2) - load_face<S>(m, P, s0, 2)) / P.dz;
    const unsigned long long kk = cand_key(fabs(d));
    kmax = kk > kmax ? kk : kmax;
  });
  block_max_commit<256>(kmax, key);
}

template <class S, class R>
constexpr size_t
mhd_trace_smem(int TX, int TY)
{
  return sizeof(double) * 3 * (TX + 3) * (TY + 3) + sizeof(S) * 5 * (TX + 2) * (TY + 2) +
         sizeof(R) * (4 * 3 * (TX + 3) * (TY + 3) + 3 * 8 * (TX + 2) * (TY + 2) + 2 * 3 * (TX + 1) * (TY + 1));
}
template <class R>
constexpr size_t
mhd_update_smem(int TX, int TY, bool stage)
{
  return sizeof(double) * (5 * TX * TY + 2 * TY + 2 * TX) + sizeof(R) * 5 * TX * TY +
         sizeof(R) * ((stage ? 2 * T_N * (TX + 2) * (TY + 2) : 0) + 5 * (TX + 1) * TY + 5 * TX * (TY + 1) + 5 * TX * TY +
                      2 * (TX + 1) * (TY + 1) + 2 * (TX + 1) * TY + 2 * TX * (TY + 1));
}

constexpr int MT_TX = EK_MT_TX, MT_TY = EK_MT_TY; // trace tile
constexpr int MU_TX = EK_MU_TX, MU_TY = EK_MU_TY; // update tile

// bytes of the compact trace in the work buffer (256-byte rounded)
inline size_t
mhd_trace_bytes(int prec, const KParams & P)
{
  // blocks of 32 trace cells x 48 fields over (nx+2)/32 x (ny+2) x (nz+2)
  const TraceGrid g = trace_grid(P);
  const size_t    blk = prec == 0 ? (size_t)kTraceBlock<double> * sizeof(double)
                                  : (size_t)kTraceBlock<float> * sizeof(float);
  return (blk * (size_t)g.nb * (size_t)g.nj * (size_t)(P.nz + 2) + 255) & ~(size_t)255;
}
// The mixed form's work buffer starts with the repair pass's tile list; the
// trace follows, 256-byte aligned.  The FP64 form holds the trace alone.
inline size_t
mhd_repair_bytes(const KParams & P)
{
  return (sizeof(int) * (size_t)(kRepairHead + repair_tiles(P, MU_TX, MU_TY)) + 255) & ~(size_t)255;
}
template <class R>
R *
mhd_trace_of(void * work, const KParams & P)
{
  return reinterpret_cast<R *>(static_cast<char *>(work) + (sizeof(R) == 8 ? 0 : mhd_repair_bytes(P)));
}
// blocks of a repair launch: one per SM (most steps list no tile); the SM
// count of each device is looked up once
inline int
repair_grid(long long tiles)
{
  static int sms_of[64] = {};
  int        dev = 0, sms = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64)
  {
    sms = __atomic_load_n(&sms_of[dev], __ATOMIC_RELAXED);
    if (sms == 0 && cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      __atomic_store_n(&sms_of[dev], sms, __ATOMIC_RELAXED);
  }
  if (sms <= 0)
    sms = 1;
  return (int)(tiles < sms ? (tiles > 0 ? tiles : 1) : sms);
}

template <class S, class R>
cudaError_t
mhd_step_t(int phase, const void * Uin, void * Uout, void * work, const KParams & P, DevClock * clk,
           int step, bool cfl_next, cudaStream_t st)
{
  // 1. dt of this step into clock slot step % 3
  if (phase == 0)
  {
    mhd_dt_kernel<S, R><<<row_blocks(P), 256, 0, st>>>(Uin, P, clk, step, nullptr);
    return cudaGetLastError();
  }
  // 2. trace
  if (phase == 1)
  {
    auto       k = mhd_trace_kernel<S, R, MT_TX, MT_TY>;
    const int  sm = (int)mhd_trace_smem<S, R>(MT_TX, MT_TY);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess)
      return e;
    const int nt = P.nz + 2;
    dim3      grid((P.nx + 2 + MT_TX - 1) / MT_TX, (P.ny + 2 + MT_TY - 1) / MT_TY, (nt + P.kchunk - 1) / P.kchunk);
    k<<<grid, MT_TX * MT_TY, sm, st>>>(Uin, mhd_trace_of<R>(work, P), P, clk, step);
    return cudaGetLastError();
  }
  // 4. the repair pass of the mixed HLLD form (after phase 2)
  if (phase == 3)
  {
    if constexpr (sizeof(R) == 8)
      return cudaErrorNotSupported;
    else
    {
      if (P.riemann != 4)
        return cudaErrorNotSupported;
      auto       k = P.mhd_stage ? mhd_repair_kernel<S, R, MU_TX, MU_TY, true> : mhd_repair_kernel<S, R, MU_TX, MU_TY, false>;
      const int  sm = (int)mhd_update_smem<R>(MU_TX, MU_TY, P.mhd_stage != 0);
      cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
      if (e != cudaSuccess)
        return e;
      k<<<repair_grid(repair_tiles(P, MU_TX, MU_TY)), MU_TX * MU_TY, sm, st>>>(
        Uin, Uout, mhd_trace_of<R>(work, P), P, clk, step, cfl_next ? 1 : 0, (int *)work);
      return cudaGetLastError();
    }
  }
  // 3. fluxes, emfs, update (trace read through L1, or staged in shared memory
  //    for the HLLD solver); the face Riemann solver is a template parameter;
  //    the mixed HLLD form lists tiles for phase 3, which must follow
  {
    auto k = P.riemann == 1   ? mhd_update_kernel<S, R, MU_TX, MU_TY, false, 1>
             : P.riemann == 2 ? mhd_update_kernel<S, R, MU_TX, MU_TY, false, 2>
             : P.mhd_stage    ? mhd_update_kernel<S, R, MU_TX, MU_TY, true, 4>
                              : mhd_update_kernel<S, R, MU_TX, MU_TY, false, 4>;
    const int  sm = (int)mhd_update_smem<R>(MU_TX, MU_TY, P.mhd_stage != 0 && P.riemann == 4);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess)
      return e;
    dim3 grid((P.nx + MU_TX - 1) / MU_TX, (P.ny + MU_TY - 1) / MU_TY, (P.nz + P.kchunk - 1) / P.kchunk);
    int * repair = sizeof(R) == 4 && P.riemann == 4 ? (int *)work : nullptr;
    k<<<grid, MU_TX * MU_TY, sm, st>>>(Uin, Uout, mhd_trace_of<R>(work, P), P, clk, step, cfl_next ? 1 : 0, repair);
    return cudaGetLastError();
  }
}

cudaError_t
mhd_step(int prec, int phase, const void * Uin, void * Uout, void * work, const KParams & P,
         DevClock * clk, int step, bool cfl_next, cudaStream_t st)
{
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  return mhd_step_t<double, double>(phase, Uin, Uout, work, P, clk, step, cfl_next, st);
#else
  if (prec == 0)
    return mhd_step_t<double, double>(phase, Uin, Uout, work, P, clk, step, cfl_next, st);
  return mhd_step_t<float, float>(phase, Uin, Uout, work, P, clk, step, cfl_next, st);
#endif
}

cudaError_t
mhd_dt(int prec, const void * U, const KParams & P, unsigned long long * key, cudaStream_t st)
{
  const int blocks = row_blocks(P);
#ifdef EK_EXACT_ONLY
  if (prec != 0)
    return cudaErrorNotSupported;
  mhd_dt_kernel<double, double><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
#else
  if (prec == 0)
    mhd_dt_kernel<double, double><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
  else
    mhd_dt_kernel<float, float><<<blocks, 256, 0, st>>>(U, P, nullptr, 0, key);
#endif
  return cudaGetLastError();
}

size_t
mhd_work_bytes(int prec, const KParams & P)
{
  // the trace; the mixed form's tile list first (cleared by the caller
  // before the first step)
  if (prec == 0)
    return mhd_trace_bytes(0, P);
  return mhd_repair_bytes(P) + mhd_trace_bytes(1, P);
}

#ifndef EK_EXACT_ONLY
cudaError_t
mhd_divb_max(int prec, const void * U, const KParams & P, double * out, cudaStream_t st)
{
  // reuses out as a key slot, then converts in place on the host side
  unsigned long long * key = reinterpret_cast<unsigned long long *>(out);
  cudaError_t          e = cudaMemsetAsync(key, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess)
    return e;
  const int blocks = row_blocks(P);
  if (prec == 0)
    mhd_divb_kernel<double><<<blocks, 256, 0, st>>>(U, P, key);
  else
    mhd_divb_kernel<float><<<blocks, 256, 0, st>>>(U, P, key);
  return cudaGetLastError();
}
#endif

} // namespace EK_NS
