// Fused hydro step kernels (2D tile, 3D tile marching in z).
//
// One launch performs the whole implementationVersion=0 step of
// SolverHydroMuscl::godunov_unsplit_impl (SolverHydroMuscl.cpp:214-243,
// 304-330) for its tile: ghost fill (virtual, ek_common.cuh), primitive
// variables, limited slopes, half-step face traces, HLLC fluxes, conservative
// update, and the CFL candidate of the NEXT step (ComputeDtFunctor on the new
// state, SolverHydroMuscl.h:589-631), reduced with one atomicMax per block.
// U is read from HBM once (plus the tile halo) and written once.
#pragma once

#include "ek_hydro.cuh"

namespace EK_NS
{

template <class R>
__device__ __forceinline__ HydroConst<R>
hydro_const(const KParams & P)
{
  HydroConst<R> C;
  if constexpr (sizeof(R) == 8)
  {
    C.gamma0 = P.gamma0;
    C.smallr = P.smallr;
    C.smallp = P.smallp;
    C.smallc = P.smallc;
    C.slope_type = P.slope_type;
    C.gamma6 = P.gamma6;
    C.smallpp = P.smallpp;
    C.entho = 1.0 / (P.gamma0 - 1.0);
  }
  else
  {
    C.gamma0 = P.gamma0f;
    C.smallr = P.smallrf;
    C.smallp = P.smallpf;
    C.smallc = P.smallcf;
    C.slope_type = P.slopef;
    C.gamma6 = P.gamma6f;
    C.smallpp = P.smallppf;
    C.entho = 1.0f / (P.gamma0f - 1.0f);
  }
  return C;
}

// Load one (TX+4) x (TY+4) plane of U (global plane gk), convert to primitive
// variables and store into sQ[NV][HY][HX]; halo cells are mapped through the
// boundary conditions.
// When the whole (TX+4) x (TY+4) halo of the tile and plane gk lie inside the
// interior (direct), the boundary mapping is the identity and is skipped.
template <class S, class R, int NV, int TX, int TY>
__device__ __forceinline__ void
load_q_plane(const S * __restrict__ U, const KParams & P, const HydroConst<R> & C, int gi0, int gj0,
             int gk, R * sQ, bool direct = false)
{
  constexpr int HX = TX + 4, HY = TY + 4, NT = TX * TY;
  for (int c = threadIdx.x; c < HX * HY; c += NT)
  {
    const int hx = c % HX, hy = c / HX;
    R         u[NV], q[NV];
    if (direct)
    {
      const long long off = (long long)gk * P.plane + (long long)(gj0 - 2 + hy) * P.isize + (gi0 - 2 + hx);
#pragma unroll
      for (int v = 0; v < NV; ++v)
        u[v] = (R)ldg(U + v * P.vstride + off);
    }
    else
    {
      const SrcCell s = src_cell(P, gi0 - 2 + hx, gj0 - 2 + hy, gk);
#pragma unroll
      for (int v = 0; v < NV; ++v)
      {
        u[v] = neg_if((R)ldg(U + v * P.vstride + s.off), flips(s, v, 0));
      }
    }
    hydro_prims<R, NV>(u, q, C);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sQ[(v * HY + hy) * HX + hx] = q[v];
  }
}

// In-place conversion of a (TX+4) x (TY+4) plane of conserved variables,
// staged in sQ[NV][HY][HX] by a tensor copy, to primitive variables.  Each
// thread converts whole cells, so no cell is read after another thread wrote it.
template <class R, int NV, int TX, int TY>
__device__ __forceinline__ void
convert_q_plane(R * sQ, const HydroConst<R> & C)
{
  constexpr int HX = TX + 4, HY = TY + 4, NT = TX * TY;
  for (int c = threadIdx.x; c < HX * HY; c += NT)
  {
    R u[NV], q[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      u[v] = sQ[v * HY * HX + c];
    hydro_prims<R, NV>(u, q, C);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sQ[v * HY * HX + c] = q[v];
  }
}

// elements between ring slots of the 3D kernel: one primitive plane rounded up
// to a multiple of 128 bytes (the alignment of a tensor-copy destination)
template <class R, int TX, int TY>
__host__ __device__ constexpr int
hydro3d_slot_elems()
{
  return (int)(((5 * (TX + 4) * (TY + 4) * sizeof(R) + 127) / 128 * 128) / sizeof(R));
}

// slopes of the cell at tile coordinates (hx, hy) of the planes qm/q0/qp
template <class R, int NV, int HX, int HY>
__device__ __forceinline__ void
cell_slopes(const R * q0, const R * qm, const R * qp, int hx, int hy, R st, R (&c)[NV], R (&dX)[NV],
            R (&dY)[NV], R (&dZ)[NV], bool three_d)
{
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    const R * p = q0 + v * HY * HX;
    const R   x = p[hy * HX + hx];
    c[v] = x;
    dX[v] = slope1<R>(x, p[hy * HX + hx + 1], p[hy * HX + hx - 1], st);
    dY[v] = slope1<R>(x, p[(hy + 1) * HX + hx], p[(hy - 1) * HX + hx], st);
    if (three_d)
      dZ[v] = slope1<R>(x, qp[(v * HY + hy) * HX + hx], qm[(v * HY + hy) * HX + hx], st);
    else
      dZ[v] = R(0);
  }
}

// ---------------------------------------------------------------------------
// 2D: one CTA = one TX x TY tile of interior cells.  hydro2d_tile is the tile
// body shared by the single-solver kernel and the ensemble kernel.
// ---------------------------------------------------------------------------
// LOADED: the caller already stored the tile's primitive plane in sQ (the
// ensemble's prefetch); otherwise it is loaded here.
// pre: the step scalars computed for the whole instance (the ensemble), else
// thread 0 computes them for this CTA.
template <class S, class R, int TX, int TY, int RS = 3, bool GRAV = false, bool LOADED = false>
__device__ __forceinline__ void
hydro2d_tile(const S * __restrict__ Uin, S * __restrict__ Uout, const KParams & P, DevClock * clk,
             int step, int bx, int by, unsigned char * smem_raw, const StepScalars<R> * pre = nullptr)
{
  constexpr int NV = 4, HX = TX + 4, HY = TY + 4, NT = TX * TY;
  constexpr int FX = TX + 2; // face-state rows in x: cells -1..TX
  R * sQ = reinterpret_cast<R *>(smem_raw);  // [NV][HY][HX]
  R * sXm = sQ + NV * HY * HX;               // XMIN state of cells -1..TX, then x-flux
  R * sXp = sXm + NV * TY * FX;              // XMAX state
  R * sYm = sXp + NV * TY * FX;              // YMIN state of cells -1..TY, then y-flux
  R * sYp = sYm + NV * (TY + 2) * TX;        // YMAX state

  StepScalars<R> ss;
  if (pre)
  {
    ss = *pre;
    if (!ss.active)
      return;
  }
  else
  {
    StepConsts c; // computed once for the step by the last block of the kernel before
    if (!step_consts(clk, step, c))
      return;
    ss.t = c.t;
    ss.dt = c.dt;
    ss.dtdx = to_r<R>(c.dtdx);
    ss.dtdy = to_r<R>(c.dtdy);
    ss.dtdz = to_r<R>(c.dtdz);
    ss.active = 1;
  }
  const double        t = ss.t, dt = ss.dt;
  const R             dtdx = ss.dtdx, dtdy = ss.dtdy;
  const HydroConst<R> C = hydro_const<R>(P);
  const R             hdt = (R)(0.5 * dt);
  const bool          kick = GRAV && P.grav_hancock; // gravity predictor of the face states
  // (dt/2) g of tile cell (cx, cy), for the predictor
  auto half_g = [&](int cx, int cy, R (&hg)[3]) {
    R g[3];
    grav_at<S, R, NV>(P, P.gw + bx * TX + cx, P.gw + by * TY + cy, 0, g);
#pragma unroll
    for (int e = 0; e < 3; ++e)
      hg[e] = hdt * g[e];
  };

  const int gi0 = P.gw + bx * TX, gj0 = P.gw + by * TY;
  if constexpr (!LOADED)
  {
    load_q_plane<S, R, NV, TX, TY>(Uin, P, C, gi0, gj0, 0, sQ);
    __syncthreads();
  }

  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  // traces of the interior cell
  {
    R c[NV], dX[NV], dY[NV], dZ[NV], s[NV], f[NV];
    cell_slopes<R, NV, HX, HY>(sQ, sQ, sQ, tx + 2, ty + 2, C.slope_type, c, dX, dY, dZ, false);
    hydro_sources<R, NV>(c, dX, dY, dZ, s, C);
    R hg[3];
    if (kick)
      half_g(tx, ty, hg);
    hydro_face<R, NV>(c, dX, s, dtdx, false, f, C.smallr);
    if (kick)
      grav_kick<R, NV>(f, hg);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sXm[(v * TY + ty) * FX + tx + 1] = f[v];
    hydro_face<R, NV>(c, dX, s, dtdx, true, f, C.smallr);
    if (kick)
      grav_kick<R, NV>(f, hg);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sXp[(v * TY + ty) * FX + tx + 1] = f[v];
    hydro_face<R, NV>(c, dY, s, dtdy, false, f, C.smallr);
    if (kick)
      grav_kick<R, NV>(f, hg);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sYm[(v * (TY + 2) + ty + 1) * TX + tx] = f[v];
    hydro_face<R, NV>(c, dY, s, dtdy, true, f, C.smallr);
    if (kick)
      grav_kick<R, NV>(f, hg);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sYp[(v * (TY + 2) + ty + 1) * TX + tx] = f[v];
  }
  // ring cells: only the face state facing the tile
  for (int r = threadIdx.x; r < 2 * (TX + TY); r += NT)
  {
    int cx, cy, kind; // kind 0: left (XMAX), 1: right (XMIN), 2: bottom (YMAX), 3: top (YMIN)
    if (r < TY)
    {
      cx = -1, cy = r, kind = 0;
    }
    else if (r < 2 * TY)
    {
      cx = TX, cy = r - TY, kind = 1;
    }
    else if (r < 2 * TY + TX)
    {
      cx = r - 2 * TY, cy = -1, kind = 2;
    }
    else
    {
      cx = r - 2 * TY - TX, cy = TY, kind = 3;
    }
    R c[NV], dX[NV], dY[NV], dZ[NV], s[NV], f[NV];
    cell_slopes<R, NV, HX, HY>(sQ, sQ, sQ, cx + 2, cy + 2, C.slope_type, c, dX, dY, dZ, false);
    hydro_sources<R, NV>(c, dX, dY, dZ, s, C);
    R hg[3];
    if (kick)
      half_g(cx, cy, hg);
    if (kind < 2)
    {
      hydro_face<R, NV>(c, dX, s, dtdx, kind == 0, f, C.smallr);
      if (kick)
        grav_kick<R, NV>(f, hg);
      R * dst = kind == 0 ? sXp : sXm;
#pragma unroll
      for (int v = 0; v < NV; ++v)
        dst[(v * TY + cy) * FX + cx + 1] = f[v];
    }
    else
    {
      hydro_face<R, NV>(c, dY, s, dtdy, kind == 2, f, C.smallr);
      if (kick)
        grav_kick<R, NV>(f, hg);
      R * dst = kind == 2 ? sYp : sYm;
#pragma unroll
      for (int v = 0; v < NV; ++v)
        dst[(v * (TY + 2) + cy + 1) * TX + cx] = f[v];
    }
  }
  __syncthreads();

  // fluxes: x-face i (left face of cell i) from XMAX(i-1), XMIN(i); stored
  // scaled by dt/dx into the XMIN slot of cell i (HydroRunFunctors2D.h:653-661)
  for (int fidx = threadIdx.x; fidx < (TX + 1) * TY; fidx += NT)
  {
    const int i = fidx % (TX + 1), j = fidx / (TX + 1);
    R         ql[NV], qr[NV], fl[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
    {
      ql[v] = sXp[(v * TY + j) * FX + i];
      qr[v] = sXm[(v * TY + j) * FX + i + 1];
    }
    hydro_riemann<RS, R, NV>(ql, qr, fl, C);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sXm[(v * TY + j) * FX + i + 1] = fl[v] * dtdx;
  }
  // y-faces: swap IU/IV around the solver (HydroRunFunctors2D.h:741-758)
  for (int fidx = threadIdx.x; fidx < TX * (TY + 1); fidx += NT)
  {
    const int i = fidx % TX, j = fidx / TX;
    R         ql[NV], qr[NV], fl[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
    {
      ql[v] = sYp[(v * (TY + 2) + j) * TX + i];
      qr[v] = sYm[(v * (TY + 2) + j + 1) * TX + i];
    }
    R tmp = ql[IU];
    ql[IU] = ql[IV];
    ql[IV] = tmp;
    tmp = qr[IU];
    qr[IU] = qr[IV];
    qr[IV] = tmp;
    hydro_riemann<RS, R, NV>(ql, qr, fl, C);
    tmp = fl[IU];
    fl[IU] = fl[IV];
    fl[IV] = tmp;
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sYm[(v * (TY + 2) + j + 1) * TX + i] = fl[v] * dtdy;
  }
  __syncthreads();

  // update (UpdateFunctor2D, HydroRunFunctors2D.h:809-836), in its order
  const int gi = gi0 + tx, gj = gj0 + ty;
  R tmax = R(-INFINITY);
  if (gi < P.nx + P.gw && gj < P.ny + P.gw)
  {
    const long long off = (long long)gj * P.isize + gi;
    R               u[NV], rho_old = R(0);
#pragma unroll
    for (int v = 0; v < NV; ++v)
    {
      R x = (R)ldg(Uin + v * P.vstride + off);
      if (v == ID)
        rho_old = x;
      x += sXm[(v * TY + ty) * FX + tx + 1];
      x -= sXm[(v * TY + ty) * FX + tx + 2];
      x += sYm[(v * (TY + 2) + ty + 1) * TX + tx];
      x -= sYm[(v * (TY + 2) + ty + 2) * TX + tx];
      u[v] = x;
    }
    R g[3];
    if constexpr (GRAV)
    {
      // gravity source term after the flux update (SolverHydroMuscl.cpp:245-252)
      grav_at<S, R, NV>(P, gi, gj, 0, g);
      grav_source<R, NV>(u, rho_old, g, hdt, C);
    }
    // the next step's dt is computed on the stored (possibly rounded) state
    R us[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
    {
      Uout[v * P.vstride + off] = (S)u[v];
      us[v] = (R)(S)u[v];
    }
    if constexpr (GRAV)
      tmax = fmax(tmax, hydro_invdt_grav<R, NV>(us, g, C, P));
    else
      tmax = fmax(tmax, hydro_invdt<R, NV>(us, C, P));
  }
  block_max_commit<NT>(cand_key((double)tmax), &clk->key[(step + 1) % 3]);
  if (bx == 0 && by == 0 && threadIdx.x == 0)
    step_commit(clk, step, t, dt);
}

template <class S, class R, int TX, int TY, int RS, bool GRAV>
__global__ void __launch_bounds__(TX * TY)
hydro2d_step(const S * __restrict__ Uin, S * __restrict__ Uout, KParams P, DevClock * clk, int step)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  hydro2d_tile<S, R, TX, TY, RS, GRAV>(Uin, Uout, P, clk, step, blockIdx.x, blockIdx.y, smem_raw);
  finalize_step(clk, P, step + 1); // the next step's dt, once its CFL key is complete
}

// ---------------------------------------------------------------------------
// Ensemble of independent 2D runs (uneven grids, own dt each): a persistent
// kernel walks the flat (instance, tile) work list; one launch = one step of
// every instance.  No inter-block waits.
// ---------------------------------------------------------------------------
// raw conserved variables of a tile's (TX+4) x (TY+4) halo plane, gathered
// from the boundary-mapped cells by per-thread asynchronous copies
template <class S, int NV, int TX, int TY>
__device__ __forceinline__ void
issue_raw_plane(const S * __restrict__ U, const KParams & P, int gi0, int gj0, S * raw)
{
  constexpr int HX = TX + 4, HY = TY + 4, NT = TX * TY;
  for (int c = threadIdx.x; c < HX * HY; c += NT)
  {
    const SrcCell s = src_cell(P, gi0 - 2 + c % HX, gj0 - 2 + c / HX, 0);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      cp_async<sizeof(S)>(raw + v * HY * HX + c, U + v * P.vstride + s.off);
  }
}
// ... and, once this thread's copies landed, the primitives of the cells it
// copied (reflecting walls flip the normal velocity, as load_q_plane does)
template <class S, class R, int NV, int TX, int TY>
__device__ __forceinline__ void
convert_raw_plane(const S * raw, const KParams & P, const HydroConst<R> & C, int gi0, int gj0, R * sQ)
{
  constexpr int HX = TX + 4, HY = TY + 4, NT = TX * TY;
  for (int c = threadIdx.x; c < HX * HY; c += NT)
  {
    const SrcCell s = src_cell(P, gi0 - 2 + c % HX, gj0 - 2 + c / HX, 0);
    R             u[NV], q[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      u[v] = neg_if((R)raw[v * HY * HX + c], flips(s, v, 0));
    hydro_prims<R, NV>(u, q, C);
#pragma unroll
    for (int v = 0; v < NV; ++v)
      sQ[v * HY * HX + c] = q[v];
  }
}

template <class S, class R, int TX, int TY>
__host__ __device__ constexpr size_t
ensemble_raw_bytes()
{
  return sizeof(S) * 4 * (TX + 4) * (TY + 4);
}

// The step scalars (active, t, dt, dt/dx, dt/dy) of every instance, once per
// step: the FP64 divisions run in one thread per instance, not per tile.
template <class R>
__global__ void
ensemble_scalars_kernel(const EnsInstance * __restrict__ insts, int n, const int * __restrict__ stepc,
                        StepScalars<R> * __restrict__ out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const KParams & P = insts[i].P;
  double          t = 0.0, dt = 0.0;
  StepScalars<R>  s;
  s.active = step_dt(P, insts[i].clk, *stepc, &t, &dt) ? 1 : 0;
  s.t = t;
  s.dt = dt;
  s.dtdx = (R)(dt / P.dx);
  s.dtdy = (R)(dt / P.dy);
  s.dtdz = (R)(dt / P.dz);
  out[i] = s;
}

template <class S, class R, int TX, int TY>
__global__ void __launch_bounds__(TX * TY)
ensemble2d_step(const EnsInstance * __restrict__ insts, const EnsTile * __restrict__ tiles, int ntiles,
                const int * __restrict__ stepc, size_t tile_smem, const StepScalars<R> * __restrict__ scal)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // raw staging of the next work item's plane, after the tile's own buffers
  S * raw = reinterpret_cast<S *>(smem_raw + tile_smem);
  // the step number lives in device memory (advanced by ensemble_advance after
  // every step), so a captured sequence of steps can be replayed as is
  const int step = *stepc;
  // the plane of work item t is gathered while item t - gridDim.x computes
  auto issue = [&](int t) {
    const EnsTile       w = tiles[t];
    const EnsInstance & in = insts[w.inst];
    issue_raw_plane<S, 4, TX, TY>((const S *)in.U[step % 2], in.P, in.P.gw + w.bx * TX, in.P.gw + w.by * TY, raw);
    cp_async_commit();
  };
  if (blockIdx.x < ntiles)
    issue(blockIdx.x);
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
  {
    const EnsTile       w = tiles[t];
    const EnsInstance & in = insts[w.inst];
    const int           gi0 = in.P.gw + w.bx * TX, gj0 = in.P.gw + w.by * TY;
    cp_async_wait_all();
    convert_raw_plane<S, R, 4, TX, TY>(raw, in.P, hydro_const<R>(in.P), gi0, gj0, reinterpret_cast<R *>(smem_raw));
    // every thread converted the cells it copied: the staging is free again
    if (t + gridDim.x < ntiles)
      issue(t + gridDim.x);
    __syncthreads(); // the primitive plane is complete
    hydro2d_tile<S, R, TX, TY, 3, false, true>((const S *)in.U[step % 2], (S *)in.U[(step + 1) % 2], in.P,
                                                in.clk, step, w.bx, w.by, smem_raw, scal + w.inst);
    __syncthreads(); // shared tiles are reused by the next work item
  }
  cp_async_wait_all(); // no copy may land after the block has left
}

__global__ void
ensemble_advance(int * stepc)
{
  *stepc += 1;
}

// FP64 mass and total energy of every instance (blockIdx.y = instance)
template <class S>
__global__ void
ensemble_totals_kernel(const EnsInstance * __restrict__ insts, const int * __restrict__ stepc,
                       double * __restrict__ out)
{
  const EnsInstance & in = insts[blockIdx.y];
  const KParams &     P = in.P;
  const S *           U = (const S *)in.U[*stepc % 2];
  double              m = 0.0, e = 0.0;
  for_interior_rows(P, [&](int i, int j, int) {
    const long long off = (long long)j * P.isize + i;
    m += (double)U[off];
    e += (double)U[P.vstride + off];
  });
  for (int o = 16; o > 0; o >>= 1)
  {
    m += __shfl_xor_sync(0xffffffffu, m, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
  }
  if ((threadIdx.x & 31) == 0)
  {
    atomicAdd(out + 2 * blockIdx.y, m);
    atomicAdd(out + 2 * blockIdx.y + 1, e);
  }
}


// ---------------------------------------------------------------------------
// 3D: one CTA = a TX x TY column of interior cells marching over kchunk planes
// ---------------------------------------------------------------------------
template <class S, class R, int TX, int TY, int RS, bool GRAV, bool TMA>
__global__ void __launch_bounds__(TX * TY, EK_MINB(R, EK_H3_MINB_F32, EK_H3_MINB_F64))
hydro3d_step(const S * __restrict__ Uin, S * __restrict__ Uout, KParams P, DevClock * clk, int step,
             const __grid_constant__ CUtensorMap tmap)
{
  constexpr int NV = 5, HX = TX + 4, HY = TY + 4, NT = TX * TY;
  constexpr int FX = TX + 2;
  constexpr int QP = hydro3d_slot_elems<R, TX, TY>(); // one primitive plane (padded)
  // [3][NV][HY][HX] ring of planes, 128-byte aligned for the tensor copies
  extern __shared__ __align__(128) unsigned char smem_ring[];
  R * sQ = reinterpret_cast<R *>(smem_ring);
  R * sXm = sQ + 3 * QP;
  R * sXp = sXm + NV * TY * FX;
  R * sYm = sXp + NV * TY * FX;
  R * sYp = sYm + NV * (TY + 2) * TX;

  StepConsts sc; // computed once for the step by the last block of the kernel before
  if (!step_consts(clk, step, sc))
    return;
  const double        t = sc.t, dt = sc.dt;
  const R             dtdx = to_r<R>(sc.dtdx), dtdy = to_r<R>(sc.dtdy), dtdz = to_r<R>(sc.dtdz);
  const HydroConst<R> C = hydro_const<R>(P);
  const R             hdt = (R)(0.5 * dt);
  const bool          kick = GRAV && P.grav_hancock; // gravity predictor of the face states

  const int gw = P.gw;
  const int gi0 = gw + blockIdx.x * TX, gj0 = gw + blockIdx.y * TY;
  const int k0 = blockIdx.z * P.kchunk; // interior plane index
  const int k1 = min(k0 + P.kchunk, P.nz);
  const int tx = threadIdx.x % TX, ty = threadIdx.x / TX;
  const int gi = gi0 + tx, gj = gj0 + ty;
  const bool own = gi < P.nx + gw && gj < P.ny + gw;
  const long long own_off = (long long)gj * P.isize + gi;

  // tile halo inside the interior in x and y: no boundary mapping needed
  const bool xy_in = gi0 - 2 >= gw && gi0 + TX + 1 < P.nx + gw && gj0 - 2 >= gw && gj0 + TY + 1 < P.ny + gw;
  auto       plane_in = [&](int gk) { return xy_in && gk >= gw && gk < P.nz + gw; };

  // Planes whose whole tile halo lies in the interior are staged by a tensor
  // copy of the (HX, HY, 1, NV) box of U, started one plane ahead (while the
  // previous plane's fluxes and update run) and converted in place; the other
  // planes are loaded through the boundary mapping.  One copy is in flight at
  // a time, on one mbarrier.
  __shared__ unsigned long long tma_bar;
  __shared__ int                tma_bad;
  const bool                    tma = TMA && xy_in && (smem_addr(sQ) & 127u) == 0;
  if constexpr (TMA)
  {
    if (threadIdx.x == 0)
    {
      tma_bad = 0;
      if (tma)
        mbar_init(&tma_bar, 1);
    }
    __syncthreads();
  }
  constexpr unsigned TMA_BYTES = NV * HX * HY * sizeof(S);
  auto tma_issue = [&](int p) { // one thread: interior plane p into its ring slot
    mbar_expect_tx(&tma_bar, TMA_BYTES);
    tma_load_4d(sQ + ((p + 3) % 3) * QP, &tmap, gi0 - 2, gj0 - 2, p + gw, 0, &tma_bar);
  };
  // The copied planes are the interior ones (0 <= p < nz) from k0 on, one per
  // iteration: plane kc+1 is in flight at the top of iteration kc when it is
  // interior, and it is copy number kc+1-k0 on the barrier (phase parity).
  auto pending = [&](int kc) { return tma && kc + 1 < P.nz; };

  // prologue: planes k0-2, k0-1, and the copy of k0
  load_q_plane<S, R, NV, TX, TY>(Uin, P, C, gi0, gj0, k0 - 2 + gw, sQ + ((k0 + 1) % 3) * QP,
                                 plane_in(k0 - 2 + gw));
  load_q_plane<S, R, NV, TX, TY>(Uin, P, C, gi0, gj0, k0 - 1 + gw, sQ + ((k0 + 2) % 3) * QP,
                                 plane_in(k0 - 1 + gw));
  if (pending(k0 - 1) && threadIdx.x == 0)
    tma_issue(k0);

  R zmax_prev[NV];        // ZMAX face state of the cell below
  R acc[NV];              // partial update of the cell below, waiting for -Fz(k)
  R rho_prev = R(0);      // its density before the update (gravity source term)
  R tmax = R(-INFINITY);  // CFL candidate max of the cells this thread wrote
  // (dt/2) g of the cell at raw indexes (i, j, k), for the predictor
  auto half_g = [&](int i, int j, int k, R (&hg)[3]) {
    R g[3];
    grav_at<S, R, NV>(P, i, j, k, g);
#pragma unroll
    for (int e = 0; e < 3; ++e)
      hg[e] = hdt * g[e];
  };

  for (int kc = k0 - 1; kc <= k1; ++kc)
  {
    // plane kc+1 into ring slot (kc+1)%3  [(kc+1+3)%3 to stay non-negative]
    if (pending(kc))
    {
      if (!mbar_wait(&tma_bar, (unsigned)(kc + 1 - k0) & 1u, 1000000000ull))
        tma_bad = 1;
      convert_q_plane<R, NV, TX, TY>(sQ + ((kc + 4) % 3) * QP, C);
    }
    else
      load_q_plane<S, R, NV, TX, TY>(Uin, P, C, gi0, gj0, kc + 1 + gw, sQ + ((kc + 4) % 3) * QP,
                                     plane_in(kc + 1 + gw));
    __syncthreads();
    if (TMA && tma_bad)
    {
      // the copy did not complete within 1 s: report it, give the copy one
      // more bounded wait so it does not land after the block has left
      if (threadIdx.x == 0)
      {
        atomicOr(&clk->error, EK_DEVERR_TMA_TIMEOUT);
        mbar_wait(&tma_bar, (unsigned)(kc + 1 - k0) & 1u, 1000000000ull);
      }
      return;
    }
    const R * q0 = sQ + ((kc + 3) % 3) * QP;
    const R * qm = sQ + ((kc + 2) % 3) * QP;
    const R * qp = sQ + ((kc + 4) % 3) * QP;
    const bool full = kc >= k0 && kc < k1;

    R fz[NV];
    {
      R c[NV], dX[NV], dY[NV], dZ[NV], s[NV], f[NV];
      cell_slopes<R, NV, HX, HY>(q0, qm, qp, tx + 2, ty + 2, C.slope_type, c, dX, dY, dZ, true);
      hydro_sources<R, NV>(c, dX, dY, dZ, s, C);
      R hg[3];
      if (kick)
        half_g(gi, gj, kc + gw, hg);
      if (full)
      {
        hydro_face<R, NV>(c, dX, s, dtdx, false, f, C.smallr);
        if (kick)
          grav_kick<R, NV>(f, hg);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          sXm[(v * TY + ty) * FX + tx + 1] = f[v];
        hydro_face<R, NV>(c, dX, s, dtdx, true, f, C.smallr);
        if (kick)
          grav_kick<R, NV>(f, hg);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          sXp[(v * TY + ty) * FX + tx + 1] = f[v];
        hydro_face<R, NV>(c, dY, s, dtdy, false, f, C.smallr);
        if (kick)
          grav_kick<R, NV>(f, hg);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          sYm[(v * (TY + 2) + ty + 1) * TX + tx] = f[v];
        hydro_face<R, NV>(c, dY, s, dtdy, true, f, C.smallr);
        if (kick)
          grav_kick<R, NV>(f, hg);
#pragma unroll
        for (int v = 0; v < NV; ++v)
          sYp[(v * (TY + 2) + ty + 1) * TX + tx] = f[v];
      }
      if (kc >= k0)
      {
        // z-face between kc-1 and kc: ZMAX(kc-1), ZMIN(kc); swap IU/IW
        // (HydroRunFunctors3D.h:672-707)
        R qr[NV];
        hydro_face<R, NV>(c, dZ, s, dtdz, false, qr, C.smallr);
        if (kick)
          grav_kick<R, NV>(qr, hg);
        R ql[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v)
          ql[v] = zmax_prev[v];
        R tmp = ql[IU];
        ql[IU] = ql[IW];
        ql[IW] = tmp;
        tmp = qr[IU];
        qr[IU] = qr[IW];
        qr[IW] = tmp;
        hydro_riemann<RS, R, NV>(ql, qr, fz, C);
        tmp = fz[IU];
        fz[IU] = fz[IW];
        fz[IW] = tmp;
#pragma unroll
        for (int v = 0; v < NV; ++v)
          fz[v] = fz[v] * dtdz;
      }
      if (kc < k1)
      {
        hydro_face<R, NV>(c, dZ, s, dtdz, true, zmax_prev, C.smallr);
        if (kick)
          grav_kick<R, NV>(zmax_prev, hg);
      }
    }
    if (full)
    {
      for (int r = threadIdx.x; r < 2 * (TX + TY); r += NT)
      {
        int cx, cy, kind;
        if (r < TY)
        {
          cx = -1, cy = r, kind = 0;
        }
        else if (r < 2 * TY)
        {
          cx = TX, cy = r - TY, kind = 1;
        }
        else if (r < 2 * TY + TX)
        {
          cx = r - 2 * TY, cy = -1, kind = 2;
        }
        else
        {
          cx = r - 2 * TY - TX, cy = TY, kind = 3;
        }
        R c[NV], dX[NV], dY[NV], dZ[NV], s[NV], f[NV];
        cell_slopes<R, NV, HX, HY>(q0, qm, qp, cx + 2, cy + 2, C.slope_type, c, dX, dY, dZ, true);
        hydro_sources<R, NV>(c, dX, dY, dZ, s, C);
        R hg[3];
        if (kick)
          half_g(gi0 + cx, gj0 + cy, kc + gw, hg);
        if (kind < 2)
        {
          hydro_face<R, NV>(c, dX, s, dtdx, kind == 0, f, C.smallr);
          if (kick)
            grav_kick<R, NV>(f, hg);
          R * dst = kind == 0 ? sXp : sXm;
#pragma unroll
          for (int v = 0; v < NV; ++v)
            dst[(v * TY + cy) * FX + cx + 1] = f[v];
        }
        else
        {
          hydro_face<R, NV>(c, dY, s, dtdy, kind == 2, f, C.smallr);
          if (kick)
            grav_kick<R, NV>(f, hg);
          R * dst = kind == 2 ? sYp : sYm;
#pragma unroll
          for (int v = 0; v < NV; ++v)
            dst[(v * (TY + 2) + cy + 1) * TX + cx] = f[v];
        }
      }
    }
    // every thread orders its generic accesses of the ring before the tensor
    // copy that will overwrite plane kc-1's slot
    if (tma)
      fence_proxy_async_smem();
    __syncthreads();
    // plane kc-1 is no longer read: start the copy of plane kc+2 into its slot
    if (kc + 1 <= k1 && pending(kc + 1) && threadIdx.x == 0)
      tma_issue(kc + 2);

    if (full)
    {
      // x- and y-faces of the plane as one work list (one HLLC code path;
      // the y-faces swap IU and IV around the solver)
      constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1);
      for (int fidx = threadIdx.x; fidx < NFX + NFY; fidx += NT)
      {
        const bool ydir = fidx >= NFX;
        const int  g = ydir ? fidx - NFX : fidx;
        const int  i = ydir ? g % TX : g % (TX + 1), j = ydir ? g / TX : g / (TX + 1);
        const R *  lsrc = ydir ? sYp + j * TX + i : sXp + j * FX + i;
        R *        rsrc = ydir ? sYm + (j + 1) * TX + i : sXm + j * FX + i + 1;
        const int  vs = ydir ? (TY + 2) * TX : TY * FX; // variable stride
        R          ql[NV], qr[NV], fl[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v)
        {
          ql[v] = lsrc[v * vs];
          qr[v] = rsrc[v * vs];
        }
        if (ydir)
        {
          R tmp = ql[IU];
          ql[IU] = ql[IV];
          ql[IV] = tmp;
          tmp = qr[IU];
          qr[IU] = qr[IV];
          qr[IV] = tmp;
        }
        hydro_riemann<RS, R, NV>(ql, qr, fl, C);
        if (ydir)
        {
          R tmp = fl[IU];
          fl[IU] = fl[IV];
          fl[IV] = tmp;
        }
        const R dtd = ydir ? dtdy : dtdx;
#pragma unroll
        for (int v = 0; v < NV; ++v)
          rsrc[v * vs] = fl[v] * dtd;
      }
      __syncthreads();
    }

    // finish the cell below: U(kc-1) -= Fz(kc)  (UpdateFunctor3D order,
    // HydroRunFunctors3D.h:775-809), store it and take its CFL candidate
    if (kc > k0 && own)
    {
      R u[NV], us[NV];
      const long long off = own_off + (long long)(kc - 1 + gw) * P.plane;
#pragma unroll
      for (int v = 0; v < NV; ++v)
        u[v] = acc[v] - fz[v];
      R g[3];
      if constexpr (GRAV)
      {
        // gravity source term after the flux update (SolverHydroMuscl.cpp:333-338)
        grav_at<S, R, NV>(P, gi, gj, kc - 1 + gw, g);
        grav_source<R, NV>(u, rho_prev, g, hdt, C);
      }
#pragma unroll
      for (int v = 0; v < NV; ++v)
      {
        Uout[v * P.vstride + off] = (S)u[v];
        us[v] = (R)(S)u[v];
      }
      if constexpr (GRAV)
        tmax = fmax(tmax, hydro_invdt_grav<R, NV>(us, g, C, P));
      else
        tmax = fmax(tmax, hydro_invdt<R, NV>(us, C, P));
    }
    if (full && own)
    {
      const long long off = own_off + (long long)(kc + gw) * P.plane;
#pragma unroll
      for (int v = 0; v < NV; ++v)
      {
        R x = (R)ldg(Uin + v * P.vstride + off);
        if (v == ID)
          rho_prev = x;
        x += sXm[(v * TY + ty) * FX + tx + 1];
        x -= sXm[(v * TY + ty) * FX + tx + 2];
        x += sYm[(v * (TY + 2) + ty + 1) * TX + tx];
        x -= sYm[(v * (TY + 2) + ty + 2) * TX + tx];
        x += fz[v];
        acc[v] = x;
      }
    }
    __syncthreads(); // ring slot and face buffers are reused next plane
  }
  block_max_commit<NT>(cand_key((double)tmax), &clk->key[(step + 1) % 3]);
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0)
    step_commit(clk, step, t, dt);
  finalize_step(clk, P, step + 1); // the next step's dt, once its CFL key is complete
}

// ---------------------------------------------------------------------------
// CFL reduction over the interior of a state (ComputeDtFunctor{2D,3D});
// used after the state is set (the constructor's compute_dt()).
// ---------------------------------------------------------------------------
template <class S, class R, int NV, bool GRAV>
__global__ void
hydro_dt_kernel(const S * __restrict__ U, KParams P, unsigned long long * key, DevClock * fin, int fin_step)
{
  const HydroConst<R> C = hydro_const<R>(P);
  R                   tmax = R(-INFINITY);
  for_interior_rows(P, [&](int i, int j, int k) {
    const long long off = (long long)k * P.plane + (long long)j * P.isize + i;
    R               u[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v)
      u[v] = (R)ldg(U + v * P.vstride + off);
    if constexpr (GRAV)
    {
      R g[3];
      grav_at<S, R, NV>(P, i, j, k, g);
      tmax = fmax(tmax, hydro_invdt_grav<R, NV>(u, g, C, P));
    }
    else
      tmax = fmax(tmax, hydro_invdt<R, NV>(u, C, P));
  });
  block_max_commit<256>(cand_key((double)tmax), key);
  if (fin)
    finalize_step(fin, P, fin_step); // the constants of the step this key is for
}

// Fill the ghost cells of a state in memory (make_boundaries_serial result,
// SolverBase.cpp:488-512), for callers that read the full array back.  U
// points at the plane of variable var0; nbvar planes are filled.
template <class S>
__global__ void
fill_ghosts_kernel(S * __restrict__ U, KParams P, int nbvar, int var0)
{
  const long long n = P.vstride;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n;
       c += (long long)gridDim.x * blockDim.x)
  {
    const int       i = (int)(c % P.isize);
    const long long r = c / P.isize;
    const int       j = (int)(r % P.jsize);
    const int       k = (int)(r / P.jsize);
    const bool ghost = i < P.gw || i >= P.nx + P.gw || j < P.gw || j >= P.ny + P.gw ||
                       (P.ksize > 1 && (k < P.gw || k >= P.nz + P.gw));
    if (!ghost)
      continue;
    const SrcCell s = src_cell(P, i, j, k);
    for (int lv = 0; lv < nbvar; ++lv)
    {
      const S x = U[(long long)lv * P.vstride + s.off];
      U[(long long)lv * P.vstride + c] = flips(s, var0 + lv, P.mhd) ? -x : x;
    }
  }
}

} // namespace EK_NS
