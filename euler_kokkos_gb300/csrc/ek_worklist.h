// The work items of one plane of the MHD 3D update kernel's tile (faces and
// edges), and their two orders.  Plain C++ with CUDA qualifiers where a CUDA
// compiler reads it, so the host tests can check the enumeration.
#pragma once

#ifdef __CUDACC__
#define EK_WL_HD __host__ __device__ __forceinline__
#else
#define EK_WL_HD inline
#endif

namespace ekc
{

template <int TX, int TY>
struct UpdTile
{
  static constexpr int XE = TX + 2, YE = TY + 2, PL = XE * YE; // trace cells per plane
  static constexpr int FXS = (TX + 1) * TY, FYS = TX * (TY + 1), FZS = TX * TY;
  static constexpr int EZS = (TX + 1) * (TY + 1), EYS = (TX + 1) * TY, EXS = TX * (TY + 1);
  // The work items of a plane, in segments of 32 (one warp each).  First the
  // edges of the tile: row TY (y-faces, x-edges, z-edges: TX each) and column
  // TX (x-faces, y-edges: TY each; z-edges: TY + 1), each kind in segments of
  // its own.  Then rows 0..TY-1 in groups of RG rows, six kinds of TX items
  // per row, their order rotated by one kind per row group: with a fixed
  // order, warp w would take the kinds w, w + 8, w + 16 (mod 6), always three
  // faces or always three edges per two warps, and edges cost about twice a
  // face.  item() is false for a padding slot.
  static constexpr int RG = TX < 32 ? 32 / TX : 1;
  static_assert(TY % RG == 0, "rows per item group must divide TY");
  static constexpr int RSEG = (TX + 31) / 32, CSEG = (TY + 1 + 31) / 32;
  static constexpr int NTAIL = 32 * 3 * (RSEG + CSEG), NMAIN = 6 * TX * TY;
  static constexpr int NITEMS = NTAIL + NMAIN;
  EK_WL_HD static bool
  item(int w, int & kind, int & li, int & lj)
  {
    if (w < NTAIL)
    {
      const int seg = w / 32, lane = w % 32;
      if (seg < 3 * RSEG)
      {
        const int q = seg / RSEG;
        kind = q == 0 ? 2 : (q == 1 ? 4 : 5);
        li = (seg % RSEG) * 32 + lane;
        lj = TY;
        return li < TX;
      }
      const int c = seg - 3 * RSEG, q = c / CSEG;
      kind = q == 0 ? 1 : (q == 1 ? 3 : 5);
      li = TX;
      lj = (c % CSEG) * 32 + lane;
      return lj < (q == 2 ? TY + 1 : TY);
    }
    const int v = w - NTAIL;
    li = v % TX;
    const int g = v / TX; // (row group, kind position, row in group)
    const int rg = g / (6 * RG);
    kind = ((g / RG) % 6 + rg) % 6;
    lj = rg * RG + g % RG;
    return true;
  }
  // the same items by kind: z-, x-, y-faces (padded to whole warps), then y-,
  // x-, z-edges; false for a padding item
  static constexpr int NFACES = FZS + FXS + FYS, NFP = (NFACES + 31) & ~31;
  static constexpr int NITEMS_K = NFP + EYS + EXS + EZS;
  EK_WL_HD static bool
  item_by_kind(int w, int & kind, int & li, int & lj)
  {
    if (w < NFP)
    {
      if (w >= NFACES)
        return false;
      int f = w;
      kind = 0;
      if (f >= FZS)
      {
        f -= FZS;
        kind = 1;
        if (f >= FXS)
          f -= FXS, kind = 2;
      }
      li = kind == 1 ? f % (TX + 1) : f % TX;
      lj = kind == 1 ? f / (TX + 1) : f / TX;
      return true;
    }
    int e = w - NFP;
    kind = 3;
    if (e >= EYS)
    {
      e -= EYS;
      kind = 4;
      if (e >= EXS)
        e -= EXS, kind = 5;
    }
    li = kind == 4 ? e % TX : e % (TX + 1);
    lj = kind == 4 ? e / TX : e / (TX + 1);
    return true;
  }
};


} // namespace ekc
