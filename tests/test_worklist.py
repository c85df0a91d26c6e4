"""The work items of the MHD 3D update kernel's tile
(euler_kokkos_gb300/csrc/ek_worklist.h), compiled as plain C++ on the host:
both orders (rows for the mixed form, kinds for FP64) visit every face and
every edge of the tile exactly once, for the tile shapes the tuner can choose,
and in the row order no warp's 32 items mix item kinds."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "euler_kokkos_gb300", "csrc")

PROGRAM = r"""
#include "ek_worklist.h"
#include <cstdio>
#include <set>
#include <tuple>

// kinds 0..5: z-, x-, y-face, y-, x-, z-edge at local cell (li, lj)
template <int TX, int TY>
static std::set<std::tuple<int, int, int>> expected()
{
  std::set<std::tuple<int, int, int>> e;
  for (int li = 0; li <= TX; ++li)
    for (int lj = 0; lj <= TY; ++lj)
    {
      if (li < TX && lj < TY) e.insert({0, li, lj});
      if (lj < TY) e.insert({1, li, lj});
      if (li < TX) e.insert({2, li, lj});
      if (lj < TY) e.insert({3, li, lj});
      if (li < TX) e.insert({4, li, lj});
      e.insert({5, li, lj});
    }
  return e;
}

template <int TX, int TY>
static int check()
{
  using T = ekc::UpdTile<TX, TY>;
  const auto want = expected<TX, TY>();
  int bad = 0;
  for (int order = 0; order < 2; ++order)
  {
    std::set<std::tuple<int, int, int>> seen;
    const int n = order == 0 ? T::NITEMS : T::NITEMS_K;
    for (int w0 = 0; w0 < n; w0 += 32)
    {
      int warp_kind = -1;
      for (int w = w0; w < w0 + 32 && w < n; ++w)
      {
        int kind, li, lj;
        if (!(order == 0 ? T::item(w, kind, li, lj) : T::item_by_kind(w, kind, li, lj)))
          continue;
        if (!seen.insert({kind, li, lj}).second)
        {
          std::printf("%dx%d order %d: item (%d, %d, %d) twice\n", TX, TY, order, kind, li, lj);
          ++bad;
        }
        if (order == 0 && warp_kind >= 0 && kind != warp_kind)
        {
          std::printf("%dx%d: warp at %d mixes kinds %d and %d\n", TX, TY, w0, warp_kind, kind);
          ++bad;
        }
        warp_kind = kind;
      }
    }
    if (seen != want)
    {
      std::printf("%dx%d order %d: %zu items, %zu expected\n", TX, TY, order, seen.size(), want.size());
      ++bad;
    }
  }
  return bad;
}

int main()
{
  const int bad = check<32, 8>() + check<16, 8>() + check<32, 4>() + check<64, 4>() + check<32, 16>() +
                  check<16, 16>() + check<8, 8>();
  std::printf(bad ? "FAIL\n" : "OK\n");
  return bad != 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_update_work_items_cover_each_face_and_edge_once(tmp_path):
    src = tmp_path / "worklist_check.cpp"
    exe = tmp_path / "worklist_check"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout
