"""Host-side helpers of the benchmark, checked on CPU against oracle states.

bench.divb_inner is the interior div B figure the low-beta MHD blast workload
reports beside the global max: face B at the left faces (U[5:8]), cells at
least `margin` cells inside the interior.
"""

import os
import sys

import numpy as np

import eko

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
from euler_kokkos_gb300 import problems as P  # noqa: E402


def _divb_all(U, p):
    g = p.gw
    bx, by, bz = U[5], U[6], U[7]
    n = U.shape[1]
    out = np.zeros((n - 2 * g,) * 3)
    for k in range(g, n - g):
        for j in range(g, n - g):
            i = np.arange(g, n - g)
            out[k - g, j - g] = ((bx[k, j, i + 1] - bx[k, j, i]) / p.dx + (by[k, j + 1, i] - by[k, j, i]) / p.dy +
                                 (bz[k + 1, j, i] - bz[k, j, i]) / p.dz)
    return np.abs(out)


def test_divb_inner_matches_direct_computation():
    ini, U0 = P.mhd_blast_3d(n=16, nsteps=30, by_ratio=0.1)
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    o.run(30)
    U = o.state()
    o.close()
    d = _divb_all(U, p)
    for m in (0, 1, 4):
        want = d[m:d.shape[0] - m, m:d.shape[1] - m, m:d.shape[2] - m].max()
        assert bench.divb_inner(U, p.gw, m, p.dx, p.dy, p.dz) == want
    # the outflow fill leaves div B in the outermost layer only; inside, CT keeps
    # it at FP64 round-off
    bscale = np.abs(U0[5:]).max() / p.dx
    assert bench.divb_inner(U, p.gw, 1, p.dx, p.dy, p.dz) <= 1e-12 * bscale
    assert bench.divb_inner(U, p.gw, 0, p.dx, p.dy, p.dz) > 1e-6 * bscale


def test_headline_traffic_covers_every_kernel_of_the_step():
    # the headline's whole-step roofline sums traffic per cell over the
    # step's kernels (ncu figures in bench.TRAFFIC_PER_CELL); a kernel
    # without an entry would leave the JSON line's `traffic` null
    names = [name for _, name in bench.KERNEL_NAMES["mhd3d"]]
    traffic = bench.TRAFFIC_PER_CELL[("mhd3d", "mixed")]
    assert "mhd_repair_kernel" in names
    assert all(name in traffic for name in names), (names, sorted(traffic))
    # and the kernel ids are distinct (ek_solver_kernel_time slots)
    ids = [i for i, _ in bench.KERNEL_NAMES["mhd3d"]]
    assert len(set(ids)) == len(ids) and all(0 <= i <= 3 for i in ids)
