"""The op-counting build of the oracle (oracle/ek_opcount.cpp): the reference
algorithm's floating-point operations per cell-update, the FLOP numerator of
the benchmark's roofline (bench.FLOPS_PER_CELL).

CPU only.  The counting build must compute exactly what the plain build
computes (same states and dt, bit for bit), and the per-cell counts the
benchmark quotes must be what it measures on the named workloads (checked
here on smaller grids of the same problems, where the boundary faces add a
little).
"""

import os
import sys

import numpy as np
import pytest

import eko

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
from euler_kokkos_gb300 import problems as P  # noqa: E402


def _run(params, U0, nsteps, counting):
    o = eko.Oracle(params, U0, counting=counting)
    dts = o.run(nsteps)
    U = o.state()
    o.close()
    return dts, U


@pytest.mark.parametrize("case", ["blast3d", "ot3d", "ot2d", "kh2d"])
def test_counting_build_is_bitwise_the_oracle(case):
    ini, U0 = {
        "blast3d": lambda: P.blast_3d(n=16, nsteps=10),
        "ot3d": lambda: P.orszag_tang_3d(n=12, nsteps=10),
        "ot2d": lambda: P.orszag_tang_2d(n=32, nsteps=10),
        "kh2d": lambda: P.kelvin_helmholtz_2d(n=32, nsteps=10),
    }[case]()
    p = eko.params_from_ini(ini)
    d0, U0_plain = _run(p, U0, 3, False)
    d1, U0_count = _run(p, U0, 3, True)
    assert np.array_equal(d0, d1)
    assert np.array_equal(U0_plain, U0_count)


def test_counts_are_deterministic_and_by_kind():
    ini, U0 = P.blast_3d(n=12, nsteps=10)
    p = eko.params_from_ini(ini)
    a = eko.count_ops(p, U0, 2)
    b = eko.count_ops(p, U0, 2)
    assert a["counts"] == b["counts"]
    assert a["steps"] == 2 and a["cell_updates"] == 2 * 12 ** 3
    c = a["counts"]
    # the step divides (primitives, HLLC) and takes square roots (sound speed)
    assert all(c[k] > 0 for k in eko.OP_KINDS)
    # one step counts about half of two
    h = eko.count_ops(p, U0, 1)["counts"]
    assert 0.4 < h["mul"] / c["mul"] < 0.6


@pytest.mark.parametrize("key,build,tol", [
    ("hydro3d", lambda: P.blast_3d(n=96, nsteps=10), 0.05),
    ("mhd3d", lambda: P.orszag_tang_3d(n=64, nsteps=10), 0.05),
    ("mhd2d", lambda: P.orszag_tang_2d(n=512, nsteps=10), 0.02),
    ("hydro2d", lambda: P.kelvin_helmholtz_2d(n=128, nsteps=10), 1e-5),  # the quoted grid itself
])
def test_bench_flop_counts(key, build, tol):
    ini, U0 = build()
    r = eko.count_ops(eko.params_from_ini(ini), U0, 2)
    pc = r["per_cell"]
    flops = pc["add"] + pc["mul"] + pc["div"] + pc["sqrt"]
    other = pc["minmax"] + pc["abs"] + pc["neg"] + pc["cmp"]
    want = bench.FLOPS_PER_CELL[key]
    # the quoted grids are at least as large, so they count at most this many
    # boundary-face operations per cell
    # (the quoted figures are rounded to 3 decimals)
    assert want["flops"] <= flops + 1e-3 and flops <= want["flops"] * (1 + tol) + 1e-3
    assert want["other"] <= other + 1e-3 and other <= want["other"] * (1 + tol) + 1e-3
