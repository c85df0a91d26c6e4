"""GPU parity of the CT-MHD 3D step through the C ABI.

* exact build: bit-identical to the reference (golden fixtures, including the
  NaN pattern the reference's HLLD degeneracy test produces in the MHD blast)
  and to the oracle on seeded states with every boundary type and odd sizes;
* FMA build: density, energy and face B within 1e-11 relative L-infinity;
* mixed form: density within 1e-5 relative L1; the CT update of the FP64 face
  field keeps max |div B| at FP64 round-off.
"""

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import golden_cases, interior, load_golden, rel_l1, rel_linf

pytestmark = pytest.mark.gpu

FP64_LINF_TOL = 1e-11
MIXED_L1_TOL = 1e-5


def run_gpu(ini, U0, nsteps, allow_nonfinite=False, **over):
    p = ek.params_from_ini(ini, **over)
    with ek.SolverFactory.create(p.solver_name, p) as s:
        s.set_state(U0)
        n = 0
        while n < nsteps and not s.finished():
            s.next_iteration(allow_nonfinite=allow_nonfinite)
            n += 1
        return s.get_state(), s.dt_history(), s.m_t, s.totals()


def run_oracle(ini, U0, nsteps):
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    dts = o.run(nsteps)
    return o.state(), dts, o.t, p


@pytest.mark.parametrize("name", golden_cases("mhd"))
def test_exact_build_matches_reference_golden_bitwise(name):
    g = load_golden(name)
    ini = str(g["ini"])
    U, dts, t, _ = run_gpu(ini, g["U0"], len(g["dts"]), allow_nonfinite=True, exact_fp=1)
    p = eko.params_from_ini(ini)
    assert np.array_equal(dts, g["dts"], equal_nan=True)
    assert np.array_equal(interior(U, p.gw, 3), interior(g["U"], p.gw, 3), equal_nan=True)


@pytest.mark.parametrize("name", [n for n in golden_cases("mhd") if "nan" not in n])
def test_fma_build_matches_reference_golden(name):
    g = load_golden(name)
    ini = str(g["ini"])
    U, dts, t, _ = run_gpu(ini, g["U0"], len(g["dts"]))
    p = eko.params_from_ini(ini)
    err = rel_linf(interior(U, p.gw, 3), interior(g["U"], p.gw, 3))
    assert err[0] <= FP64_LINF_TOL and err[1] <= FP64_LINF_TOL, err
    assert max(err[5:]) <= FP64_LINF_TOL, err
    assert np.max(np.abs(dts - g["dts"]) / g["dts"]) <= 1e-13


CASES = [
    ("periodic_odd", lambda: P.smooth_random(dim=3, mhd=True, nx=21, ny=11, nz=9, seed=51, bc=(3,) * 6,
                                             nsteps=4), 4, {"kchunk": 4}),
    ("reflect_outflow", lambda: P.smooth_random(dim=3, mhd=True, nx=18, ny=20, nz=7, seed=52,
                                                bc=(1, 2, 2, 1, 1, 2), slope_type=1.0, nsteps=3), 3, {}),
    ("orszag_tang", lambda: P.orszag_tang_3d(n=20, nsteps=5), 5, {"kchunk": 6}),
]


@pytest.mark.parametrize("label,build,nsteps,over", CASES, ids=[c[0] for c in CASES])
def test_exact_build_matches_oracle_bitwise(label, build, nsteps, over):
    ini, U0 = build()
    Ug, dg, tg, _ = run_gpu(ini, U0, nsteps, exact_fp=1, **over)
    Uo, do, to, p = run_oracle(ini, U0, nsteps)
    assert np.array_equal(dg, do)
    assert np.array_equal(interior(Ug, p.gw, 3), interior(Uo, p.gw, 3))


def test_mixed_precision_orszag_tang_error_and_divb():
    ini, U0 = P.orszag_tang_3d(n=32, nsteps=10)
    Ug, dg, _, tot = run_gpu(ini, U0, 10, precision=ek.EK_PREC_MIXED)
    Uo, do, _, p = run_oracle(ini, U0, 10)
    err = rel_l1(interior(Ug, p.gw, 3), interior(Uo, p.gw, 3))
    assert err[0] <= MIXED_L1_TOL, err
    # face B is FP64 and updated by CT in FP64: div B stays at round-off of |B|/dx
    bscale = np.abs(U0[5:]).max() / p.dx
    assert tot[2] <= 1e-12 * bscale, (tot[2], bscale)


def test_fp64_divb_stays_at_roundoff():
    ini, U0 = P.smooth_random(dim=3, mhd=True, nx=24, ny=16, nz=12, seed=61, bc=(3,) * 6, nsteps=8)
    p = eko.params_from_ini(ini)
    _, _, _, tot = run_gpu(ini, U0, 8)
    bscale = np.abs(U0[5:]).max() / p.dx
    assert tot[2] <= 1e-12 * bscale, (tot[2], bscale)


def _divb_inner(U, p, margin):
    """max |div B| of the cells at least `margin` cells inside the interior
    (face B at the left faces, U[5:8]; FP64 on the host)."""
    g = p.gw
    bx, by, bz = U[5], U[6], U[7]
    sl = slice(g + margin, -(g + margin))
    sp = slice(g + margin + 1, U.shape[1] - (g + margin) + 1)
    d = (np.abs((bx[sl, sl, sp] - bx[sl, sl, sl]) / p.dx + (by[sl, sp, sl] - by[sl, sl, sl]) / p.dy +
                (bz[sp, sl, sl] - bz[sl, sl, sl]) / p.dz))
    return float(d.max())


def test_mixed_precision_low_beta_blast_error_and_divb():
    # low-beta blast (beta ~ 0.025 outside the sphere: the total energy is
    # mostly magnetic, so the pressure recovered from it cancels; the mixed
    # form does that subtraction in FP64), with a small transverse field so
    # the reference's HLLD star state is defined; 30 steps as configured
    ini, U0 = P.mhd_blast_3d(n=48, nsteps=30, by_ratio=0.1)
    Ug, dg, _, tot = run_gpu(ini, U0, 30, precision=ek.EK_PREC_MIXED)
    U64, d64, _, tot64 = run_gpu(ini, U0, 30)
    p = eko.params_from_ini(ini)
    assert len(dg) == len(d64) == 30 and np.all(np.isfinite(Ug))
    err = rel_l1(interior(Ug, p.gw, 3), interior(U64, p.gw, 3))
    assert err[0] <= MIXED_L1_TOL and err[1] <= MIXED_L1_TOL, err
    assert np.abs(dg / d64 - 1).max() <= 1e-5
    # CT keeps div B at FP64 round-off wherever only CT updates the faces; the
    # blast reaches the outflow boundary in these 30 steps, where the face-B
    # boundary fill (BoundariesFunctors.h:814-831, face values copied like
    # cell values) makes div B non-zero in the reference's arithmetic too
    bscale = np.abs(U0[5:]).max() / p.dx
    for U in (Ug, U64):
        assert _divb_inner(U, p, 4) <= 1e-12 * bscale, (_divb_inner(U, p, 4), bscale)
    assert _divb_inner(U0, p, 0) <= 1e-12 * bscale


@pytest.mark.parametrize("n,kchunk,stage", [(64, 0, 0), (64, 6, 0), (68, 6, 0), (64, 0, 1)],
                         ids=["64", "64_kchunk6", "68_partial_tiles", "64_staged_trace"])
def test_mixed_hlld_repair_pass_low_beta_blast(n, kchunk, stage):
    # faces of the low-beta blast whose FP32 HLLD star-state denominator
    # rho (S - u)(S - u*) - Bn^2 cancels: the update kernel lists their tiles
    # and the repair kernel (one launch per step) recomputes them with those
    # faces in FP64.  kchunk 6: partial tile columns along z; 68^3: partial
    # tiles in x and y; stage: the update and repair kernels with the trace
    # planes staged in shared memory.
    ini, U0 = P.mhd_blast_3d(n=n, nsteps=30, by_ratio=0.1)
    p = ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED, kchunk=kchunk, mhd_stage=stage)
    with ek.Solver(p) as s:
        s.set_state(U0)
        s.set_profiling(True)
        assert s.run(30) == 30
        Ug, dg, repairs = s.get_state(), s.dt_history(), s.hlld_repairs()
        _, launches = s.kernel_time(3)
    U64, d64, _, _ = run_gpu(ini, U0, 30)
    q = eko.params_from_ini(ini)
    assert repairs > 0 and launches == 30, (repairs, launches)
    assert np.all(np.isfinite(Ug))
    err = rel_l1(interior(Ug, q.gw, 3), interior(U64, q.gw, 3))
    assert err[0] <= MIXED_L1_TOL and err[1] <= MIXED_L1_TOL, err
    assert np.abs(dg / d64 - 1).max() <= 1e-5


def test_repair_pass_only_for_mixed_hlld():
    # FP64, and the mixed form with another face solver, have no repair pass
    ini, U0 = P.orszag_tang_3d(n=16, nsteps=2)
    for over in ({}, {"precision": ek.EK_PREC_MIXED, "riemann": 2}):
        p = ek.params_from_ini(ini, **over)
        with ek.Solver(p) as s:
            s.set_state(U0)
            s.set_profiling(True)
            s.run(2)
            assert s.hlld_repairs() == 0
            assert s.kernel_time(3)[1] == 0

