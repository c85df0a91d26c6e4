"""GPU parity of the fused hydro step (2D and 3D) through the C ABI.

* exact build (FP64, no FMA contraction): the whole run is bit-identical to
  the reference (golden fixtures) and to the oracle on seeded inputs, dt
  sequence included;
* fast build (FP64 with FMA contraction): within 1e-11 relative L-infinity of
  density/energy after the run, dt within 1e-13 relative;
* mixed form (FP32 with FP64 islands): within 1e-5 relative L1 in density.
"""

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import golden_cases, interior, load_golden, rel_l1, rel_linf

pytestmark = pytest.mark.gpu

FP64_LINF_TOL = 1e-11  # density/energy after the run, FMA build vs reference
DT_REL_TOL = 1e-13
MIXED_L1_TOL = 1e-5


def run_gpu(ini, U0, nsteps, G=None, **over):
    p = ek.params_from_ini(ini, **over)
    with ek.SolverFactory.create(p.solver_name, p) as s:
        s.set_state(U0)
        if G is not None:
            s.set_gravity_field(G)
        done = s.run(nsteps)
        assert done == nsteps
        return s.get_state(), s.dt_history(), s.m_t, s.m_iteration


def run_oracle(ini, U0, nsteps):
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    dts = o.run(nsteps)
    return o.state(), dts, o.t, p


@pytest.mark.parametrize("name", golden_cases("hydro"))
def test_exact_build_matches_reference_golden_bitwise(name):
    g = load_golden(name)
    ini = str(g["ini"])
    U, dts, t, it = run_gpu(ini, g["U0"], len(g["dts"]), G=g.get("G"), exact_fp=1)
    p = eko.params_from_ini(ini)
    assert np.array_equal(dts, g["dts"])
    assert np.array_equal(interior(U, p.gw, p.dim), interior(g["U"], p.gw, p.dim))
    assert t == float(g["t"]) and it == int(g["iteration"])


@pytest.mark.parametrize("name", golden_cases("hydro"))
def test_fma_build_matches_reference_golden(name):
    g = load_golden(name)
    ini = str(g["ini"])
    U, dts, t, it = run_gpu(ini, g["U0"], len(g["dts"]), G=g.get("G"))
    p = eko.params_from_ini(ini)
    err = rel_linf(interior(U, p.gw, p.dim), interior(g["U"], p.gw, p.dim))
    assert err[0] <= FP64_LINF_TOL and err[1] <= FP64_LINF_TOL, err
    assert np.max(np.abs(dts - g["dts"]) / g["dts"]) <= DT_REL_TOL


CASES = [
    # odd sizes: partial tiles in x/y, several z-chunks with a short tail
    ("2d_odd_reflect", lambda: P.smooth_random(dim=2, nx=37, ny=23, seed=21, bc=(1, 1, 1, 1, 1, 1),
                                               slope_type=1.0, nsteps=12), 12, {}),
    ("2d_periodic_outflow", lambda: P.smooth_random(dim=2, nx=64, ny=9, seed=22, bc=(3, 3, 2, 2, 1, 1),
                                                    slope_type=2.0, nsteps=9), 9, {}),
    ("3d_odd_mixed", lambda: P.smooth_random(dim=3, nx=35, ny=17, nz=41, seed=23, bc=(1, 2, 3, 3, 2, 1),
                                             slope_type=2.0, nsteps=6), 6, {"kchunk": 16}),
    ("3d_thin", lambda: P.smooth_random(dim=3, nx=8, ny=40, nz=3, seed=24, bc=(3, 3, 1, 1, 3, 3),
                                        slope_type=1.0, nsteps=5), 5, {"kchunk": 2}),
    ("3d_blast", lambda: P.blast_3d(n=24, nsteps=8), 8, {"kchunk": 7}),
]


@pytest.mark.parametrize("label,build,nsteps,over", CASES, ids=[c[0] for c in CASES])
def test_exact_build_matches_oracle_bitwise(label, build, nsteps, over):
    ini, U0 = build()
    Ug, dg, tg, _ = run_gpu(ini, U0, nsteps, exact_fp=1, **over)
    Uo, do, to, p = run_oracle(ini, U0, nsteps)
    assert np.array_equal(dg, do)
    assert np.array_equal(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
    assert tg == to


def test_next_iteration_api_matches_run_and_reference_loop():
    ini, U0 = P.implode_2d(n=40, nsteps=7)
    p = ek.params_from_ini(ini, exact_fp=1)
    with ek.Solver(p) as s:
        s.set_state(U0)
        dt0 = s.compute_dt()
        steps = 0
        while not s.finished():  # main.cpp:126-131
            s.next_iteration()
            steps += 1
        assert steps == 7 and s.m_iteration == 7
        U1 = s.get_state()
        h = s.dt_history()
    assert h[0] == dt0
    U2, d2, _, _ = run_gpu(ini, U0, 7, exact_fp=1)
    assert np.array_equal(interior(U1, 2, 2), interior(U2, 2, 2)) and np.array_equal(h, d2)


def test_tend_clamps_last_step_like_reference():
    ini, U0 = P.implode_2d(n=32, nsteps=1000)
    ini = ini.replace("tEnd=1e30", "tEnd=0.01")
    p = ek.params_from_ini(ini, exact_fp=1)
    with ek.Solver(p) as s:
        s.set_state(U0)
        n = s.run(1000)
        U = s.get_state()
        dts = s.dt_history()
        t = s.m_t
        assert s.finished()
    Uo, do, to, pp = run_oracle(ini, U0, 1000)
    assert n == len(do)
    assert np.array_equal(dts, do) and t == to
    assert np.array_equal(interior(U, 2, 2), interior(Uo, 2, 2))


def test_layout_right_round_trip_and_ghosts():
    ini, U0 = P.smooth_random(dim=3, nx=10, ny=7, nz=5, seed=31, bc=(1, 2, 3, 3, 1, 2), nsteps=1)
    p = ek.params_from_ini(ini)
    with ek.Solver(p) as s:
        # LayoutRight input (var fastest, as the OpenMP build's host arrays)
        UR = np.ascontiguousarray(np.transpose(U0, (3, 2, 1, 0)))
        s.set_state(UR, layout=ek.EK_LAYOUT_RIGHT)
        UL = s.get_state()
        assert np.array_equal(interior(UL, 2, 3), interior(U0, 2, 3))
        back = s.get_state(layout=ek.EK_LAYOUT_RIGHT)
        assert np.array_equal(np.transpose(back, (3, 2, 1, 0)), UL)
    # ghosts returned by get_state follow make_boundaries (oracle fills them the reference way)
    o = eko.Oracle(eko.params_from_ini(ini), U0)
    Uo = o.state()
    assert np.array_equal(UL, Uo)


def test_mixed_precision_blast_error_bound():
    ini, U0 = P.blast_3d(n=48, nsteps=10)
    Ug, dg, _, _ = run_gpu(ini, U0, 10, precision=ek.EK_PREC_MIXED)
    Uo, do, _, p = run_oracle(ini, U0, 10)
    err = rel_l1(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
    assert err[0] <= MIXED_L1_TOL, err
    assert np.max(np.abs(dg - do) / do) < 1e-4


def test_mixed_precision_implode_error_bound():
    ini, U0 = P.implode_2d(n=64, nsteps=30)
    Ug, _, _, _ = run_gpu(ini, U0, 30, precision=ek.EK_PREC_MIXED)
    Uo, _, _, p = run_oracle(ini, U0, 30)
    err = rel_l1(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
    assert err[0] <= MIXED_L1_TOL, err


def test_totals_are_fp64_and_conserved_periodic():
    ini, U0 = P.smooth_random(dim=3, nx=32, ny=24, nz=16, seed=41, bc=(3,) * 6, nsteps=20)
    for prec in (ek.EK_PREC_FP64, ek.EK_PREC_MIXED):
        p = ek.params_from_ini(ini, precision=prec)
        with ek.Solver(p) as s:
            s.set_state(U0)
            m0 = s.totals()[0]
            s.run(20)
            m1 = s.totals()[0]
        assert abs(m1 - m0) / m0 < (1e-13 if prec == 0 else 1e-6)


@pytest.mark.parametrize("prec", [ek.EK_PREC_FP64, ek.EK_PREC_MIXED])
def test_state_transfer_layouts_and_precisions(prec):
    # set_state/get_state convert and transpose on the device (staging chunks)
    cases = [P.smooth_random(dim=3, nx=10, ny=7, nz=5, seed=32, bc=(1, 2, 3, 3, 1, 2), nsteps=1),
             P.smooth_random(dim=3, mhd=True, nx=9, ny=6, nz=5, seed=33, bc=(3,) * 6, nsteps=1),
             P.smooth_random(dim=2, nx=13, ny=11, seed=34, bc=(3, 3, 2, 2, 1, 1), nsteps=1)]
    for ini, U0 in cases:
        p = ek.params_from_ini(ini, precision=prec)
        o = eko.Oracle(eko.params_from_ini(ini), U0)
        want = o.state()  # ghosts filled the reference way
        if prec == ek.EK_PREC_MIXED:
            nh = 5 if p.mhd else p.nbvar  # FP32 hydro planes, FP64 face B
            want = want.copy()
            want[:nh] = want[:nh].astype(np.float32).astype(np.float64)
        with ek.Solver(p) as s:
            s.set_state(np.ascontiguousarray(np.transpose(U0, (3, 2, 1, 0))), layout=ek.EK_LAYOUT_RIGHT)
            UL = s.get_state()
            UR = s.get_state(layout=ek.EK_LAYOUT_RIGHT)
            s.set_state(U0)
            UL2 = s.get_state(out=np.empty_like(U0))
        assert np.array_equal(UL, want)
        assert np.array_equal(np.transpose(UR, (3, 2, 1, 0)), want)
        assert np.array_equal(UL2, want)


def test_state_transfer_in_several_chunks():
    # 45.8 M values: more than one 32 Mi-value staging chunk
    n = 200
    ini, _ = P.blast_3d(n=8, nsteps=1)
    ini = ini.replace("nx=8", "nx=%d" % (n + 8)).replace("ny=8", "ny=%d" % (n + 8)).replace("nz=8", "nz=%d" % n)
    p = ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED)
    shp = p.shape
    rng = np.random.default_rng(5)
    U0 = np.empty(shp)
    U0[0] = 1.0 + 0.1 * rng.random(shp[1:])
    U0[1] = 2.0 + 0.1 * rng.random(shp[1:])
    U0[2:] = 0.01 * rng.standard_normal((3,) + shp[1:])
    with ek.Solver(p) as s:
        s.set_state(np.ascontiguousarray(np.transpose(U0, (3, 2, 1, 0))), layout=ek.EK_LAYOUT_RIGHT)
        got = s.get_state(layout=ek.EK_LAYOUT_RIGHT)
    gw = p.ghost_width
    a = np.transpose(got, (3, 2, 1, 0))[:, gw:-gw, gw:-gw, gw:-gw]
    assert np.array_equal(a, U0[:, gw:-gw, gw:-gw, gw:-gw].astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("prec", [ek.EK_PREC_FP64, ek.EK_PREC_MIXED])
def test_tensor_copy_staging_matches_plain_loads(prec):
    # interior planes staged by tensor copies (isize % 4 == 0, tiles whose halo
    # is interior) give the same bits as the plain boundary-mapped loads
    ini, U0 = P.smooth_random(dim=3, nx=68, ny=52, nz=21, seed=51, bc=(1, 2, 3, 3, 2, 1), slope_type=2.0,
                              nsteps=6)
    out = []
    for no_tma in (0, 1):
        U, d, _, _ = run_gpu(ini, U0, 6, precision=prec, no_tma=no_tma, kchunk=8)
        out.append((U, d))
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][0], out[1][0])


def test_tensor_copy_staging_exact_matches_oracle():
    ini, U0 = P.blast_3d(n=64, nsteps=5)
    Ug, dg, tg, _ = run_gpu(ini, U0, 5, exact_fp=1, kchunk=16)
    Uo, do, to, p = run_oracle(ini, U0, 5)
    assert np.array_equal(dg, do)
    assert np.array_equal(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))


@pytest.mark.parametrize("name", golden_cases("hydro", bitwise=False))
def test_atomic_update_version_fixtures_to_roundoff(name):
    # decks run by the reference at implementationVersion 2 (face fluxes added
    # with atomics): the fused version-0 step equals them up to the summation order
    g = load_golden(name)
    ini = str(g["ini"])
    p = eko.params_from_ini(ini)
    assert ek.params_from_ini(ini).implementation_version == 2
    U, dts, t, it = run_gpu(ini, g["U0"], len(g["dts"]), exact_fp=1)
    assert np.max(np.abs(dts - g["dts"]) / g["dts"]) <= 1e-13
    err = rel_linf(interior(U, p.gw, p.dim), interior(g["U"], p.gw, p.dim))
    assert np.all(err <= 1e-13), err
