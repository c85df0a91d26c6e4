"""GPU parity of static gravity (hydro, [gravity] enabled) through the C ABI.

The reference fixtures rt*/grav* (tests/golden) are checked by
test_gpu_hydro.py with every other hydro fixture (exact build bitwise, FMA
build within the FP64 tolerances).  Here: the oracle on larger and ragged
grids (partial tiles, z-chunks, ghost-cell gravity read by the predictor),
field and layout equivalences, the mixed form, and the API's refusals.
"""

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import interior, rel_l1

pytestmark = pytest.mark.gpu

MIXED_L1_TOL = 1e-5


def _field(shape, dim, seed):
    rng = np.random.default_rng(seed)
    k, j, i = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing="ij")
    G = np.empty((dim,) + shape)
    for c in range(dim):
        a = rng.uniform(0.2, 1.5, 4)
        G[c] = a[0] * np.sin(0.37 * i + a[1]) * np.cos(0.23 * j + a[2]) * np.cos(0.41 * k + a[3]) - 0.5
    return G


def run_gpu(ini, U0, nsteps, G=None, layout=ek.EK_LAYOUT_LEFT, **over):
    p = ek.params_from_ini(ini, **over)
    with ek.Solver(p) as s:
        s.set_state(U0)
        if G is not None:
            s.set_gravity_field(G, layout)
        assert s.run(nsteps) == nsteps
        return s.get_state(), s.dt_history(), s.m_t


def run_oracle(ini, U0, nsteps, G=None):
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0, gravity_field=G)
    dts = o.run(nsteps)
    return o.state(), dts, o.t, p


CASES = [
    # ragged 2D tiles, HLLC + predictor, a non-uniform field
    ("2d_ragged_field_hllc", lambda: P.rayleigh_taylor(dim=2, nx=37, ny=51, nsteps=10, riemann="hllc",
                                                       hancock=True, noise=0.02, g=-0.3), 10, True, {}),
    ("2d_uniform_approx", lambda: P.rayleigh_taylor(dim=2, nx=40, nsteps=15, noise=0.01), 15, False, {}),
    ("2d_field_hll_minmod", lambda: P.rayleigh_taylor(dim=2, nx=33, ny=29, nsteps=8, riemann="hll",
                                                      hancock=True, noise=0.03, slope_type=1.0), 8, True, {}),
    # 3D: several z-chunks with a short tail, partial tiles
    ("3d_ragged_field_hllc", lambda: P.rayleigh_taylor(dim=3, nx=19, ny=13, nz=37, nsteps=6, riemann="hllc",
                                                       hancock=True, noise=0.02, g=-0.3), 6, True, {"kchunk": 8}),
    ("3d_uniform_llf", lambda: P.rayleigh_taylor(dim=3, nx=12, nsteps=6, riemann="llf", hancock=True,
                                                 noise=0.01), 6, False, {"kchunk": 5}),
    ("3d_uniform_approx", lambda: P.rayleigh_taylor(dim=3, nx=10, ny=14, nz=30, nsteps=6, noise=0.01), 6,
     False, {}),
]


@pytest.mark.parametrize("label,build,nsteps,field,over", CASES, ids=[c[0] for c in CASES])
def test_exact_build_matches_oracle_bitwise(label, build, nsteps, field, over):
    ini, U0 = build()
    p = eko.params_from_ini(ini)
    G = _field(U0.shape[1:], p.dim, 7) if field else None
    Ug, dg, tg = run_gpu(ini, U0, nsteps, G=G, exact_fp=1, **over)
    Uo, do, to, p = run_oracle(ini, U0, nsteps, G=G)
    assert np.array_equal(dg, do)
    assert np.array_equal(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
    assert tg == to


@pytest.mark.parametrize("dim", [2, 3])
def test_uniform_field_equals_uniform_parameters_and_layouts(dim):
    ini, U0 = P.rayleigh_taylor(dim=dim, nx=20 if dim == 2 else 8, nsteps=6, riemann="hllc", hancock=True,
                                noise=0.02)
    p = eko.params_from_ini(ini)
    Ua, da, _ = run_gpu(ini, U0, 6, exact_fp=1)
    G = np.empty((dim,) + U0.shape[1:])
    for c in range(dim):
        G[c] = p.gravity[c]
    Ub, db, _ = run_gpu(ini, U0, 6, G=G, exact_fp=1)
    assert np.array_equal(da, db) and np.array_equal(Ua, Ub)
    # a non-uniform field in LayoutRight equals the same field in LayoutLeft
    F = _field(U0.shape[1:], dim, 11)
    Uc, dc, _ = run_gpu(ini, U0, 6, G=F, exact_fp=1)
    Ud, dd, _ = run_gpu(ini, U0, 6, G=np.ascontiguousarray(np.transpose(F, (3, 2, 1, 0))),
                        layout=ek.EK_LAYOUT_RIGHT, exact_fp=1)
    assert np.array_equal(dc, dd) and np.array_equal(Uc, Ud)
    assert not np.array_equal(Uc, Ua)


def test_field_reset_and_mid_run_change_match_oracle():
    ini, U0 = P.rayleigh_taylor(dim=2, nx=24, nsteps=10, riemann="hllc", hancock=True, noise=0.02)
    p = eko.params_from_ini(ini)
    F = _field(U0.shape[1:], 2, 5)
    pe = ek.params_from_ini(ini, exact_fp=1)
    with ek.Solver(pe) as s:
        s.set_state(U0)
        s.set_gravity_field(F)
        s.set_gravity_field(None)  # back to the uniform field
        s.run(4)
        dt_uniform = s.dt_history()
        s.set_gravity_field(F)  # the next steps use the field (dt recomputed)
        s.run(4)
        Ug, dg = s.get_state(), s.dt_history()
    o = eko.Oracle(p, U0)
    do = list(o.run(4))
    eko.lib().eko_set_gravity_field(o._h, np.ascontiguousarray(F).ctypes.data)
    do += list(o.run(4))
    assert np.array_equal(dt_uniform, do[:4])
    assert np.array_equal(dg, np.array(do))
    assert np.array_equal(interior(Ug, 2, 2), interior(o.state(), 2, 2))


@pytest.mark.parametrize("dim", [2, 3])
def test_mixed_precision_error_bound(dim):
    ini, U0 = P.rayleigh_taylor(dim=dim, nx=64 if dim == 2 else 16, nsteps=20, riemann="hllc", hancock=True,
                                noise=0.02, g=-0.3)
    p = eko.params_from_ini(ini)
    G = _field(U0.shape[1:], dim, 3)
    Ug, dg, _ = run_gpu(ini, U0, 20, G=G, precision=ek.EK_PREC_MIXED)
    Uo, do, _, p = run_oracle(ini, U0, 20, G=G)
    err = rel_l1(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
    assert err[0] <= MIXED_L1_TOL and err[1] <= MIXED_L1_TOL, err
    assert np.max(np.abs(dg - do) / do) < 1e-5


def test_mhd_ignores_gravity_and_refusals():
    # SolverMHDMuscl has no gravity terms: [gravity] enabled changes nothing
    ini, U0 = P.orszag_tang_3d(n=12, nsteps=3)
    ini_g = ini + "\n[gravity]\nenabled=yes\nhancock_predictor_enabled=yes\n"
    Ua, da, _ = run_gpu(ini, U0, 3, exact_fp=1)
    Ub, db, _ = run_gpu(ini_g, U0, 3, exact_fp=1)
    assert np.array_equal(Ua, Ub) and np.array_equal(da, db)
    p = ek.params_from_ini(ini_g)
    with ek.Solver(p) as s:
        with pytest.raises(ek.EkError):
            s.set_gravity_field(np.zeros((3,) + U0.shape[1:]))
    # hydro without gravity: no field to set
    ini2, U2 = P.implode_2d(n=16, nsteps=2)
    with ek.Solver(ek.params_from_ini(ini2)) as s:
        s.set_state(U2)
        with pytest.raises(ek.EkError):
            s.set_gravity_field(np.zeros((2,) + U2.shape[1:]))
    # ensembles run without gravity
    ini3, _ = P.rayleigh_taylor(dim=2, nx=16, nsteps=2, riemann="hllc")
    with pytest.raises(ek.EkError):
        ek.Ensemble([ek.params_from_ini(ini3)])


def test_gravity_with_tensor_copy_staging_matches_oracle():
    # a grid with tiles whose halo is interior (tensor-copy staged planes)
    ini, U0 = P.rayleigh_taylor(dim=3, nx=40, ny=40, nz=48, nsteps=4, riemann="hllc", hancock=True, noise=0.02)
    p = eko.params_from_ini(ini)
    G = _field(U0.shape[1:], 3, 13)
    Ug, dg, tg = run_gpu(ini, U0, 4, G=G, exact_fp=1, kchunk=12)
    Uo, do, to, p = run_oracle(ini, U0, 4, G=G)
    assert np.array_equal(dg, do)
    assert np.array_equal(interior(Ug, p.gw, p.dim), interior(Uo, p.gw, p.dim))
