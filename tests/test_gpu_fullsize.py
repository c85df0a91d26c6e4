"""Parity at the configured workloads' full sizes.

* 2D implode 256^2, 100 steps, FP64: the exact build equals the oracle bit for
  bit (state and dt sequence); the FMA build is within the drop-in tolerances
  (dt 1e-13, fields 1e-11 relative L-infinity).
* FP64 drop-in against the oracle (the reference algorithm's CPU restatement,
  OpenMP on the host cores) from the same injected state, at the 3D configs'
  full sizes: the exact build equals the oracle bit for bit after 5 steps
  (16-plane z-chunk seams through the whole depth); the FMA build's dt
  sequence is within 1e-13 relative and density and energy within 1e-11
  relative L-infinity after the run; for MHD the magnetic field within 1e-11
  of its own scale (max |B - B_ref| over the components / max |B_ref|):
  - 3D blast 256^3, 50 steps;
  - 3D MHD Orszag-Tang 256^3, OT_STEPS steps (the config's 100 by default;
    EK_FULLSIZE_OT_STEPS lowers it where the host cores are slow: the oracle
    runs this case at a few Mcell-updates/s).
* 3D blast 256^3, 50 steps: the mixed form is within 1e-5 relative L1 of the
  FP64 drop-in in density and energy; mass is conserved in both forms while
  the blast is inside the box (outflow boundaries, nothing has left).
* 3D MHD Orszag-Tang 256^3, 100 steps: mixed within 1e-5 relative L1 of FP64;
  periodic box: mass and total energy conserved, max |div B| at FP64
  round-off in both forms.
* 512-instance Kelvin-Helmholtz ensemble, 200 steps: sampled instances equal
  their single-solver runs bit for bit (state and dt sequence).
* 3D MHD low-beta blast 512^3 (transverse field), 30 steps: the mixed form
  stays within 1e-5 L1 of FP64 in density and energy and its dt sequence
  within 1e-5.  At this size the FP32 HLLD meets near-degenerate star states
  (|estar| << Bn^2): the repair kernel recomputes their tiles with those faces
  in FP64, and the test checks that it did.
"""

import os

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import interior, rel_l1, rel_linf

pytestmark = pytest.mark.gpu

OT_STEPS = int(os.environ.get("EK_FULLSIZE_OT_STEPS", "100"))
EXACT_STEPS = 5
FP64_DT_TOL, FP64_FIELD_TOL = 1e-13, 1e-11


def _oracle_snapshots(ini, U0, nsteps):
    """Oracle state and dt sequence after EXACT_STEPS and after nsteps steps."""
    o = eko.Oracle(eko.params_from_ini(ini), U0)
    try:
        d5 = o.run(EXACT_STEPS)
        U5 = o.state()
        dn = o.run(nsteps - EXACT_STEPS)
        return {"U5": U5, "dts5": np.asarray(d5), "U": o.state(),
                "dts": np.concatenate([np.asarray(d5), np.asarray(dn)])}
    finally:
        o.close()


@pytest.fixture(scope="module")
def blast_256():
    ini, U0 = P.blast_3d(n=256, nsteps=50)
    return ini, U0, _oracle_snapshots(ini, U0, 50)


@pytest.fixture(scope="module")
def orszag_tang_256():
    ini, U0 = P.orszag_tang_3d(n=256, nsteps=OT_STEPS)
    return ini, U0, _oracle_snapshots(ini, U0, OT_STEPS)


def _check_fp64_drop_in(ini, U0, ref, nsteps, gw, nvar_checked):
    # exact build: bitwise after EXACT_STEPS steps
    Ue, de, _, _, n = _run(ini, U0, EXACT_STEPS, exact_fp=1)
    assert n == EXACT_STEPS
    assert np.array_equal(de, ref["dts5"])
    assert np.array_equal(interior(Ue, gw, 3), interior(ref["U5"], gw, 3))
    del Ue
    # FMA build: the drop-in tolerances after the whole run
    Uf, df, _, _, n = _run(ini, U0, nsteps)
    assert n == nsteps
    dt_err = np.abs(df / ref["dts"] - 1).max()
    assert dt_err <= FP64_DT_TOL, dt_err
    a, b = interior(Uf, gw, 3), interior(ref["U"], gw, 3)
    err = rel_linf(a, b)
    print("fp64 vs oracle: %d steps, dt rel err %.3g, rel Linf per variable %s" % (nsteps, dt_err, err))
    # density (0) and energy (1) against their own scale
    assert err[[0, 1]].max() <= FP64_FIELD_TOL, err
    if nvar_checked > 5:
        # the magnetic field as a vector: max |B - B_ref| over the components
        # against max |B_ref| (a component that stays near zero, such as Bz of
        # Orszag-Tang, would otherwise be measured against its own tiny scale)
        bscale = max(float(np.abs(b[c]).max()) for c in range(5, 8))
        berr = max(float(np.abs(a[c] - b[c]).max()) for c in range(5, 8)) / bscale
        print("fp64 vs oracle: max |B - B_ref| / max |B_ref| = %.3g" % berr)
        assert berr <= FP64_FIELD_TOL, (berr, err)


def _run(ini, U0, nsteps, **over):
    p = ek.params_from_ini(ini, **over)
    with ek.Solver(p) as s:
        s.set_state(U0)
        tot0 = s.totals()
        done = s.run(nsteps)
        return s.get_state(), s.dt_history(), tot0, s.totals(), done


def test_implode_256_fp64_matches_oracle():
    ini, U0 = P.implode_2d(n=256, nsteps=100)
    Ue, de, _, _, n = _run(ini, U0, 100, exact_fp=1)
    assert n == 100
    o = eko.Oracle(eko.params_from_ini(ini), U0)
    do = o.run(100)
    Uo = o.state()
    o.close()
    assert np.array_equal(de, do)
    assert np.array_equal(interior(Ue, 2, 2), interior(Uo, 2, 2))
    Uf, df, _, _, _ = _run(ini, U0, 100)
    assert np.abs(df / do - 1).max() <= 1e-13
    assert rel_linf(interior(Uf, 2, 2), interior(Uo, 2, 2)).max() <= 1e-11


def test_blast_256_fp64_matches_oracle(blast_256):
    ini, U0, ref = blast_256
    _check_fp64_drop_in(ini, U0, ref, 50, 2, 5)


def test_orszag_tang_256_fp64_matches_oracle(orszag_tang_256):
    ini, U0, ref = orszag_tang_256
    _check_fp64_drop_in(ini, U0, ref, OT_STEPS, 3, 8)


def test_blast_256_mixed_vs_fp64():
    ini, U0 = P.blast_3d(n=256, nsteps=50)
    Um, dm, t0m, t1m, n = _run(ini, U0, 50, precision=ek.EK_PREC_MIXED)
    U64, d64, t064, t164, _ = _run(ini, U0, 50)
    assert n == 50
    err = rel_l1(interior(Um, 2, 3), interior(U64, 2, 3))
    assert err[0] <= 1e-5 and err[1] <= 1e-5, err
    assert np.abs(dm / d64 - 1).max() <= 1e-5
    # FP64 totals of each form: mass conserved (to the form's rounding)
    assert abs(t164[0] / t064[0] - 1) <= 1e-12
    assert abs(t1m[0] / t0m[0] - 1) <= 1e-6


def test_orszag_tang_256_mixed_vs_fp64_conservation_divb():
    ini, U0 = P.orszag_tang_3d(n=256, nsteps=100)
    p = eko.params_from_ini(ini)
    Um, dm, t0m, t1m, n = _run(ini, U0, 100, precision=ek.EK_PREC_MIXED)
    U64, d64, t064, t164, _ = _run(ini, U0, 100)
    assert n == 100
    err = rel_l1(interior(Um, 3, 3), interior(U64, 3, 3))
    assert err[0] <= 1e-5 and err[1] <= 1e-5, err
    assert np.abs(dm / d64 - 1).max() <= 1e-5
    for a, b, tol in ((t064, t164, 1e-11), (t0m, t1m, 1e-6)):
        assert abs(b[0] / a[0] - 1) <= tol and abs(b[1] / a[1] - 1) <= tol, (a, b)
    bscale = np.abs(U0[5:]).max() / p.dx
    assert t1m[2] <= 1e-12 * bscale and t164[2] <= 1e-12 * bscale, (t1m[2], t164[2], bscale)


def test_kh_ensemble_512_matches_single_solvers():
    cases = P.kh_ensemble(n_inst=512, nsteps=10 ** 6)
    params = [ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED) for ini, _ in cases]
    with ek.Ensemble(params) as e:
        for i, (_, U0) in enumerate(cases):
            e.set_state(i, U0)
        e.run(200)
        e.synchronize()
        for i in (0, 1, 255, 510, 511):
            with ek.Solver(params[i]) as s:
                s.set_state(cases[i][1])
                s.run(200)
                assert np.array_equal(e.dt_history(i), s.dt_history()), i
                assert np.array_equal(e.get_state(i), s.get_state()), i


def test_mhd_blast_lowbeta_512_mixed_vs_fp64():
    ini, U0 = P.mhd_blast_3d(n=512, nsteps=30, by_ratio=0.1)
    out = {}
    for name, over in (("mixed", dict(precision=ek.EK_PREC_MIXED)), ("fp64", {})):
        p = ek.params_from_ini(ini, **over)
        with ek.Solver(p) as s:
            s.set_state(U0)
            n = s.run(30, allow_nonfinite=True)
            assert n == 30
            out[name] = (s.get_state()[:2, 3:-3, 3:-3, 3:-3].copy(), s.dt_history())
            if name == "mixed":
                repairs = s.hlld_repairs()
    del U0
    (am, dm), (af, df) = out["mixed"], out["fp64"]
    assert np.abs(dm / df - 1).max() <= 1e-5, np.abs(dm / df - 1).max()
    err = rel_l1(am, af)
    print("low-beta blast 512^3, 30 steps: L1 rho %.3g E %.3g, max dt diff %.3g, tiles repaired %d" %
          (err[0], err[1], np.abs(dm / df - 1).max(), repairs))
    # the FP32 star states of this case are ill-conditioned on some faces:
    # the repair pass must have run
    assert repairs > 0
    assert err[0] <= 1e-5 and err[1] <= 1e-5, err
