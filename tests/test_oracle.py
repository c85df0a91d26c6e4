"""The oracle (C restatement, oracle/ek_oracle.c) against the reference.

The golden fixtures in tests/golden were produced by the reference's OWN
solver sources (compiled unmodified against a Kokkos-API shim, see
tests/golden/make_golden.py).  The restatement must reproduce them bit for bit:
final state, dt sequence and final time -- including the NaN pattern of the
MHD blast case, where the reference's HLLD degenerate-state test divides 0/0.
"""

import numpy as np
import pytest

import eko
from helpers import golden_cases, interior, load_golden


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_bitwise(name):
    g = load_golden(name)
    p = eko.params_from_ini(str(g["ini"]))
    o = eko.Oracle(p, g["U0"], gravity_field=g.get("G"))
    dts = o.run(len(g["dts"]))
    assert np.array_equal(dts, g["dts"], equal_nan=True)
    U = o.state()
    a, b = interior(U, p.gw, p.dim), interior(g["U"], p.gw, p.dim)
    assert np.array_equal(a, b, equal_nan=True)
    assert o.iteration == int(g["iteration"])
    assert np.array_equal(np.array(o.t), g["t"], equal_nan=True)


def test_oracle_conserves_mass_periodic():
    # periodic boundaries: total mass is conserved to round-off
    from euler_kokkos_gb300 import problems as P

    ini, U0 = P.smooth_random(dim=3, nx=12, ny=10, nz=8, seed=11, bc=(3,) * 6, nsteps=5)
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    m0 = interior(U0, p.gw, p.dim)[0].sum()
    o.run(5)
    m1 = interior(o.state(), p.gw, p.dim)[0].sum()
    assert abs(m1 - m0) / m0 < 1e-13


def test_oracle_implode_symmetry():
    # the implode problem is symmetric about the diagonal x = y
    from euler_kokkos_gb300 import problems as P

    ini, U0 = P.implode_2d(n=24, nsteps=10)
    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    o.run(10)
    rho = interior(o.state(), p.gw, p.dim)[0, 0]
    assert np.allclose(rho, rho.T, rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", golden_cases(bitwise=False))
def test_oracle_matches_atomic_update_versions_to_roundoff(name):
    # fixtures written by the reference's hydro implementationVersion 2, which
    # adds the face fluxes with atomics: version 0's arithmetic (the oracle)
    # equals them up to the summation order
    g = load_golden(name)
    p = eko.params_from_ini(str(g["ini"]))
    o = eko.Oracle(p, g["U0"])
    dts = o.run(len(g["dts"]))
    assert np.max(np.abs(dts - g["dts"]) / g["dts"]) <= 1e-13
    a, b = interior(o.state(), p.gw, p.dim), interior(g["U"], p.gw, p.dim)
    scale = np.abs(b).reshape(b.shape[0], -1).max(axis=1)
    err = np.abs(a - b).reshape(b.shape[0], -1).max(axis=1) / np.where(scale > 0, scale, 1)
    assert np.all(err <= 1e-13), err
