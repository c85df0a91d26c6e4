"""CPU tests of the drop-in boundary: the .ini front end and the C ABI
surface of libek_gb300.so (no GPU needed)."""

import ctypes
import os
import re

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DECK = """
# a deck written the way the reference's settings/*.ini are
[run]
solver_name=Hydro_Muscl_3D
tEnd=0.25
nStepmax=37
nOutput=0
nlog = 5   ; trailing comment
[MESH]
nx=17
ny=9
nz=5
xmin=0.0
xmax=2.0
ymin=-0.5
ymax=0.5
zmin=0.
zmax=0.3
boundary_type_xmin=1
boundary_type_xmax=2
boundary_type_ymin=3
boundary_type_ymax=3
boundary_type_zmin=2
boundary_type_zmax=1

[hydro]
gamma0=1.666
cfl=0.45
riemann=hllc
slope_type=2
problem=blast
smallr=1e-7
[other]
implementationVersion=0
"""


def _fields(p):
    return dict(dim=p.dim, mhd=int(p.mhd), nx=p.nx, ny=p.ny, nz=p.nz, nbvar=p.nbvar,
                isize=p.isize, jsize=p.jsize, ksize=p.ksize, dx=p.dx, dy=p.dy, dz=p.dz,
                gamma0=p.gamma0, cfl=p.cfl, slope_type=p.slope_type, smallr=p.smallr,
                smallc=p.smallc, smallp=p.smallp, smallpp=p.smallpp, tEnd=p.tEnd,
                nStepmax=p.nStepmax, riemann=p.riemann, bc=list(p.bc)[:6])


@pytest.mark.parametrize("deck", [DECK, P.blast_3d(n=8, nsteps=3)[0], P.implode_2d(n=8)[0],
                                  P.orszag_tang_3d(n=6)[0], P.kelvin_helmholtz_2d(n=8)[0]])
def test_ini_front_end_matches_oracle_restatement(deck):
    a = ek.params_from_ini(deck)
    b = eko.params_from_ini(deck)
    fa, fb = _fields(a), _fields(b)
    for k in fa:
        assert fa[k] == fb[k], k


def test_reals_are_rounded_through_float():
    p = ek.params_from_ini(DECK)
    # cfl=0.45 is read by strtof: the double is the float nearest 0.45
    assert p.cfl == float(np.float32(0.45)) and p.cfl != 0.45
    assert p.gamma0 == float(np.float32(1.666))
    assert p.smallc == float(np.float32(1e-10))
    assert p.tEnd == float(np.float32(0.25))
    assert p.isize == 17 + 4 and p.ksize == 5 + 4
    assert p.dx == float(np.float32(2.0)) / 17


def test_gb300_section_and_defaults():
    p = ek.params_from_ini(DECK + "\n[gb300]\nprecision=mixed\nkchunk=16\n")
    assert p.precision == ek.EK_PREC_MIXED and p.kchunk == 16
    q = ek.params_from_ini(DECK)
    assert q.precision == ek.EK_PREC_FP64 and q.exact_fp == 0


def test_unknown_solver_is_an_error_not_an_abort():
    with pytest.raises(ek.EkError) as e:
        ek.params_from_ini("[run]\nsolver_name=Nope\n")
    assert e.value.status == 1
    with pytest.raises(ek.EkError) as e:
        ek.SolverFactory.create("Nope", ek.params_from_ini(DECK))
    assert e.value.status == 1


def test_parse_error_reported():
    with pytest.raises(ek.EkError) as e:
        ek.params_from_ini("[run\nsolver_name=Hydro_Muscl_2D\n")
    assert e.value.status == 6


def test_library_exports_every_declared_symbol():
    header = open(os.path.join(ROOT, "include", "ek_gb300.h")).read()
    names = set(re.findall(r"\b(ek_[a-z_0-9]+)\s*\(", header))
    assert len(names) >= 18
    L = ek.load_library()
    for n in sorted(names):
        assert hasattr(L, n), n
    assert L.ek_abi_version() == 1


def test_status_strings():
    L = ek.load_library()
    for s in range(8):
        assert L.ek_status_string(s)


@pytest.mark.skipif(__import__("conftest").gpu_available(), reason="checks the no-GPU path")
def test_create_without_gpu_fails_cleanly():
    with pytest.raises(ek.EkError) as e:
        ek.Solver(ek.params_from_ini(DECK))
    assert e.value.status == 7


def test_create_rejects_unsupported_configurations():
    # validation happens before any device call
    p = ek.params_from_ini(DECK)
    for bad in (dict(riemann=4), dict(riemann=7), dict(slope_type=3.0), dict(slope_type=1.5),
                dict(slope_type=-1.0), dict(implementation_version=3),
                dict(nx=1, isize=5), dict(exact_fp=1, precision=1)):
        with pytest.raises(ek.EkError) as e:
            ek.Solver(p.copy(**bad))
        assert e.value.status in (1, 2), bad
    # the MHD implementationVersions 1 and 2 compute another scheme in the reference
    from euler_kokkos_gb300 import problems as P

    for dim, v in ((3, 2), (3, 1), (2, 2), (2, 1)):
        ini = (P.orszag_tang_3d(n=8, nsteps=1) if dim == 3 else P.orszag_tang_2d(n=8, nsteps=1))[0]
        q = ek.params_from_ini(ini.replace("implementationVersion=0", "implementationVersion=%d" % v))
        assert q.implementation_version == v
        with pytest.raises(ek.EkError) as e:
            ek.Solver(q)
        assert e.value.status == 2, (dim, v)
    # the MHD slope routines have no slope_type 0 branch (MHDBaseFunctor3D.h:379)
    for ini in (P.orszag_tang_3d(n=8, nsteps=1)[0], P.orszag_tang_2d(n=8, nsteps=1)[0]):
        with pytest.raises(ek.EkError) as e:
            ek.Solver(ek.params_from_ini(ini).copy(slope_type=0.0))
        assert e.value.status == 2


def test_gravity_sections_parse_like_reference():
    # [gravity] (GravityParams.h:32-37) and the Rayleigh-Taylor field
    # (RayleighTaylorInstabilityParams.h:28-34), against the oracle's front end
    from euler_kokkos_gb300 import problems as P

    for dim, hancock in ((2, False), (3, True)):
        ini, _ = P.rayleigh_taylor(dim=dim, nx=8, nsteps=2, hancock=hancock, g=-0.3)
        p = ek.params_from_ini(ini)
        o = eko.params_from_ini(ini)
        assert p.gravity_enabled == 1 and p.gravity_static == 1 and p.gravity_hancock == int(hancock)
        assert p.gravity_well_balanced == 0
        assert list(p.gravity) == list(o.gravity) and o.grav_enabled and o.grav_hancock == hancock
    q = ek.params_from_ini("[run]\nsolver_name=Hydro_Muscl_2D\n[mesh]\nnx=8\nny=8\n[hydro]\nproblem=rayleigh_taylor\n"
                          "[gravity]\nenabled=true\nwell_balanced_reconstruction_enabled=on\n")
    assert q.gravity_enabled == 1 and q.gravity_well_balanced == 1 and list(q.gravity) == [0.0, np.float32(-0.1), 0.0]
    r = ek.params_from_ini("[run]\nsolver_name=Hydro_Muscl_3D\n[mesh]\nnx=8\nny=8\nnz=8\n[hydro]\nproblem=implode\n"
                          "[gravity]\nenabled=Yes\n[rayleigh_taylor]\ngz=-1\n")
    # getBool is case-sensitive (Yes -> default false); the field is RT-only
    assert r.gravity_enabled == 0 and list(r.gravity) == [0.0, 0.0, 0.0]
