"""Restart files: a run continued from a restart file equals the uninterrupted
run.  The restarted solver starts at iteration 0 with the saved time and
output counter (the reference's init_restart, SolverHydroMuscl.h:512-580);
states and time steps are bit-identical in both builds and precisions."""

import numpy as np
import pytest

import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import interior

pytestmark = pytest.mark.gpu

CASES = [
    ("hydro3d", lambda: P.blast_3d(n=24, nsteps=10 ** 6)),
    ("hydro2d", lambda: P.implode_2d(n=40, nsteps=10 ** 6)),
    ("mhd3d", lambda: P.orszag_tang_3d(n=16, nsteps=10 ** 6)),
    ("mhd2d", lambda: P.orszag_tang_2d(n=32, nsteps=10 ** 6)),
]


@pytest.mark.parametrize("over", [dict(exact_fp=1), dict(precision=1)], ids=["exact", "mixed"])
@pytest.mark.parametrize("label,build", CASES, ids=[c[0] for c in CASES])
def test_restart_continues_bitwise(label, build, over, tmp_path):
    ini, U0 = build()
    p = ek.params_from_ini(ini, **over)
    with ek.Solver(p) as s:
        s.set_state(U0)
        s.run(6)
        U_ref, t_ref, dts_ref = s.get_state(), s.m_t, s.dt_history()
    path = str(tmp_path / "restart.bin")
    with ek.Solver(p) as s:
        s.set_state(U0)
        s.run(3)
        s.save_restart(path, times_saved=5)
    with ek.Solver(p) as s:
        assert s.load_restart(path) == 5
        assert s.m_iteration == 0
        s.run(3)
        U, t, dts = s.get_state(), s.m_t, s.dt_history()
    gw = p.ghost_width
    assert t == t_ref
    assert np.array_equal(dts[:3], dts_ref[3:6])
    assert np.array_equal(interior(U, gw, p.dim), interior(U_ref, gw, p.dim))


def test_restart_rejects_other_grid(tmp_path):
    ini, U0 = P.blast_3d(n=16, nsteps=10)
    path = str(tmp_path / "r.bin")
    with ek.Solver(ek.params_from_ini(ini)) as s:
        s.set_state(U0)
        s.run(1)
        s.save_restart(path)
        s.load_restart(path, reset_time=True)
        assert s.m_t == 0.0
    ini2, _ = P.blast_3d(n=12, nsteps=10)
    with ek.Solver(ek.params_from_ini(ini2)) as s:
        with pytest.raises(ek.EkError) as e:
            s.load_restart(path)
        assert e.value.status == ek.EK_ERR_INVALID
