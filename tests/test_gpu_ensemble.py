"""The batched 2D ensemble (persistent kernel per step, CUDA graph replay).

Every instance of an ensemble must evolve exactly as the same run on its own:
bitwise against the oracle in the exact FP64 build, and bitwise against the
single-solver mixed path in the mixed form (the ensemble runs the same tile
code), each instance with its own grid, boundaries and time step.
"""

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import interior

pytestmark = pytest.mark.gpu


def _cases():
    cases = P.kh_ensemble(n_inst=6, sizes=(16, 24, 40), nsteps=8)
    cases.append(P.implode_2d(n=33, ny=20, nsteps=8))
    cases.append(P.smooth_random(dim=2, nx=45, ny=17, seed=77, bc=(1, 2, 3, 3, 1, 1), nsteps=8))
    return cases


@pytest.mark.parametrize("graph", [False, True])
def test_ensemble_exact_matches_oracle_per_instance(graph):
    cases = _cases()
    params = [ek.params_from_ini(ini, exact_fp=1) for ini, _ in cases]
    with ek.Ensemble(params) as e:
        for i, (_, U0) in enumerate(cases):
            e.set_state(i, U0)
        e.run(4, graph=graph)
        e.run(4, graph=graph)  # replay
        e.synchronize()
        for i, (ini, U0) in enumerate(cases):
            o = eko.Oracle(eko.params_from_ini(ini), U0)
            do = o.run(8)
            assert np.array_equal(e.dt_history(i), do), i
            assert np.array_equal(interior(e.get_state(i), 2, 2), interior(o.state(), 2, 2)), i


def test_ensemble_mixed_matches_single_solver_bitwise():
    cases = _cases()
    params = [ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED) for ini, _ in cases]
    with ek.Ensemble(params) as e:
        for i, (_, U0) in enumerate(cases):
            e.set_state(i, U0)
        e.run(8)
        e.synchronize()
        tot = e.totals()
        for i, (ini, U0) in enumerate(cases):
            with ek.Solver(params[i]) as s:
                s.set_state(U0)
                s.run(8)
                assert np.array_equal(e.get_state(i), s.get_state()), i
                assert np.array_equal(e.dt_history(i), s.dt_history()), i
                assert abs(tot[i, 0] - s.totals()[0]) <= 1e-12 * abs(tot[i, 0])


def test_ensemble_instances_stop_at_their_tend():
    a = P.implode_2d(n=24, nsteps=100)
    b = P.implode_2d(n=24, nsteps=100)
    ini_b = b[0].replace("tEnd=1e30", "tEnd=0.004")
    params = [ek.params_from_ini(a[0], exact_fp=1), ek.params_from_ini(ini_b, exact_fp=1)]
    with ek.Ensemble(params) as e:
        e.set_state(0, a[1])
        e.set_state(1, b[1])
        e.run(20)
        e.synchronize()
        ta, _, ia = e.time(0)
        tb, _, ib = e.time(1)
        assert ia == 20 and ib < 20 and tb == float(np.float32(0.004))  # tEnd read through strtof
        o = eko.Oracle(eko.params_from_ini(ini_b), b[1])
        do = o.run(20)
        assert len(do) == ib and np.array_equal(e.dt_history(1), do)
        assert np.array_equal(interior(e.get_state(1), 2, 2), interior(o.state(), 2, 2))
