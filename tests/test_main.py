"""ek_main: the reference's driver loop (main.cpp:53-159) in C++ over the C
ABI, with the reference harness's command line.  GPU: the exact build run
through it reproduces the golden fixtures bit for bit (final state, dt
sequence, time).  CPU: argument errors and the no-GPU path."""

import os
import subprocess
import sys

import numpy as np
import pytest

import eko
from euler_kokkos_gb300 import build as B
from helpers import golden_cases, interior, load_golden

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def _run(args, **kw):
    return subprocess.run([B.main_path()] + [str(a) for a in args], capture_output=True, text=True, timeout=600,
                          **kw)


def test_usage_and_bad_inputs(tmp_path):
    r = _run([])
    assert r.returncode == 2 and "usage" in r.stderr
    r = _run([tmp_path / "missing.ini", 1, tmp_path / "o.ekst", tmp_path / "u0.ekst"])
    assert r.returncode == 2


@pytest.mark.skipif(__import__("conftest").gpu_available(), reason="checks the no-GPU path")
def test_no_gpu_is_a_clean_error(tmp_path):
    g = load_golden("implode2d_32")
    ini = tmp_path / "case.ini"
    ini.write_text(str(g["ini"]))
    p = eko.params_from_ini(str(g["ini"]))
    eko.write_ekst(str(tmp_path / "u0.ekst"), g["U0"], p.dim, p.gw)
    r = _run([ini, 5, tmp_path / "o.ekst", tmp_path / "u0.ekst"])
    assert r.returncode == 1 and "no CUDA device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["implode2d_32", "blast3d_12", "ot3d_12", "ot2d_24", "mhdblast3d_10_nan",
                                  "rt3d_hllc_hancock", "deck_mhd_brio_wu_2d_x", "deck_kelvin_helmholtz_3D"])
def test_driver_reproduces_reference_bitwise(name, tmp_path):
    g = load_golden(name)
    ini = str(g["ini"]) + "\n[gb300]\nexact=1\n"
    (tmp_path / "case.ini").write_text(ini)
    p = eko.params_from_ini(ini)
    eko.write_ekst(str(tmp_path / "u0.ekst"), g["U0"], p.dim, p.gw)
    r = _run([tmp_path / "case.ini", len(g["dts"]), tmp_path / "out.ekst", tmp_path / "u0.ekst"])
    assert r.returncode == 0, r.stderr
    out = eko.read_ekst(str(tmp_path / "out.ekst"))
    assert np.array_equal(out["dts"], g["dts"], equal_nan=True)
    assert np.array_equal(interior(out["U"], p.gw, p.dim), interior(g["U"], p.gw, p.dim), equal_nan=True)
    assert out["iteration"] == int(g["iteration"])
    assert np.array_equal(np.array(out["t"]), g["t"], equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("name,nlog", [("blast3d_12", 1), ("ot3d_12", 2)])
def test_driver_prints_the_reference_log_and_perf_lines(name, nlog, tmp_path):
    """The step log of next_iteration_impl (SolverHydroMuscl.h:646-652,
    SolverMHDMuscl.h:752-758: iteration, dt and t before the step, every nlog
    steps), "final time is" (main.cpp:150-151) and the timer summary with the
    Perf line (solver_utils.h:15-55)."""
    import re

    g = load_golden(name)
    ini = re.sub(r"(?m)^nlog=.*$", "nlog=%d" % nlog, str(g["ini"])) + "\n[gb300]\nexact=1\n"
    (tmp_path / "case.ini").write_text(ini)
    p = eko.params_from_ini(ini)
    eko.write_ekst(str(tmp_path / "u0.ekst"), g["U0"], p.dim, p.gw)
    dts = g["dts"]
    r = _run([tmp_path / "case.ini", len(dts), tmp_path / "out.ekst", tmp_path / "u0.ekst"])
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "Start computation...."
    want, t = [], 0.0
    for n in range(len(dts)):
        # m_dt before step n is the previous step's dt (the constructor's for n = 0)
        if n % nlog == 0:
            want.append("time step=%7d (dt=% 10.8f t=% 10.8f)" % (n, dts[max(n - 1, 0)], t))
        t += dts[n]
    assert [l for l in lines if l.startswith("time step=")] == want
    assert "final time is %f" % t in lines
    for label in ("total        time", "godunov      time", "compute dt   time", "boundaries   time",
                  "comp. prim.  time", "comp. flux   time", "hydro update time", "io           time"):
        assert any(l.startswith(label + " : ") for l in lines), label
    perf = [l for l in lines if l.startswith("Perf              : ")]
    assert len(perf) == 1 and perf[0].endswith(" number of Mcell-updates/s")
    assert float(perf[0].split(":")[1].split()[0]) > 0
