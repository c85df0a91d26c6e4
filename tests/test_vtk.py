"""VTK output parity: files written by the library equal, byte for byte, the
files the reference's own writer (save_VTK_2D/3D, IO_VTK.cpp:24-400) wrote
for the same final states (tests/golden/*.vti, made by make_golden.py).

CPU tests: ek_write_vtk on the reference's final state.  GPU test: the exact
build's solver runs the case and writes its state with ek_solver_save_vtk.
"""

import os
import sys

import numpy as np
import pytest

import euler_kokkos_gb300 as ek
from helpers import GOLDEN, load_golden

sys.path.insert(0, GOLDEN)
from make_golden import VTK_CASES, with_output  # noqa: E402


def _params(ini, out_dir, ascii, **over):
    return ek.params_from_ini(with_output(ini, out_dir, "ref", ascii), **over)


@pytest.mark.parametrize("fixture", sorted(VTK_CASES))
def test_writer_matches_reference_file(fixture, tmp_path):
    case, ascii = VTK_CASES[fixture]
    g = load_golden(case)
    p = _params(str(g["ini"]), str(tmp_path), ascii)
    fname = ek.write_vtk(p, g["U"], step=0)
    with open(os.path.join(GOLDEN, fixture), "rb") as f:
        want = f.read()
    with open(fname, "rb") as f:
        got = f.read()
    assert got == want


def test_layout_right_and_file_names(tmp_path):
    g = load_golden("implode2d_32")
    p = _params(str(g["ini"]), str(tmp_path), False)
    a = ek.write_vtk(p, g["U"], step=7)
    b = ek.write_vtk(p, np.ascontiguousarray(g["U"].transpose(3, 2, 1, 0)), step=7, debug_name="dbg",
                     layout=ek.EK_LAYOUT_RIGHT)
    assert a.endswith("ref_0000007.vti") and b.endswith("ref_dbg_0000007.vti")
    assert open(a, "rb").read() == open(b, "rb").read()


def test_output_section_defaults():
    g = load_golden("implode2d_32")
    p = ek.params_from_ini(str(g["ini"]))
    assert p.output_prefix == "implode" and p.vtk_enabled == 0 and p.vtk_ascii == 0
    q = ek.params_from_ini("[run]\nsolver_name=Hydro_Muscl_2D\n[mesh]\nnx=8\nny=8\n")
    assert q.output_dir == "./" and q.output_prefix == "output" and q.vtk_enabled == 1


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", sorted(VTK_CASES))
def test_solver_save_vtk_matches_reference_file(fixture, tmp_path):
    case, ascii = VTK_CASES[fixture]
    g = load_golden(case)
    p = _params(str(g["ini"]), str(tmp_path), ascii, exact_fp=1)
    with ek.SolverFactory.create(p.solver_name, p) as s:
        s.set_state(g["U0"])
        s.run(len(g["dts"]))
        fname = s.save_vtk(0)
    with open(os.path.join(GOLDEN, fixture), "rb") as f:
        want = f.read()
    assert open(fname, "rb").read() == want
