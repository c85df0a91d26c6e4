"""The reference-side plugin (euler_kokkos_gb300/plugin/ek_gb300_plugin.cpp)
and the Kokkos-free SolverBase interface (include/ek/solver.hpp).

* The plugin is compiled into the reference's OWN driver (src/main.cpp and
  its solver sources, against the repository's Kokkos-API shim) and linked
  with libek_gb300 (oracle/Makefile.ref, target `plugin`).  Registered under
  the reference's solver names, it replaces the built-in solvers: on a
  machine without a GPU the reference's main() stops in the library with its
  "no CUDA device" message, while the same driver without the plugin runs the
  deck on the CPU.  Needs the reference's sources: EK_REFERENCE, or the tree
  oracle/build.sh built the harness from (oracle/_ref/reference_path).
* ek/solver.hpp compiles as plain C++17 against the library alone.  ek_main
  is built on it, so the GPU tests of ek_main run it on the device.
"""

import os
import shutil
import subprocess

import pytest

from conftest import gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
LIBDIR = os.path.join(ROOT, "euler_kokkos_gb300", "_build")


def _reference_tree():
    ref = os.environ.get("EK_REFERENCE")
    if not ref:
        rec = os.path.join(ORACLE, "_ref", "reference_path")
        if os.path.exists(rec):
            ref = open(rec).read().strip()
    return ref if ref and os.path.isdir(os.path.join(ref, "src")) else None


def _deck(ref, tmp_path):
    """The reference's 2D implode deck at 32^2, 20 steps, no output."""
    out = []
    for line in open(os.path.join(ref, "settings", "test_implode_2D.ini")).read().splitlines():
        key = line.split("=", 1)[0].strip()
        if key in ("nx", "ny"):
            line = key + "=32"
        elif key == "nStepmax":
            line = "nStepmax=20"
        elif key == "nOutput":
            line = "nOutput=0"
        out.append(line)
    path = tmp_path / "deck.ini"
    path.write_text("\n".join(out) + "\n")
    return path


@pytest.fixture(scope="module")
def plugin_build():
    ref = _reference_tree()
    if ref is None:
        pytest.skip("the reference's sources are not available (EK_REFERENCE)")
    r = subprocess.run(["make", "-s", "-C", ORACLE, "-f", "Makefile.ref", "REF=" + ref, "LIBEK=" + LIBDIR,
                        "plugin"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return ref, os.path.join(ORACLE, "_ref", "euler_kokkos"), os.path.join(ORACLE, "_ref", "euler_kokkos_gb300")


def test_plugin_links_the_library(plugin_build):
    _, _, exe = plugin_build
    if shutil.which("ldd"):
        r = subprocess.run(["ldd", exe], capture_output=True, text=True)
        assert "libek_gb300.so" in r.stdout


def test_reference_main_without_the_plugin_runs_on_the_cpu(plugin_build, tmp_path):
    ref, exe, _ = plugin_build
    deck = _deck(ref, tmp_path)
    r = subprocess.run([exe, str(deck)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert r.returncode == 0, r.stderr
    assert "Start computation...." in r.stdout and "number of Mcell-updates/s" in r.stdout


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU path of the plugin")
def test_plugin_replaces_the_factory_solvers(plugin_build, tmp_path):
    ref, _, exe = plugin_build
    deck = _deck(ref, tmp_path)
    r = subprocess.run([exe, str(deck)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    # the reference's main() ran (its banner) and SolverFactory::create built
    # the plugin's solver, which stopped in the library
    assert "Kokkos configuration" in r.stdout
    assert r.returncode != 0
    assert "libek_gb300: no CUDA device" in r.stderr
    assert "Start computation" not in r.stdout


def test_solver_hpp_compiles_against_the_library_alone(tmp_path):
    src = tmp_path / "use_solver.cpp"
    src.write_text(r'''
#include "ek/solver.hpp"
#include <cstdio>
int main()
{
  const std::string ini = "[run]\nsolver_name=Hydro_Muscl_2D\nnStepmax=3\n[mesh]\nnx=16\nny=16\n";
  try
  {
    ek::Solver s(ini);
    std::vector<double> U(s.state_size(), 1.0);
    s.set_state(U.data());
    while (!s.finished())
      s.next_iteration();
    std::printf("ran %d steps, t = %g, cells %lld\n", s.m_iteration, s.m_t, s.m_nCells);
    return 0;
  }
  catch (const ek::Error & e)
  {
    std::printf("status %d: %s\n", (int)e.status, e.what());
    return 3;
  }
}
''')
    exe = tmp_path / "use_solver"
    cxx = shutil.which("g++") or shutil.which("c++")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        str(src), "-L" + LIBDIR, "-lek_gb300", "-Wl,-rpath," + LIBDIR, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    if gpu_available():
        assert r.returncode == 0 and "ran 3 steps" in r.stdout, r.stdout + r.stderr
    else:
        assert r.returncode == 3 and "status 7" in r.stdout, r.stdout
