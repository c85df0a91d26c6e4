"""Generate the golden fixtures of tests/golden from the reference itself.

Each fixture is the reference's OWN solver code (the upstream sources compiled
unmodified against the Kokkos-API shim, oracle/_ref/ref_run, built by
oracle/build.sh) run on a seeded initial state from euler_kokkos_gb300.problems.
Stored per case (compressed .npz): the .ini text, the injected initial state
U0, the final state U, the dt sequence and the final time.

Run from the repository root, with EK_REFERENCE naming the reference's source
tree (oracle/build.sh builds the harness from it):
    EK_REFERENCE=<reference tree> python tests/golden/make_golden.py [case ...]
(no case names: every case)
"""

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import eko  # noqa: E402
from euler_kokkos_gb300 import problems as P  # noqa: E402

CASES = {
    # name: (builder, nsteps)
    "implode2d_32": (lambda: P.implode_2d(n=32, nsteps=20), 20),
    "implode2d_mixedbc_mc": (lambda: P.implode_2d(n=24, ny=20, nsteps=12, bc=(2, 2, 3, 3),
                                                   slope_type=2.0), 12),
    "kh2d_16": (lambda: P.kelvin_helmholtz_2d(n=16, nsteps=10), 10),
    "hydro2d_random_reflect": (lambda: P.smooth_random(dim=2, nx=20, ny=14, seed=3, bc=(1, 1, 1, 1, 1, 1),
                                                        slope_type=1.0, nsteps=10), 10),
    "blast3d_12": (lambda: P.blast_3d(n=12, nsteps=8), 8),
    "hydro3d_random_mixedbc": (lambda: P.smooth_random(dim=3, nx=10, ny=8, nz=6, seed=4,
                                                        bc=(1, 1, 3, 3, 2, 2), slope_type=2.0,
                                                        nsteps=6), 6),
    "ot3d_12": (lambda: P.orszag_tang_3d(n=12, nsteps=6), 6),
    "mhd3d_random_periodic": (lambda: P.smooth_random(dim=3, mhd=True, nx=8, ny=10, nz=7, seed=5,
                                                       slope_type=2.0, nsteps=4), 4),
    "mhd3d_random_reflect_minmod": (lambda: P.smooth_random(dim=3, mhd=True, nx=8, ny=8, nz=8, seed=6,
                                                             bc=(1, 1, 1, 1, 1, 1), slope_type=1.0,
                                                             nsteps=4), 4),
    "mhd3d_random_outflow": (lambda: P.smooth_random(dim=3, mhd=True, nx=9, ny=8, nz=8, seed=7,
                                                      bc=(2, 2, 2, 2, 2, 2), slope_type=2.0,
                                                      nsteps=4), 4),
    "mhdblast3d_10_nan": (lambda: P.mhd_blast_3d(n=10, nsteps=3), 3),
    # the same low-beta blast with a small transverse field (no 0/0 in HLLD)
    "mhdblast3d_lowbeta_12": (lambda: P.mhd_blast_3d(n=12, nsteps=6, by_ratio=0.1), 6),
    # hydro slope_type 0: zero slopes, first order (HydroBaseFunctor2D.h:488-502,
    # HydroBaseFunctor3D.h:498-520)
    "implode2d_first_order": (lambda: P.implode_2d(n=24, nsteps=10, slope_type=0.0), 10),
    "blast3d_first_order": (lambda: P.blast_3d(n=10, nsteps=5, slope_type=0.0), 5),
    "ot2d_24": (lambda: P.orszag_tang_2d(n=24, nsteps=8), 8),
    "ot2d_noise_20x16": (lambda: P.orszag_tang_2d(n=20, ny=16, nsteps=6, vz_noise=1e-2), 6),
    "mhd2d_random_periodic": (lambda: P.smooth_random(dim=2, mhd=True, nx=20, ny=14, seed=8,
                                                       slope_type=2.0, nsteps=6), 6),
    "mhd2d_random_reflect_minmod": (lambda: P.smooth_random(dim=2, mhd=True, nx=16, ny=12, seed=9,
                                                             bc=(1, 1, 1, 1, 1, 1), slope_type=1.0,
                                                             nsteps=6), 6),
    "mhd2d_random_mixedbc": (lambda: P.smooth_random(dim=2, mhd=True, nx=18, ny=16, seed=10,
                                                      bc=(2, 2, 3, 3, 1, 1), slope_type=2.0,
                                                      nsteps=6), 6),
    # the other Riemann solvers of the path (riemann = approx / llf / hll)
    "implode2d_llf": (lambda: P.implode_2d(n=24, nsteps=10, riemann="llf"), 10),
    "implode2d_hll": (lambda: P.implode_2d(n=24, nsteps=10, riemann="hll"), 10),
    "implode2d_approx": (lambda: P.implode_2d(n=24, nsteps=10, riemann="approx"), 10),
    "hydro2d_random_approx_mc": (lambda: P.smooth_random(dim=2, nx=18, ny=15, seed=12, bc=(2, 2, 3, 3, 1, 1),
                                                          slope_type=2.0, nsteps=8, riemann="approx"), 8),
    "blast3d_llf": (lambda: P.blast_3d(n=10, nsteps=5, riemann="llf"), 5),
    "blast3d_approx": (lambda: P.blast_3d(n=10, nsteps=5, riemann="approx"), 5),
    "ot3d_hll": (lambda: P.orszag_tang_3d(n=10, nsteps=4, riemann="hll"), 4),
    "ot3d_llf": (lambda: P.orszag_tang_3d(n=10, nsteps=4, riemann="llf"), 4),
    "ot2d_hll": (lambda: P.orszag_tang_2d(n=20, nsteps=6, riemann="hll"), 6),
    "ot2d_llf": (lambda: P.orszag_tang_2d(n=20, nsteps=6, riemann="llf"), 6),
    # static gravity (Rayleigh-Taylor decks; the reference's init sets the
    # uniform field): CFL with gravity, source term, Hancock predictor
    "rt2d_approx": (lambda: P.rayleigh_taylor(dim=2, nx=16, nsteps=12, noise=0.01), 12),
    "rt2d_hllc_hancock": (lambda: P.rayleigh_taylor(dim=2, nx=12, ny=30, nsteps=10, riemann="hllc", hancock=True,
                                                    noise=0.02, slope_type=1.0, g=-0.3), 10),
    "rt3d_approx": (lambda: P.rayleigh_taylor(dim=3, nx=6, nsteps=6, noise=0.01), 6),
    "rt3d_hllc_hancock": (lambda: P.rayleigh_taylor(dim=3, nx=8, ny=6, nz=16, nsteps=5, riemann="hllc",
                                                    hancock=True, noise=0.02, g=-0.3), 5),
    # a non-uniform field (builder returns the field too; the harness loads
    # it into the reference solver's gravity_field)
    "grav2d_field_llf": (lambda: _with_field(P.rayleigh_taylor(dim=2, nx=14, ny=20, nsteps=8, riemann="llf",
                                                               hancock=True, noise=0.02), 31), 8),
    "grav3d_field_hllc": (lambda: _with_field(P.rayleigh_taylor(dim=3, nx=6, ny=8, nz=10, nsteps=5,
                                                                riemann="hllc", hancock=True, noise=0.02), 32), 5),
}


# The reference's own input decks (settings/*.ini; the MPI decks excepted),
# at reduced grid sizes, run from the reference's OWN init for a few steps:
# fixture name: (deck file, mesh overrides, steps, implementationVersion
# override or None).  Hydro version 2 only changes the summation order of the
# update (atomics); the MHD versions 1 and 2 compute other numbers.  Those
# decks run at version 0 here; the round-off equivalence of hydro version 2
# is pinned by the *_v2 fixtures.
DECKS = {
    "deck_blast_2D": ("test_blast_2D.ini", {"nx": 32, "ny": 48}, 10, None),
    "deck_blast_3D": ("test_blast_3D.ini", {"nx": 16, "ny": 12, "nz": 8}, 6, None),
    "deck_four_quadrant_2D": ("test_four_quadrant_2D.ini", {"nx": 32, "ny": 32}, 10, None),
    "deck_four_quadrant_3D": ("test_four_quadrant_3D.ini", {"nx": 12, "ny": 12, "nz": 12}, 5, None),
    "deck_implode_2D": ("test_implode_2D.ini", {"nx": 32, "ny": 16}, 10, None),
    "deck_implode_3D": ("test_implode_3D.ini", {"nx": 16, "ny": 12, "nz": 8}, 6, None),
    "deck_mhd_blast_2D": ("test_mhd_blast_2D.ini", {"nx": 32, "ny": 48}, 6, None),
    "deck_mhd_blast_3D": ("test_mhd_blast_3D.ini", {"nx": 12, "ny": 12, "nz": 12}, 4, 0),
    "deck_mhd_brio_wu_2d_x": ("test_mhd_brio_wu_2d_x.ini", {"nx": 64, "ny": 8}, 10, 0),
    "deck_mhd_brio_wu_2d_y": ("test_mhd_brio_wu_2d_y.ini", {"nx": 8, "ny": 64}, 10, 0),
    "deck_mhd_brio_wu_3d_x": ("test_mhd_brio_wu_3d_x.ini", {"nx": 48, "ny": 6, "nz": 6}, 6, 0),
    "deck_mhd_brio_wu_3d_y": ("test_mhd_brio_wu_3d_y.ini", {"nx": 6, "ny": 48, "nz": 6}, 6, 0),
    "deck_mhd_brio_wu_3d_z": ("test_mhd_brio_wu_3d_z.ini", {"nx": 6, "ny": 6, "nz": 48}, 6, 0),
    "deck_mhd_orszag_tang_2D": ("test_mhd_orszag_tang_2D.ini", {"nx": 32, "ny": 32}, 8, None),
    "deck_mhd_orszag_tang_3D": ("test_mhd_orszag_tang_3D.ini", {"nx": 16, "ny": 16, "nz": 8}, 5, None),
    "deck_mhd_rotor": ("test_mhd_rotor.ini", {"nx": 32, "ny": 32}, 8, None),
    "deck_gresho_vortex_2D": ("test_muscl_gresho_vortex_2D.ini", {"nx": 32, "ny": 32}, 8, None),
    "deck_isentropic_vortex_2d": ("test_muscl_isentropic_vortex_2d.ini", {"nx": 32, "ny": 32}, 8, None),
    "deck_kelvin_helmholtz_2D": ("test_muscl_kelvin_helmholtz_2D.ini", {"nx": 32, "ny": 32}, 8, None),
    "deck_kelvin_helmholtz_2D_mhd": ("test_muscl_kelvin_helmholtz_2D_mhd.ini", {"nx": 32, "ny": 32}, 6, None),
    "deck_kelvin_helmholtz_3D": ("test_muscl_kelvin_helmholtz_3D.ini", {"nx": 16, "ny": 16, "nz": 16}, 5, None),
    "deck_rayleigh_taylor_2d": ("test_rayleigh_taylor_2d.ini", {"nx": 20, "ny": 60}, 10, None),
    "deck_rayleigh_taylor_3d": ("test_rayleigh_taylor_3d.ini", {"nx": 10, "ny": 10, "nz": 30}, 5, None),
    "deck_mhd_fieldloop2d": ("mhd_fieldloop2d.ini", {"nx": 32, "ny": 20}, 8, None),
    "deck_mhd_fieldloop3d": ("mhd_fieldloop3d.ini", {"nx": 16, "ny": 8, "nz": 8}, 5, None),
    # the reference's atomic-update versions, as the decks ask for them
    "deck_implode_2D_v2": ("test_implode_2D.ini", {"nx": 32, "ny": 16}, 10, 2),
    "deck_kelvin_helmholtz_3D_v2": ("test_muscl_kelvin_helmholtz_3D.ini", {"nx": 16, "ny": 16, "nz": 16}, 5, 2),
}
SETTINGS = os.path.join(os.environ.get("EK_REFERENCE", ""), "settings")


def deck_text(fname, mesh, nsteps, version):
    """The deck with its mesh resized, nStepmax = nsteps, output off and
    (optionally) implementationVersion replaced."""
    out, sec = [], ""
    with open(os.path.join(SETTINGS, fname)) as f:
        lines = f.read().splitlines()
    for line in lines:
        t = line.strip()
        if t.startswith("["):
            sec = t[1:t.index("]")].lower() if "]" in t else ""
            out.append(line)
            continue
        key = t.split("=", 1)[0].strip() if "=" in t and not t.startswith(("#", ";")) else None
        if sec == "mesh" and key in mesh:
            line = "%s=%d" % (key, mesh[key])
        elif sec == "run" and key and key.lower() == "nstepmax":
            line = "nStepmax=%d" % nsteps
        elif sec == "output" and key and key.lower() in ("vtk_enabled", "hdf5_enabled", "pnetcdf_enabled"):
            line = "%s=false" % key
        elif sec == "other" and key == "implementationVersion" and version is not None:
            line = "implementationVersion=%d" % version
        out.append(line)
    return "\n".join(out) + "\n"


def make_decks(names, out_dir):
    work = tempfile.mkdtemp(prefix="ek_deck_")
    for name in names:
        fname, mesh, nsteps, version = DECKS[name]
        ini = deck_text(fname, mesh, nsteps, version)
        res = eko.run_reference_deck(ini, nsteps, os.path.join(work, name))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), ini=np.array(ini), U0=res["U0"],
                            U=res["U"], dts=res["dts"], t=np.array(res["t"]),
                            iteration=np.array(res["iteration"]))
        print(name, res["U0"].shape, "steps", len(res["dts"]), "nan", int(np.isnan(res["U"]).sum()))


def _with_field(case, seed):
    """(ini, U0) -> (ini, U0, G): a seeded smooth gravity field, one
    component per dimension, on every cell (ghosts included)."""
    ini, U0 = case
    dim = 3 if U0.shape[1] > 1 else 2
    rng = np.random.default_rng(seed)
    shp = U0.shape[1:]
    k, j, i = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shp], indexing="ij")
    G = np.empty((dim,) + shp)
    for c in range(dim):
        a = rng.uniform(0.2, 1.0, 4)
        G[c] = a[0] * np.sin(0.4 * i + a[1]) * np.cos(0.3 * j + a[2]) * np.cos(0.5 * k + a[3]) - 0.3
    return ini, U0, G


# VTK output parity: the reference writes the final state of these cases with
# its own writer (save_VTK_2D/3D); the fixture is the written file.
VTK_CASES = {
    # fixture name: (golden case, ascii)
    "implode2d_32.vti": ("implode2d_32", False),
    "ot3d_12.vti": ("ot3d_12", False),
    "kh2d_16_ascii.vti": ("kh2d_16", True),
    "mhd2d_random_periodic_ascii.vti": ("mhd2d_random_periodic", True),
}


def with_output(ini, out_dir, prefix, ascii):
    """The deck with its [output] section replaced: VTK on, given dir/prefix."""
    lines, skip = [], False
    for line in ini.splitlines():
        if line.strip().startswith("["):
            skip = line.strip() == "[output]"
            if skip:
                lines += ["[output]", "outputDir=" + out_dir, "outputPrefix=" + prefix,
                          "vtk_enabled=true", "hdf5_enabled=false",
                          "outputVtkAscii=" + ("true" if ascii else "false")]
                continue
        if not skip:
            lines.append(line)
    return "\n".join(lines) + "\n"


def make_vtk(names):
    out_dir = os.path.dirname(os.path.abspath(__file__))
    for fname in names:
        case, ascii = VTK_CASES[fname]
        build, nsteps = CASES[case]
        ini, U0 = build()
        work = tempfile.mkdtemp(prefix="ek_vtk_")
        ini_o = with_output(ini, work, "ref", ascii)
        eko.run_reference(ini_o, U0, nsteps, work, save=True)
        src = os.path.join(work, "ref_0000000.vti")
        with open(src, "rb") as f, open(os.path.join(out_dir, fname), "wb") as g:
            g.write(f.read())
        print(fname, os.path.getsize(os.path.join(out_dir, fname)), "bytes")


def main():
    if not os.path.isdir(os.path.join(os.environ.get("EK_REFERENCE", ""), "src")):
        sys.exit("make_golden: set EK_REFERENCE to the reference's source tree")
    out_dir = os.path.dirname(os.path.abspath(__file__))
    work = tempfile.mkdtemp(prefix="ek_golden_")
    names = sys.argv[1:] or list(CASES) + list(VTK_CASES) + list(DECKS)
    make_vtk([n for n in names if n in VTK_CASES])
    make_decks([n for n in names if n in DECKS], out_dir)
    for name in [n for n in names if n in CASES]:
        build, nsteps = CASES[name]
        case = build()
        ini, U0 = case[:2]
        G = case[2] if len(case) > 2 else None
        res = eko.run_reference(ini, U0, nsteps, os.path.join(work, name), gravity_field=G)
        extra = {} if G is None else {"G": G}
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), ini=np.array(ini), U0=U0,
                            U=res["U"], dts=res["dts"], t=np.array(res["t"]),
                            iteration=np.array(res["iteration"]), **extra)
        print(name, U0.shape, "steps", len(res["dts"]), "nan", int(np.isnan(res["U"]).sum()))


if __name__ == "__main__":
    main()
