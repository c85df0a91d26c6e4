"""Helpers shared by the test modules (imported by tests only)."""

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _solver_of(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        ini = str(z["ini"])
    solver = version = None
    for line in ini.splitlines():
        t = line.strip()
        if t.startswith("solver_name="):
            solver = t.split("=", 1)[1].strip()
        elif t.startswith("implementationVersion="):
            version = int(t.split("=", 1)[1].split()[0])
    return solver, version or 0


def golden_cases(kind=None, bitwise=True):
    """Names of the golden fixtures; kind: 'hydro', 'mhd' (3D), 'mhd2d' or None.
    bitwise: the fixtures the version-0 arithmetic reproduces bit for bit
    (False: the ones written by the reference's atomic-update hydro version 2,
    equal up to the summation order)."""
    names = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz")))
    out = []
    for n in names:
        solver, version = _solver_of(n)
        mhd = solver.startswith("MHD")
        atomic = not mhd and version == 2
        if atomic == bitwise:
            continue
        if kind is None or (kind == "hydro" and not mhd) or (kind == "mhd" and solver == "MHD_Muscl_3D") or \
                (kind == "mhd2d" and solver == "MHD_Muscl_2D"):
            out.append(n)
    return out


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def interior(U, gw, dim):
    if dim == 2:
        return U[:, :, gw:-gw, gw:-gw]
    return U[:, gw:-gw, gw:-gw, gw:-gw]


def rel_linf(a, b):
    """max |a-b| / max |b| per variable (NaNs must coincide)."""
    out = []
    for v in range(a.shape[0]):
        x, y = a[v], b[v]
        scale = np.nanmax(np.abs(y)) or 1.0
        d = np.abs(x - y)
        out.append(float(np.nanmax(d) / scale) if d.size else 0.0)
    return np.array(out)


def rel_l1(a, b):
    out = []
    for v in range(a.shape[0]):
        x, y = a[v], b[v]
        denom = np.sum(np.abs(y)) or 1.0
        out.append(float(np.sum(np.abs(x - y)) / denom))
    return np.array(out)
