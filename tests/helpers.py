"""Helpers shared by the test modules (imported by tests only)."""

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_cases(kind=None):
    """Names of the golden fixtures; kind: 'hydro', 'mhd' (3D), 'mhd2d' or None."""
    names = sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz")))
    is_mhd = [n.startswith("mhd") or n.startswith("ot") for n in names]
    if kind == "hydro":
        return [n for n, m in zip(names, is_mhd) if not m]
    if kind == "mhd":
        return [n for n, m in zip(names, is_mhd) if m and "2d" not in n]
    if kind == "mhd2d":
        return [n for n, m in zip(names, is_mhd) if m and "2d" in n]
    return names


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
