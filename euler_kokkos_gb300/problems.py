"""Seeded synthetic initial states for the benchmark and parity workloads.

Each builder returns ``(ini_text, U0)``: an input deck in the reference's own
.ini format (the same keys its ConfigMap/HydroParams read) and the full
ghost-inclusive conserved state U0 of shape (nbvar, ksize, jsize, isize),
float64, in the reference's LayoutLeft order (i fastest, variable slowest).

The deterministic part of every state follows the reference init functors
(cited per builder).  The seeded noise the workloads add is drawn from a
counter-based generator, ``splitmix64(seed ^ global_cell_index)`` mapped to
[-1, 1), so it does not depend on any thread or tile decomposition.

Reals are first passed through float32, because the reference reads every
real parameter through ``strtof`` (utils/config/ConfigMap.cpp:37-46).
"""

from __future__ import annotations

import math

import numpy as np

__all__ = [
    "splitmix_uniform",
    "implode_2d",
    "blast_3d",
    "orszag_tang_3d",
    "orszag_tang_2d",
    "mhd_blast_3d",
    "kelvin_helmholtz_2d",
    "rayleigh_taylor",
    "kh_ensemble",
    "smooth_random",
    "ini_text",
]

_M64 = (1 << 64) - 1


def splitmix_uniform(seed: int, index: np.ndarray) -> np.ndarray:
    """U[-1,1) from splitmix64(seed ^ index), vectorised over ``index``."""
    z = (np.uint64(seed & _M64) ^ index.astype(np.uint64)) + np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def _f(x: float) -> float:
    """A real parameter as the reference sees it (strtof then double)."""
    return float(np.float32(x))


def ini_text(sections: dict) -> str:
    out = []
    for sec, kv in sections.items():
        out.append("[%s]" % sec)
        for k, v in kv.items():
            out.append("%s=%s" % (k, v))
        out.append("")
    return "\n".join(out)


def _deck(solver, nx, ny, nz, bc, gamma0, cfl, slope_type, riemann, problem, nsteps, extra=None):
    sec = {
        "run": {"solver_name": solver, "tEnd": "1e30", "nStepmax": nsteps, "nOutput": 0, "nlog": 1000000},
        "mesh": {"nx": nx, "ny": ny, "nz": nz, "xmin": 0.0, "xmax": 1.0, "ymin": 0.0, "ymax": 1.0,
                 "zmin": 0.0, "zmax": 1.0,
                 "boundary_type_xmin": bc[0], "boundary_type_xmax": bc[1],
                 "boundary_type_ymin": bc[2], "boundary_type_ymax": bc[3],
                 "boundary_type_zmin": bc[4], "boundary_type_zmax": bc[5]},
        "hydro": {"gamma0": repr(gamma0), "cfl": repr(cfl), "niter_riemann": 10, "iorder": 2,
                  "slope_type": repr(slope_type), "problem": problem, "riemann": riemann},
        "output": {"outputPrefix": problem, "vtk_enabled": "false", "hdf5_enabled": "false"},
        "other": {"implementationVersion": 0},
    }
    if extra:
        for k, v in extra.items():
            sec.setdefault(k, {}).update(v)
    return ini_text(sec)


def _centres(n, gw, lo, d):
    i = np.arange(n + 2 * gw, dtype=np.float64)
    return lo + d / 2 + (i - gw) * d


def implode_2d(n=256, ny=None, nsteps=100, bc=(1, 1, 1, 1), slope_type=1.0, cfl=0.8,
               gamma0=1.4, riemann="hllc"):
    """2D implode: HydroInitFunctors2D.h:60-140 (shape 0).  Outer state where
    x + y > (xmin+xmax)/2 + ymin, inner state (rho 0.125, p 0.14) elsewhere."""
    ny = n if ny is None else ny
    gw = 2
    ini = _deck("Hydro_Muscl_2D", n, ny, 1, list(bc) + [1, 1], gamma0, cfl, slope_type, riemann,
                "implode", nsteps,
                {"implode": {"density_outer": 1.0, "pressure_outer": 1.0,
                             "density_inner": 0.125, "pressure_inner": 0.14}})
    g = _f(gamma0)
    dx, dy = 1.0 / n, 1.0 / ny
    x = _centres(n, gw, 0.0, dx)[None, :]
    y = _centres(ny, gw, 0.0, dy)[:, None]
    outer = (x + y) > (0.0 + 1.0) / 2.0 + 0.0
    rho_out, p_out, rho_in, p_in = 1.0, 1.0, _f(0.125), _f(0.14)
    U = np.zeros((4, 1, ny + 2 * gw, n + 2 * gw))
    U[0, 0] = np.where(outer, rho_out, rho_in)
    U[1, 0] = np.where(outer, p_out / (g - 1.0) + 0.5 * rho_out * (0.0 * 0.0 + 0.0 * 0.0),
                       p_in / (g - 1.0) + 0.5 * rho_in * (0.0 * 0.0 + 0.0 * 0.0))
    return ini, U


def blast_3d(n=256, nsteps=50, seed=0xB1A57, noise=0.01, bc=(2,) * 6, slope_type=1.0, cfl=0.7,
             gamma0=1.4, riemann="hllc"):
    """3D blast: HydroInitFunctors3D.h:195-262 (density_out 1, pressure_in 10,
    pressure_out 0.1, radius 0.1 at the centre) plus rho_out*(1 + noise*u)."""
    gw = 2
    ini = _deck("Hydro_Muscl_3D", n, n, n, bc, gamma0, cfl, slope_type, riemann, "blast", nsteps,
                {"blast": {"radius": 0.1, "center_x": 0.5, "center_y": 0.5, "center_z": 0.5,
                           "density_in": 1.0, "density_out": 1.0,
                           "pressure_in": 10.0, "pressure_out": 0.1}})
    g = _f(gamma0)
    d = 1.0 / n
    s = n + 2 * gw
    x = _centres(n, gw, 0.0, d)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    r = _f(0.1)
    c = _f(0.5)
    d2 = (X - c) * (X - c) + (Y - c) * (Y - c) + (Z - c) * (Z - c)
    inside = d2 < r * r
    idx = np.arange(s * s * s, dtype=np.uint64).reshape(s, s, s)
    u = splitmix_uniform(seed, idx)
    U = np.zeros((5, s, s, s))
    U[0] = np.where(inside, 1.0, 1.0 * (1.0 + noise * u))
    U[1] = np.where(inside, _f(10.0) / (g - 1.0), _f(0.1) / (g - 1.0))
    return ini, U


def orszag_tang_3d(n=256, nsteps=100, seed=0x0257A6, vz_noise=1e-3, slope_type=2.0, cfl=0.8,
                   gamma0=5.0 / 3.0, riemann="hlld"):
    """3D Orszag-Tang (vortex along z, kt = 0): MHDInitFunctors3D.h:441-547.
    rho = gamma p0 = 25/(36 pi), p0 = 5/(12 pi), v = (-sin 2 pi y, sin 2 pi x,
    vz_noise*u).  Face-centred B is the discrete curl of
    A_z = B0 (cos(4 pi x)/(4 pi) + cos(2 pi y)/(2 pi)), B0 = 1/sqrt(4 pi),
    so the discrete div B vanishes to round-off; the total energy uses the
    face-averaged B as in the reference."""
    gw = 3
    ini = _deck("MHD_Muscl_3D", n, n, n, (3,) * 6, gamma0, cfl, slope_type, riemann,
                "orszag_tang", nsteps, {"OrszagTang": {"kt": 0.0, "vortex_dir": 2}})
    g = _f(gamma0)
    d = 1.0 / n
    s = n + 2 * gw
    B0 = 1.0 / math.sqrt(4 * math.pi)
    p0 = g / (4 * math.pi)
    d0 = g * p0
    xc = _centres(n, gw, 0.0, d)
    xf = xc - d / 2  # left faces
    X, Y = xc[None, None, :], xc[None, :, None]
    XF, YF = xf[None, None, :], xf[None, :, None]

    def Az(xx, yy):
        return B0 * (np.cos(4 * math.pi * xx) / (4 * math.pi) + np.cos(2 * math.pi * yy) / (2 * math.pi))

    idx = np.arange(s * s * s, dtype=np.uint64).reshape(s, s, s)
    u = splitmix_uniform(seed, idx)
    U = np.zeros((8, s, s, s))
    U[0] = d0
    U[2] = np.broadcast_to(-d0 * np.sin(Y * 2 * math.pi), (s, s, s))
    U[3] = np.broadcast_to(d0 * np.sin(X * 2 * math.pi), (s, s, s))
    U[4] = d0 * vz_noise * u
    # Bx on the x-face (x_{i-1/2}, y_j): (Az(x, y_{j+1/2}) - Az(x, y_{j-1/2})) / dy
    U[5] = np.broadcast_to((Az(XF, YF + d) - Az(XF, YF)) / d, (s, s, s))
    # By on the y-face (x_i, y_{j-1/2}): -(Az(x_{i+1/2}, y) - Az(x_{i-1/2}, y)) / dx
    U[6] = np.broadcast_to(-(Az(XF + d, YF) - Az(XF, YF)) / d, (s, s, s))
    U[7] = 0.0
    # total energy from face-averaged B, cells with i,j,k < size-1 (MHDInitFunctors3D.h:523-547)
    e = np.zeros((s, s, s))
    rho = U[0]
    bxc = (U[5][:, :, :-1] + U[5][:, :, 1:]) / 2
    byc = (U[6][:, :-1, :] + U[6][:, 1:, :]) / 2
    bzc = (U[7][:-1] + U[7][1:]) / 2
    ekin = 0.5 * (U[2] ** 2 / rho + U[3] ** 2 / rho + U[4] ** 2 / rho)
    e[:-1, :-1, :-1] = (p0 / (g - 1.0) + ekin[:-1, :-1, :-1]
                        + 0.5 * (bxc[:-1, :-1, :] ** 2 + byc[:-1, :, :-1] ** 2 + bzc[:, :-1, :-1] ** 2))
    U[1] = e
    return ini, U


def orszag_tang_2d(n=512, ny=None, nsteps=100, seed=0x0257A6, vz_noise=0.0, slope_type=2.0, cfl=0.8,
                   gamma0=5.0 / 3.0, riemann="hlld"):
    """2D Orszag-Tang: MHDInitFunctors2D.h:345-470.  rho = gamma p0, p0 =
    gamma/(4 pi), v = (-sin 2 pi y, sin 2 pi x, vz_noise*u), B = (-B0 sin 2 pi y,
    B0 sin 4 pi x, 0) at cell centres (each component constant along its own
    direction, so the discrete div B is exactly zero), B0 = 1/sqrt(4 pi); the
    total energy uses the face-averaged B for cells i, j < size-1."""
    ny = n if ny is None else ny
    gw = 3
    ini = _deck("MHD_Muscl_2D", n, ny, 1, (3, 3, 3, 3, 3, 3), gamma0, cfl, slope_type, riemann,
                "orszag_tang", nsteps, {"OrszagTang": {"kt": 0.0, "vortex_dir": 2}})
    g = _f(gamma0)
    twopi = 2 * math.pi
    B0 = 1.0 / math.sqrt(2 * twopi)
    p0 = g / (2 * twopi)
    d0 = g * p0
    X = _centres(n, gw, 0.0, 1.0 / n)[None, :]
    Y = _centres(ny, gw, 0.0, 1.0 / ny)[:, None]
    sy, sx = ny + 2 * gw, n + 2 * gw
    idx = np.arange(sx * sy, dtype=np.uint64).reshape(sy, sx)
    U = np.zeros((8, 1, sy, sx))
    U[0, 0] = d0
    U[2, 0] = np.broadcast_to(-d0 * np.sin(Y * twopi), (sy, sx))
    U[3, 0] = np.broadcast_to(d0 * np.sin(X * twopi), (sy, sx))
    U[4, 0] = d0 * vz_noise * splitmix_uniform(seed, idx) if vz_noise else 0.0
    U[5, 0] = np.broadcast_to(-B0 * np.sin(Y * twopi), (sy, sx))
    U[6, 0] = np.broadcast_to(B0 * np.sin(2.0 * X * twopi), (sy, sx))
    U[7, 0] = 0.0
    u0 = U[:, 0]
    e = np.zeros((sy, sx))
    e[:-1, :-1] = (p0 / (g - 1.0)
                   + 0.5 * (u0[2, :-1, :-1] ** 2 / u0[0, :-1, :-1] + u0[3, :-1, :-1] ** 2 / u0[0, :-1, :-1])
                   + 0.5 * (((u0[5, :-1, :-1] + u0[5, :-1, 1:]) / 2) ** 2
                            + ((u0[6, :-1, :-1] + u0[6, 1:, :-1]) / 2) ** 2))
    U[1, 0] = e
    return ini, U


def mhd_blast_3d(n=512, nsteps=30, seed=0x10B37A, noise=0.005, slope_type=2.0, cfl=0.8,
                 gamma0=5.0 / 3.0, riemann="hlld", by_ratio=0.0):
    """Low-beta 3D MHD blast: MHDInitFunctors3D.h:290-365 with uniform
    B = (10/sqrt(4 pi), by_ratio * 10/sqrt(4 pi), 0) on every face (div B = 0
    exactly), background rho = 1 + noise*u, p 0.1, sphere r 0.1 at the centre
    with p 10.

    by_ratio = 0 is the configuration as specified.  With the field along x
    only, the x-face fast speed equals the Alfven speed in the quiescent
    medium, and the reference's HLLD star state divides 0/0
    (RiemannSolvers_MHD.h:204-221): the run is NaN after its first step.  A
    small uniform transverse component (by_ratio > 0) keeps the field
    divergence-free and the plasma beta low, and avoids that degeneracy."""
    gw = 3
    bx = 10.0 / math.sqrt(4 * math.pi)
    by = by_ratio * bx
    ini = _deck("MHD_Muscl_3D", n, n, n, (2,) * 6, gamma0, cfl, slope_type, riemann, "blast",
                nsteps, {"blast": {"radius": 0.1, "center_x": 0.5, "center_y": 0.5, "center_z": 0.5,
                                   "density_in": 1.0, "density_out": 1.0, "pressure_in": 10.0,
                                   "pressure_out": 0.1, "bx_in": bx, "by_in": by, "bz_in": 0.0,
                                   "bx_out": bx, "by_out": by, "bz_out": 0.0}})
    g = _f(gamma0)
    bxf, byf = _f(bx), _f(by)
    d = 1.0 / n
    s = n + 2 * gw
    x = _centres(n, gw, 0.0, d)
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    r, c = _f(0.1), _f(0.5)
    d2 = (X - c) * (X - c) + (Y - c) * (Y - c) + (Z - c) * (Z - c)
    inside = d2 < r * r
    idx = np.arange(s * s * s, dtype=np.uint64).reshape(s, s, s)
    u = splitmix_uniform(seed, idx)
    U = np.zeros((8, s, s, s))
    U[0] = np.where(inside, 1.0, 1.0 * (1.0 + noise * u))
    U[5] = bxf
    U[6] = byf
    emag = 0.5 * (bxf * bxf + byf * byf + 0.0)
    U[1] = np.where(inside, _f(10.0) / (g - 1.0) + emag, _f(0.1) / (g - 1.0) + emag)
    return ini, U


def mhd_blast_2d(n=1024, nsteps=100, seed=0x10B372, noise=0.005, slope_type=2.0, cfl=0.8,
                 gamma0=5.0 / 3.0, riemann="hlld", by_ratio=0.1):
    """Low-beta 2D MHD blast: MHDInitFunctors2D.h:248-340 with uniform
    B = (10/sqrt(4 pi), by_ratio * 10/sqrt(4 pi), 0) on every face, background
    rho = 1 + noise*u, p 0.1, disc r 0.1 at the centre with p 10; outflow
    boundaries.  The transverse component keeps the HLLD star states away from
    the 0/0 of a field along x only (see mhd_blast_3d)."""
    gw = 3
    bx = 10.0 / math.sqrt(4 * math.pi)
    by = by_ratio * bx
    ini = _deck("MHD_Muscl_2D", n, n, 1, (2,) * 6, gamma0, cfl, slope_type, riemann, "blast",
                nsteps, {"blast": {"radius": 0.1, "center_x": 0.5, "center_y": 0.5,
                                   "density_in": 1.0, "density_out": 1.0, "pressure_in": 10.0,
                                   "pressure_out": 0.1, "bx_in": bx, "by_in": by, "bz_in": 0.0,
                                   "bx_out": bx, "by_out": by, "bz_out": 0.0}})
    g = _f(gamma0)
    bxf, byf = _f(bx), _f(by)
    s = n + 2 * gw
    x = _centres(n, gw, 0.0, 1.0 / n)
    X, Y = x[None, :], x[:, None]
    r, c = _f(0.1), _f(0.5)
    inside = (X - c) * (X - c) + (Y - c) * (Y - c) < r * r
    u = splitmix_uniform(seed, np.arange(s * s, dtype=np.uint64).reshape(s, s))
    U = np.zeros((8, 1, s, s))
    U[0, 0] = np.where(inside, 1.0, 1.0 * (1.0 + noise * u))
    U[5, 0] = bxf
    U[6, 0] = byf
    emag = 0.5 * (bxf * bxf + byf * byf + 0.0)
    U[1, 0] = np.where(inside, _f(10.0) / (g - 1.0) + emag, _f(0.1) / (g - 1.0) + emag)
    return ini, U


def kelvin_helmholtz_2d(n=128, shear=0.5, ratio=2.0, seed=20261203, nsteps=200, ampl=0.01,
                        pressure=2.5, slope_type=2.0, cfl=0.8, gamma0=1.4, riemann="hllc"):
    """2D Kelvin-Helmholtz, random-perturbation branch of
    HydroInitFunctors2D.h:276-309: band 0.25 < y < 0.75 holds rho = ratio,
    vx = -shear/2, outside rho = 1, vx = +shear/2, p = pressure; both velocity
    components get ampl * u with u from the counter-based generator.  x is
    periodic, y reflecting."""
    gw = 2
    ini = _deck("Hydro_Muscl_2D", n, n, 1, (3, 3, 1, 1, 1, 1), gamma0, cfl, slope_type, riemann,
                "kelvin_helmholtz", nsteps,
                {"KH": {"d_in": ratio, "d_out": 1.0, "pressure": pressure,
                        "vflow_in": -shear / 2, "vflow_out": shear / 2,
                        "perturbation_rand": "true", "perturbation_sine_robertson": "false",
                        "amplitude": ampl, "rand_seed": seed & 0x7FFFFFFF}})
    g = _f(gamma0)
    d = 1.0 / n
    s = n + 2 * gw
    x = _centres(n, gw, 0.0, d)
    yn = x[:, None] * np.ones((1, s))
    inband = ~((yn < 0.25) | (yn > 0.75))
    dens = np.where(inband, _f(ratio), 1.0)
    vx = np.where(inband, _f(-shear / 2), _f(shear / 2))
    idx = np.arange(s * s, dtype=np.uint64).reshape(s, s)
    a = _f(ampl)
    uu = vx + a * 0.5 * splitmix_uniform(seed, 2 * idx)
    vv = 0.0 + a * 0.5 * splitmix_uniform(seed, 2 * idx + 1)
    U = np.zeros((4, 1, s, s))
    U[0, 0] = dens
    U[2, 0] = dens * uu
    U[3, 0] = dens * vv
    U[1, 0] = _f(pressure) / (g - 1.0) + 0.5 * dens * (uu * uu + vv * vv)
    return ini, U


def rayleigh_taylor(dim=2, nx=100, ny=None, nz=None, nsteps=100, amplitude=0.01, d0=1.0, d1=2.0,
                    g=-0.1, hancock=False, riemann="approx", slope_type=2.0, cfl=0.7, gamma0=1.4,
                    seed=0x5A7E, noise=0.0):
    """Rayleigh-Taylor instability under static gravity (the reference's
    settings/test_rayleigh_taylor_{2d,3d}.ini decks, [gravity] enabled): the
    init of HydroInitFunctors2D.h:690-772 / HydroInitFunctors3D.h:757-843 --
    density d1 above the mid-plane of the gravity axis (y in 2D, z in 3D) and
    d0 below, a cosine velocity perturbation along that axis, hydrostatic
    energy (P0 + rho g.x)/(gamma0 - 1) -- on [-0.5,0.5]^(dim-1) x [-1.5,1.5],
    periodic across and reflecting along the gravity axis.  g is the gravity
    component along that axis; noise adds rho*(1 + noise*u) with the seeded
    splitmix noise.  hancock turns on [gravity] hancock_predictor_enabled."""
    if dim == 2:
        ny = 3 * nx if ny is None else ny
        nz = 1
        bc = (3, 3, 1, 1, 1, 1)
        mesh = {"xmin": -0.5, "xmax": 0.5, "ymin": -1.5, "ymax": 1.5}
        gvec = (0.0, _f(g), 0.0)
    else:
        ny = nx if ny is None else ny
        nz = 3 * nx if nz is None else nz
        bc = (3, 3, 3, 3, 1, 1)
        mesh = {"xmin": -0.5, "xmax": 0.5, "ymin": -0.5, "ymax": 0.5, "zmin": -1.5, "zmax": 1.5}
        gvec = (0.0, 0.0, _f(g))
    gw = 2
    rt = {"amplitude": amplitude, "d0": d0, "d1": d1, "gx": 0.0, "gy": g if dim == 2 else 0.0}
    if dim == 3:
        rt["gz"] = g
    grav = {"enabled": "yes", "static": "yes"}
    if hancock:
        grav["hancock_predictor_enabled"] = "yes"
    ini = _deck("Hydro_Muscl_%dD" % dim, nx, ny, nz, bc, gamma0, cfl, slope_type, riemann, "rayleigh_taylor",
                nsteps, {"mesh": mesh, "gravity": grav, "rayleigh_taylor": rt})
    gam = _f(gamma0)
    lo = [_f(mesh["xmin"]), _f(mesh["ymin"]), _f(mesh.get("zmin", 0.0))]
    hi = [_f(mesh["xmax"]), _f(mesh["ymax"]), _f(mesh.get("zmax", 1.0))]
    n = (nx, ny, nz)
    d = [(hi[a] - lo[a]) / n[a] for a in range(3)]
    x = _centres(nx, gw, lo[0], d[0])[None, None, :]
    y = _centres(ny, gw, lo[1], d[1])[None, :, None]
    z = _centres(nz, gw, lo[2], d[2])[:, None, None] if dim == 3 else np.zeros((1, 1, 1))
    shp = (nz + 2 * gw if dim == 3 else 1, ny + 2 * gw, nx + 2 * gw)
    axis = y if dim == 2 else z
    mid = (lo[1] + hi[1]) / 2 if dim == 2 else (lo[2] + hi[2]) / 2
    rho = np.broadcast_to(np.where(axis > mid, _f(d1), _f(d0)), shp).copy()
    if noise:
        idx = np.arange(int(np.prod(shp)), dtype=np.uint64).reshape(shp)
        rho = rho * (1.0 + noise * splitmix_uniform(seed, idx))
    Lx, Ly = hi[0] - lo[0], hi[1] - lo[1]
    pert = _f(amplitude) * rho * (1 + np.cos(2 * math.pi * x / Lx)) * (1 + np.cos(2 * math.pi * y / Ly)) / 4
    nb = 4 if dim == 2 else 5
    U = np.zeros((nb,) + shp)
    U[0] = rho
    U[2 + (dim - 1)] = np.broadcast_to(pert, shp)
    gx, gy, gz = gvec
    U[1] = (1.0 + rho * (gx * x + gy * y + gz * z)) / (gam - 1.0)
    return ini, U


def smooth_random(dim=3, mhd=False, nx=16, ny=None, nz=None, seed=1, bc=None, slope_type=2.0,
                  cfl=0.7, gamma0=None, nsteps=10, amp=0.3, riemann=None):
    """A seeded smooth state on an arbitrary (possibly non-cubic) grid, for
    parity tests: rho ~ 1 +- amp, p ~ 1 +- amp/2, |v| ~ amp, and for MHD a
    face-centred B that is the discrete curl of a seeded smooth vector
    potential (so div B vanishes to round-off)."""
    ny = nx if ny is None else ny
    nz = (nx if dim == 3 else 1) if nz is None else nz
    gw = 3 if mhd else 2
    if gamma0 is None:
        gamma0 = 5.0 / 3.0 if mhd else 1.4
    if bc is None:
        bc = (3,) * 6
    if riemann is None:
        riemann = "hlld" if mhd else "hllc"
    solver = ("MHD" if mhd else "Hydro") + "_Muscl_%dD" % dim
    ini = _deck(solver, nx, ny, nz if dim == 3 else 1, bc, gamma0, cfl, slope_type, riemann,
                "random", nsteps)
    rng = np.random.default_rng(seed)
    g = _f(gamma0)
    shp = (nz + 2 * gw if dim == 3 else 1, ny + 2 * gw, nx + 2 * gw)
    x = _centres(nx, gw, 0.0, 1.0 / nx)[None, None, :]
    y = _centres(ny, gw, 0.0, 1.0 / ny)[None, :, None]
    z = _centres(nz, gw, 0.0, 1.0 / nz)[:, None, None] if dim == 3 else np.zeros((1, 1, 1))

    def field(a):
        ph = rng.uniform(0, 2 * math.pi, 3)
        kk = rng.integers(1, 3, 3)
        return a * np.sin(2 * math.pi * kk[0] * x + ph[0]) * np.cos(2 * math.pi * kk[1] * y + ph[1]) \
            * np.cos(2 * math.pi * kk[2] * z + ph[2])

    rho = np.broadcast_to(1.0 + field(amp), shp)
    pr = np.broadcast_to(1.0 + field(amp / 2), shp)
    vel = [np.broadcast_to(field(amp), shp) for _ in range(3)]
    nb = 8 if mhd else (4 if dim == 2 else 5)
    U = np.zeros((nb,) + shp)
    U[0] = rho
    U[2] = rho * vel[0]
    U[3] = rho * vel[1]
    if dim == 3 or mhd:
        U[4] = rho * vel[2] if (dim == 3 or mhd) else 0.0
    if dim == 2 and not mhd:
        U[1] = pr / (g - 1.0) + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2)
        return ini, U
    if not mhd:
        U[1] = pr / (g - 1.0) + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2)
        return ini, U
    # face-centred B = discrete curl of a nodal/edge vector potential
    dx, dy, dz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    xf, yf = x - dx / 2, y - dy / 2
    zf = z - dz / 2 if dim == 3 else z
    coef = rng.uniform(-0.5, 0.5, (3, 3))
    ph = rng.uniform(0, 2 * math.pi, (3, 3))

    def pot(c, X, Y, Z):
        return (coef[c, 0] * np.sin(2 * math.pi * X + ph[c, 0]) / (2 * math.pi)
                + coef[c, 1] * np.sin(2 * math.pi * Y + ph[c, 1]) / (2 * math.pi)
                + coef[c, 2] * np.sin(2 * math.pi * Z + ph[c, 2]) / (2 * math.pi)
                + coef[c, 0] * coef[c, 1] * np.cos(2 * math.pi * (X + Y) + ph[c, 2]) / (2 * math.pi))

    # Ax on x-edges (x_i, y_{j-1/2}, z_{k-1/2}), Ay on y-edges, Az on z-edges
    def Ax(i0, j0, k0):
        return pot(0, x + i0 * dx, yf + j0 * dy, zf + k0 * dz)

    def Ay(i0, j0, k0):
        return pot(1, xf + i0 * dx, y + j0 * dy, zf + k0 * dz)

    def Az(i0, j0, k0):
        return pot(2, xf + i0 * dx, yf + j0 * dy, z + k0 * dz)

    if dim == 3:
        bx = (Az(0, 1, 0) - Az(0, 0, 0)) / dy - (Ay(0, 0, 1) - Ay(0, 0, 0)) / dz
        by = (Ax(0, 0, 1) - Ax(0, 0, 0)) / dz - (Az(1, 0, 0) - Az(0, 0, 0)) / dx
        bz = (Ay(1, 0, 0) - Ay(0, 0, 0)) / dx - (Ax(0, 1, 0) - Ax(0, 0, 0)) / dy
    else:
        bx = (Az(0, 1, 0) - Az(0, 0, 0)) / dy
        by = -(Az(1, 0, 0) - Az(0, 0, 0)) / dx
        bz = 0.2 + field(0.1)
    U[5] = np.broadcast_to(bx, shp)
    U[6] = np.broadcast_to(by, shp)
    U[7] = np.broadcast_to(bz, shp)
    bxc = U[5].copy()
    bxc[..., :-1] = 0.5 * (U[5][..., :-1] + U[5][..., 1:])
    byc = U[6].copy()
    byc[:, :-1, :] = 0.5 * (U[6][:, :-1, :] + U[6][:, 1:, :])
    bzc = U[7].copy()
    if dim == 3:
        bzc[:-1] = 0.5 * (U[7][:-1] + U[7][1:])
    U[1] = pr / (g - 1.0) + 0.5 * rho * (vel[0] ** 2 + vel[1] ** 2 + vel[2] ** 2) \
        + 0.5 * (bxc ** 2 + byc ** 2 + bzc ** 2)
    return ini, U


KH_SIZES = (64, 96, 128, 192, 256)


def kh_ensemble(n_inst=512, seed=20261203, nsteps=200, sizes=KH_SIZES):
    """The batched Kelvin-Helmholtz workload: instance n draws its grid from
    ``sizes`` (squared), its shear speed from U[0.2, 1.0] and its density ratio
    from U[1.5, 3] with splitmix64(seed + n); each instance is periodic in x,
    reflecting in y, with a seeded 1% velocity perturbation."""
    out = []
    for n in range(n_inst):
        r = splitmix_uniform(seed + n, np.arange(3, dtype=np.uint64))  # U[-1, 1)
        size = sizes[int((r[0] + 1.0) / 2.0 * len(sizes)) % len(sizes)]
        shear = 0.2 + 0.8 * (r[1] + 1.0) / 2.0
        ratio = 1.5 + 1.5 * (r[2] + 1.0) / 2.0
        out.append(kelvin_helmholtz_2d(n=size, shear=shear, ratio=ratio, seed=seed + 7919 * n, nsteps=nsteps))
    return out
