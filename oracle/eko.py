"""Python side of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests, the smoke check and the CPU-baseline leg of the benchmark import
this module.  It provides:

* ``parse_ini`` / ``params_from_ini``: a restatement of the reference input
  front end -- inih parsing with lower-cased ``section.name`` keys
  (utils/config/inih/ini.cpp:80-160, INIReader.cpp:105-111), ``getFloat``
  through C ``strtof`` so every real is rounded to float first
  (utils/config/ConfigMap.cpp:37-46), and the parameter derivation of
  HydroParams (shared/HydroParams.cpp:37-180, 327-359) and SolverBase
  (shared/SolverBase.cpp:21-40);
* ``Oracle``: a ctypes wrapper of the C restatement in ek_oracle.c;
* ``read_ekst`` / ``write_ekst`` for the state files the reference harness
  (oracle/_ref/ref_run) reads and writes.
"""

from __future__ import annotations

import ctypes
import os
import struct
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libek_oracle.so")
OPS_LIB_PATH = os.path.join(HERE, "_build", "libek_oracle_ops.so")
REF_RUN = os.path.join(HERE, "_ref", "ref_run")
REF_RUN_FAST = os.path.join(HERE, "_ref", "ref_run_fast")

_libc = ctypes.CDLL(None)
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]
_libc.strtol.restype = ctypes.c_long
_libc.strtol.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int]


# --------------------------------------------------------------------------
# INI front end
# --------------------------------------------------------------------------
def _find_char_or_comment(s: str, c: str) -> int:
    was_ws = False
    i = 0
    while i < len(s) and s[i] != c and not (was_ws and s[i] == ";"):
        was_ws = s[i].isspace()
        i += 1
    return i


def parse_ini(text: str) -> dict:
    """inih semantics: returns {"section.name": value} with lower-cased keys."""
    values: dict = {}
    section = ""
    prev_name = ""
    for raw in text.splitlines():
        line = raw[:199]  # MAX_LINE 200 (fgets keeps 199 chars)
        stripped = line.rstrip()
        start_off = len(stripped) - len(stripped.lstrip())
        start = stripped.lstrip()
        if prev_name and start and start_off > 0:
            values[(section + "." + prev_name).lower()] = start
            continue
        if not start or start[0] in ";#":
            continue
        if start[0] == "[":
            end = _find_char_or_comment(start[1:], "]")
            if end < len(start) - 1 and start[1 + end] == "]":
                section = start[1 : 1 + end][:49]
                prev_name = ""
            continue
        end = _find_char_or_comment(start, "=")
        if end < len(start) and start[end] == "=":
            name = start[:end].rstrip()
            value = start[end + 1 :].lstrip()
            e2 = _find_char_or_comment(value, "\0")
            if e2 < len(value) and value[e2] == ";":
                value = value[:e2]
            value = value.rstrip()
            prev_name = name[:49]
            values[(section + "." + name).lower()] = value
    return values


def get_string(cfg: dict, section: str, name: str, default: str) -> str:
    return cfg.get((section + "." + name).lower(), default)


def get_float(cfg: dict, section: str, name: str, default: float) -> float:
    """ConfigMap::getFloat: strtof, float result promoted to double."""
    s = get_string(cfg, section, name, "")
    b = s.encode()
    end = ctypes.c_char_p()
    buf = ctypes.create_string_buffer(b)
    v = _libc.strtof(buf, ctypes.byref(end))
    consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.addressof(buf)
    if consumed > 0:
        return float(np.float32(v))
    return float(np.float32(default))


def get_integer(cfg: dict, section: str, name: str, default: int) -> int:
    s = get_string(cfg, section, name, "")
    buf = ctypes.create_string_buffer(s.encode())
    end = ctypes.c_char_p()
    v = _libc.strtol(buf, ctypes.byref(end), 0)
    consumed = ctypes.cast(end, ctypes.c_void_p).value - ctypes.addressof(buf)
    return int(v) if consumed > 0 else int(default)


def get_bool(cfg: dict, section: str, name: str, default: bool) -> bool:
    s = get_string(cfg, section, name, "")
    val = default
    if s in ("1", "yes", "true", "on"):
        val = True
    if s in ("0", "no", "false", "off"):
        val = False
    if not s:
        val = default
    return val


class eko_params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("mhd", ctypes.c_int),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("gw", ctypes.c_int),
        ("nbvar", ctypes.c_int),
        ("isize", ctypes.c_int),
        ("jsize", ctypes.c_int),
        ("ksize", ctypes.c_int),
        ("xmin", ctypes.c_double),
        ("ymin", ctypes.c_double),
        ("zmin", ctypes.c_double),
        ("dx", ctypes.c_double),
        ("dy", ctypes.c_double),
        ("dz", ctypes.c_double),
        ("bc", ctypes.c_int * 6),
        ("gamma0", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("slope_type", ctypes.c_double),
        ("smallr", ctypes.c_double),
        ("smallc", ctypes.c_double),
        ("smallp", ctypes.c_double),
        ("smallpp", ctypes.c_double),
        ("cIso", ctypes.c_double),
        ("Omega0", ctypes.c_double),
        ("riemann", ctypes.c_int),
        ("tEnd", ctypes.c_double),
        ("nStepmax", ctypes.c_int),
        ("gamma6", ctypes.c_double),
        ("grav_enabled", ctypes.c_int),
        ("grav_hancock", ctypes.c_int),
        ("gravity", ctypes.c_double * 3),
    ]


RIEMANN = {"approx": 0, "llf": 1, "hll": 2, "hllc": 3, "hlld": 4}


@dataclass
class Params:
    """Derived run parameters, as HydroParams::HydroParams + init computes them."""

    solver_name: str
    dim: int
    mhd: bool
    nx: int
    ny: int
    nz: int
    gw: int
    nbvar: int
    isize: int
    jsize: int
    ksize: int
    xmin: float
    xmax: float
    ymin: float
    ymax: float
    zmin: float
    zmax: float
    dx: float
    dy: float
    dz: float
    bc: list
    gamma0: float
    cfl: float
    slope_type: float
    smallr: float
    smallc: float
    smallp: float
    smallpp: float
    gamma6: float
    riemann: int
    tEnd: float
    nStepmax: int
    problem: str
    grav_enabled: bool = False
    grav_hancock: bool = False
    gravity: tuple = (0.0, 0.0, 0.0)
    extra: dict = field(default_factory=dict)

    def to_c(self) -> eko_params:
        p = eko_params()
        p.dim, p.mhd = self.dim, int(self.mhd)
        p.nx, p.ny, p.nz = self.nx, self.ny, self.nz
        p.gw, p.nbvar = self.gw, self.nbvar
        p.isize, p.jsize, p.ksize = self.isize, self.jsize, self.ksize
        p.xmin, p.ymin, p.zmin = self.xmin, self.ymin, self.zmin
        p.dx, p.dy, p.dz = self.dx, self.dy, self.dz
        for i in range(6):
            p.bc[i] = self.bc[i]
        p.gamma0, p.cfl, p.slope_type = self.gamma0, self.cfl, self.slope_type
        p.smallr, p.smallc, p.smallp, p.smallpp = self.smallr, self.smallc, self.smallp, self.smallpp
        p.cIso, p.Omega0 = 0.0, 0.0
        p.riemann = self.riemann
        p.tEnd, p.nStepmax = self.tEnd, self.nStepmax
        p.gamma6 = self.gamma6
        p.grav_enabled, p.grav_hancock = int(self.grav_enabled), int(self.grav_hancock)
        for i in range(3):
            p.gravity[i] = self.gravity[i]
        return p

    @property
    def shape(self):
        """numpy shape of the full state (var, k, j, i)."""
        return (self.nbvar, self.ksize if self.dim == 3 else 1, self.jsize, self.isize)


def params_from_ini(text: str) -> Params:
    cfg = parse_ini(text)
    name = get_string(cfg, "run", "solver_name", "unknown")
    dims = {"Hydro_Muscl_2D": (2, False, 4, 2), "Hydro_Muscl_3D": (3, False, 5, 2),
            "MHD_Muscl_2D": (2, True, 8, 3), "MHD_Muscl_3D": (3, True, 8, 3)}
    if name not in dims:
        raise ValueError("Solver name not valid : " + name)
    dim, mhd, nbvar, gw = dims[name]
    nx = get_integer(cfg, "mesh", "nx", 1)
    ny = get_integer(cfg, "mesh", "ny", 1)
    nz = get_integer(cfg, "mesh", "nz", 1)
    xmin = get_float(cfg, "mesh", "xmin", 0.0)
    xmax = get_float(cfg, "mesh", "xmax", 1.0)
    ymin = get_float(cfg, "mesh", "ymin", 0.0)
    ymax = get_float(cfg, "mesh", "ymax", 1.0)
    zmin = get_float(cfg, "mesh", "zmin", 0.0)
    zmax = get_float(cfg, "mesh", "zmax", 1.0)
    bc = [get_integer(cfg, "mesh", "boundary_type_" + f, 1)
          for f in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")]
    rs = get_string(cfg, "hydro", "riemann", "approx")
    riemann = RIEMANN.get(rs, 0)
    gamma0 = get_float(cfg, "hydro", "gamma0", 1.4)
    cfl = get_float(cfg, "hydro", "cfl", 0.5)
    slope_type = get_float(cfg, "hydro", "slope_type", 1.0)
    smallc = get_float(cfg, "hydro", "smallc", 1e-10)
    smallr = get_float(cfg, "hydro", "smallr", 1e-10)
    isize = nx + 2 * gw
    jsize = ny + 2 * gw
    ksize = nz + 2 * gw
    dx = (xmax - xmin) / nx
    dy = (ymax - ymin) / ny
    dz = (zmax - zmin) / nz
    smallp = smallc * smallc / gamma0
    smallpp = smallr * smallp
    gamma6 = (gamma0 + 1.0) / (2.0 * gamma0)
    problem = get_string(cfg, "hydro", "problem", "unknown")
    # GravityParams (shared/GravityParams.h:32-37); the field is the uniform
    # one of the Rayleigh-Taylor init (RayleighTaylorInstabilityParams.h:28-34),
    # zero for the other problems
    gravity = (0.0, 0.0, 0.0)
    if problem == "rayleigh_taylor":
        gravity = (get_float(cfg, "rayleigh_taylor", "gx", 0.0), get_float(cfg, "rayleigh_taylor", "gy", -0.1),
                   get_float(cfg, "rayleigh_taylor", "gz", 0.0) if dim == 3 else 0.0)
    return Params(
        solver_name=name, dim=dim, mhd=mhd, nx=nx, ny=ny, nz=nz, gw=gw, nbvar=nbvar,
        isize=isize, jsize=jsize, ksize=ksize, xmin=xmin, xmax=xmax, ymin=ymin, ymax=ymax,
        zmin=zmin, zmax=zmax, dx=dx, dy=dy, dz=dz, bc=bc, gamma0=gamma0, cfl=cfl,
        slope_type=slope_type, smallr=smallr, smallc=smallc, smallp=smallp, smallpp=smallpp,
        gamma6=gamma6, riemann=riemann,
        tEnd=get_float(cfg, "run", "tend", 0.0),
        nStepmax=get_integer(cfg, "run", "nstepmax", 1000),
        problem=problem,
        grav_enabled=get_bool(cfg, "gravity", "enabled", False) and not mhd,
        grav_hancock=get_bool(cfg, "gravity", "hancock_predictor_enabled", False),
        gravity=gravity,
        extra=cfg,
    )


# --------------------------------------------------------------------------
# EKST state files
# --------------------------------------------------------------------------
_HDR = struct.Struct("<8s8qd")


def write_ekst(path: str, U: np.ndarray, dim: int, gw: int, t: float = 0.0,
               iteration: int = 0, dts=()) -> None:
    nb, ks, js, is_ = U.shape
    with open(path, "wb") as f:
        f.write(_HDR.pack(b"EKSTATE1", dim, nb, is_, js, ks, gw, iteration, len(dts), t))
        if len(dts):
            f.write(np.asarray(dts, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(U, dtype="<f8").tobytes())


def read_ekst(path: str):
    b = open(path, "rb").read()
    magic, dim, nb, is_, js, ks, gw, it, ndt, t = _HDR.unpack_from(b, 0)
    if magic != b"EKSTATE1":
        raise ValueError("not an EKST file")
    off = _HDR.size
    dts = np.frombuffer(b, dtype="<f8", count=ndt, offset=off).copy()
    off += 8 * ndt
    U = np.frombuffer(b, dtype="<f8", count=nb * ks * js * is_, offset=off).reshape(nb, ks, js, is_).copy()
    return {"dim": dim, "gw": gw, "iteration": it, "t": t, "dts": dts, "U": U}


def run_reference(ini_text: str, U0: np.ndarray, nsteps: int, workdir: str, fast: bool = False,
                  threads: int | None = None, save: bool = False, gravity_field: np.ndarray | None = None):
    """Run the reference's own solver (oracle/_ref) on an injected state;
    save: also write the final state through the reference's output path
    (save_solution, as the .ini's [output] section configures it);
    gravity_field: (dim, ksize, jsize, isize) array replacing the static
    gravity field of a hydro run with [gravity] enabled."""
    exe = REF_RUN_FAST if fast else REF_RUN
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    workdir = os.path.abspath(workdir)
    os.makedirs(workdir, exist_ok=True)
    ini = os.path.join(workdir, "case.ini")
    u0 = os.path.join(workdir, "u0.ekst")
    out = os.path.join(workdir, "out.ekst")
    with open(ini, "w") as f:
        f.write(ini_text)
    p = params_from_ini(ini_text)
    write_ekst(u0, U0, p.dim, p.gw)
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    if save:
        env["EK_REF_SAVE"] = "1"
    if gravity_field is not None:
        gpath = os.path.join(workdir, "gravity.ekst")
        write_ekst(gpath, gravity_field, p.dim, p.gw)
        env["EK_REF_GRAVITY"] = gpath
    subprocess.run([exe, ini, str(nsteps), out, u0], check=True, cwd=workdir, env=env,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return read_ekst(out)


def run_reference_deck(ini_text: str, nsteps: int, workdir: str):
    """Run the reference's own solver (oracle/_ref) from its own init (no
    injected state); returns the initial state too (EK_REF_DUMP0)."""
    if not os.path.exists(REF_RUN):
        raise FileNotFoundError(REF_RUN)
    workdir = os.path.abspath(workdir)
    os.makedirs(workdir, exist_ok=True)
    ini = os.path.join(workdir, "deck.ini")
    out = os.path.join(workdir, "out.ekst")
    u0 = os.path.join(workdir, "u0.ekst")
    with open(ini, "w") as f:
        f.write(ini_text)
    env = dict(os.environ, EK_REF_DUMP0=u0)
    subprocess.run([REF_RUN, ini, str(nsteps), out], check=True, cwd=workdir, env=env,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    res = read_ekst(out)
    res["U0"] = read_ekst(u0)["U"]
    return res


# --------------------------------------------------------------------------
# C restatement
# --------------------------------------------------------------------------
_lib = None
_ops_lib = None


def _load(path: str):
    if not os.path.exists(path):
        raise FileNotFoundError(path + " (run oracle/build.sh)")
    L = ctypes.CDLL(path)
    L.eko_create.restype = ctypes.c_void_p
    L.eko_create.argtypes = [ctypes.POINTER(eko_params), ctypes.c_void_p, ctypes.c_double]
    L.eko_destroy.argtypes = [ctypes.c_void_p]
    L.eko_next_iteration.argtypes = [ctypes.c_void_p]
    L.eko_finished.argtypes = [ctypes.c_void_p]
    L.eko_get_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.eko_time.argtypes = [ctypes.c_void_p]
    L.eko_time.restype = ctypes.c_double
    L.eko_dt.argtypes = [ctypes.c_void_p]
    L.eko_dt.restype = ctypes.c_double
    L.eko_iteration.argtypes = [ctypes.c_void_p]
    L.eko_set_gravity_field.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.eko_set_gravity_field.restype = ctypes.c_int
    L.eko_num_threads.restype = ctypes.c_int
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = _load(LIB_PATH)
    return _lib


def ops_lib():
    """The op-counting build of the restatement (ek_opcount.cpp)."""
    global _ops_lib
    if _ops_lib is None:
        L = _load(OPS_LIB_PATH)
        L.eko_ops_read.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.eko_ops_read.restype = ctypes.c_int
        _ops_lib = L
    return _ops_lib


class Oracle:
    """One oracle run: create on an injected state, step, read back."""

    def __init__(self, params: Params, U0: np.ndarray, t0: float = 0.0, gravity_field: np.ndarray | None = None,
                 counting: bool = False):
        self.params = params
        self._L = ops_lib() if counting else lib()
        self._cp = params.to_c()
        U0 = np.ascontiguousarray(U0, dtype=np.float64)
        assert U0.shape == params.shape, (U0.shape, params.shape)
        self._h = self._L.eko_create(ctypes.byref(self._cp), U0.ctypes.data, t0)
        if not self._h:
            raise ValueError("oracle does not support this configuration")
        if gravity_field is not None:
            G = np.ascontiguousarray(gravity_field, dtype=np.float64)
            assert G.shape == (params.dim,) + params.shape[1:], G.shape
            if self._L.eko_set_gravity_field(self._h, G.ctypes.data) != 0:
                raise ValueError("gravity is not enabled in these parameters")

    def close(self):
        if self._h:
            self._L.eko_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def next_iteration(self):
        self._L.eko_next_iteration(self._h)

    def finished(self) -> bool:
        return bool(self._L.eko_finished(self._h))

    @property
    def t(self):
        return self._L.eko_time(self._h)

    @property
    def dt(self):
        return self._L.eko_dt(self._h)

    @property
    def iteration(self):
        return self._L.eko_iteration(self._h)

    def state(self) -> np.ndarray:
        U = np.empty(self.params.shape, dtype=np.float64)
        self._L.eko_get_state(self._h, U.ctypes.data)
        return U

    def run(self, nsteps: int):
        dts = []
        for _ in range(nsteps):
            if self.finished():
                break
            self.next_iteration()
            dts.append(self.dt)
        return np.array(dts)


def num_threads() -> int:
    return lib().eko_num_threads()


OP_KINDS = ("add", "mul", "div", "sqrt", "minmax", "abs", "neg", "cmp")


def count_ops(params: Params, U0: np.ndarray, nsteps: int, t0: float = 0.0) -> dict:
    """Floating-point operations of `nsteps` reference steps (implementationVersion 0,
    the compute_dt reduction and boundary fill included) on the injected state U0,
    counted by kind by the op-counting build; "per_cell" divides by the interior
    cell-updates.  The constructor's own compute_dt is not counted."""
    o = Oracle(params, U0, t0, counting=True)
    L = o._L
    L.eko_ops_reset()
    done = 0
    for _ in range(nsteps):
        if o.finished():
            break
        o.next_iteration()
        done += 1
    out = (ctypes.c_ulonglong * len(OP_KINDS))()
    L.eko_ops_read(out, len(OP_KINDS))
    o.close()
    counts = {k: int(out[i]) for i, k in enumerate(OP_KINDS)}
    cells = params.nx * params.ny * (params.nz if params.dim == 3 else 1) * done
    return {"counts": counts, "steps": done, "cell_updates": cells,
            "per_cell": {k: v / cells for k, v in counts.items()}}
