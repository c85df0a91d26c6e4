"""GB300-native unsplit MUSCL-Hancock step (hydro 2D/3D, CT-MHD 3D).

Python host layer over the C ABI of ``libek_gb300.so`` (include/ek_gb300.h).
It mirrors the reference's solver interface -- ``SolverFactory.create`` by
solver name, and a solver object with ``compute_dt``, ``next_iteration``,
``finished``, ``m_t``/``m_dt``/``m_iteration`` (shared/SolverBase.h:53-259)
-- so a driver loop reads like the reference's ``src/main.cpp:126-131``:

    params = params_from_ini(open("case.ini").read())
    solver = SolverFactory.create(params.solver_name, params)
    solver.set_state(U0)
    while not solver.finished():
        solver.next_iteration()

There is no CPU fallback: every call goes to the CUDA library, and creating
a solver without a GPU raises ``EkError(EK_ERR_NO_DEVICE)``.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = [
    "EkError",
    "Params",
    "Solver",
    "Ensemble",
    "SolverFactory",
    "params_from_ini",
    "load_library",
    "library_path",
    "EK_PREC_FP64",
    "EK_PREC_MIXED",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
EK_OK, EK_ERR_INVALID, EK_ERR_UNSUPPORTED, EK_ERR_CUDA = 0, 1, 2, 3
EK_ERR_NO_MEMORY, EK_ERR_NONFINITE, EK_ERR_PARSE, EK_ERR_NO_DEVICE = 4, 5, 6, 7
EK_LAYOUT_LEFT, EK_LAYOUT_RIGHT = 0, 1
EK_PREC_FP64, EK_PREC_MIXED = 0, 1


class Params(ctypes.Structure):
    """ctypes mirror of ``ek_params`` (include/ek_gb300.h)."""

    _fields_ = [
        ("dim", ctypes.c_int), ("mhd", ctypes.c_int),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("ghost_width", ctypes.c_int), ("nbvar", ctypes.c_int),
        ("isize", ctypes.c_int), ("jsize", ctypes.c_int), ("ksize", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
        ("ymax", ctypes.c_double), ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("bc", ctypes.c_int * 6),
        ("gamma0", ctypes.c_double), ("gamma6", ctypes.c_double), ("cfl", ctypes.c_double),
        ("slope_type", ctypes.c_double), ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("smallp", ctypes.c_double), ("smallpp", ctypes.c_double), ("cIso", ctypes.c_double),
        ("Omega0", ctypes.c_double),
        ("riemann", ctypes.c_int), ("implementation_version", ctypes.c_int),
        ("nStepmax", ctypes.c_int), ("tEnd", ctypes.c_double), ("tCurrent", ctypes.c_double),
        ("nOutput", ctypes.c_int), ("nlog", ctypes.c_int),
        ("precision", ctypes.c_int), ("exact_fp", ctypes.c_int), ("kchunk", ctypes.c_int),
        ("mhd_stage", ctypes.c_int),
        ("solver_name_", ctypes.c_char * 32), ("problem_", ctypes.c_char * 32),
        ("output_dir_", ctypes.c_char * 256), ("output_prefix_", ctypes.c_char * 128),
        ("vtk_enabled", ctypes.c_int), ("vtk_ascii", ctypes.c_int),
        ("gravity_enabled", ctypes.c_int), ("gravity_static", ctypes.c_int),
        ("gravity_hancock", ctypes.c_int), ("gravity_well_balanced", ctypes.c_int),
        ("gravity", ctypes.c_double * 3),
        ("no_tma", ctypes.c_int),
    ]

    @property
    def output_dir(self) -> str:
        return self.output_dir_.decode()

    @output_dir.setter
    def output_dir(self, v: str):
        self.output_dir_ = v.encode()

    @property
    def output_prefix(self) -> str:
        return self.output_prefix_.decode()

    @output_prefix.setter
    def output_prefix(self, v: str):
        self.output_prefix_ = v.encode()

    @property
    def solver_name(self) -> str:
        return self.solver_name_.decode()

    @property
    def problem(self) -> str:
        return self.problem_.decode()

    @property
    def shape(self):
        """numpy shape of a full state: (nbvar, ksize, jsize, isize)."""
        return (self.nbvar, self.ksize if self.dim == 3 else 1, self.jsize, self.isize)

    def copy(self, **changes) -> "Params":
        p = Params()
        ctypes.memmove(ctypes.byref(p), ctypes.byref(self), ctypes.sizeof(Params))
        for k, v in changes.items():
            setattr(p, k, v)
        return p


class EkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


_lib = None


def library_path() -> str:
    return os.environ.get("EK_GB300_LIB", os.path.join(_HERE, "_build", "libek_gb300.so"))


def load_library():
    """Load libek_gb300.so; it must have been built (python -m euler_kokkos_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise EkError(EK_ERR_UNSUPPORTED, "CUDA library not built: %s (run python -m euler_kokkos_gb300.build)" % path)
    L = ctypes.CDLL(path)
    c_p = ctypes.c_void_p
    sig = {
        "ek_abi_version": (ctypes.c_int, []),
        "ek_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "ek_last_error": (ctypes.c_char_p, []),
        "ek_params_from_ini": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(Params)]),
        "ek_solver_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.POINTER(c_p)]),
        "ek_solver_destroy": (ctypes.c_int, [c_p]),
        "ek_solver_set_state": (ctypes.c_int, [c_p, c_p, ctypes.c_int]),
        "ek_solver_get_state": (ctypes.c_int, [c_p, c_p, ctypes.c_int]),
        "ek_solver_set_gravity_field": (ctypes.c_int, [c_p, c_p, ctypes.c_int]),
        "ek_measure_fma_rate": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
        "ek_selftest_bounded_wait": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                                    ctypes.POINTER(ctypes.c_double)]),
        "ek_solver_compute_dt": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_double)]),
        "ek_solver_next_iteration": (ctypes.c_int, [c_p]),
        "ek_solver_run": (ctypes.c_int, [c_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
        "ek_solver_finished": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_int)]),
        "ek_solver_time": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]),
        "ek_solver_dt_history": (ctypes.c_int, [c_p, c_p, ctypes.c_int]),
        "ek_solver_totals": (ctypes.c_int, [c_p, c_p]),
        "ek_solver_device_state": (ctypes.c_int, [c_p, ctypes.POINTER(c_p), ctypes.POINTER(ctypes.c_size_t)]),
        "ek_solver_synchronize": (ctypes.c_int, [c_p]),
        "ek_solver_launch_count": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_longlong)]),
        "ek_solver_stream": (ctypes.c_int, [c_p, ctypes.POINTER(c_p)]),
        "ek_write_vtk": (ctypes.c_int, [ctypes.POINTER(Params), c_p, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_char_p]),
        "ek_solver_save_vtk": (ctypes.c_int, [c_p, ctypes.c_int, ctypes.c_char_p]),
        "ek_solver_save_restart": (ctypes.c_int, [c_p, ctypes.c_char_p, ctypes.c_int]),
        "ek_solver_load_restart": (ctypes.c_int, [c_p, ctypes.c_char_p, ctypes.c_int,
                                                  ctypes.POINTER(ctypes.c_int)]),
        "ek_solver_set_profiling": (ctypes.c_int, [c_p, ctypes.c_int]),
        "ek_solver_kernel_time": (ctypes.c_int, [c_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                 ctypes.POINTER(ctypes.c_longlong)]),
        "ek_solver_hlld_repairs": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_longlong)]),
        "ek_ensemble_create": (ctypes.c_int, [ctypes.POINTER(Params), ctypes.c_int, ctypes.POINTER(c_p)]),
        "ek_ensemble_destroy": (ctypes.c_int, [c_p]),
        "ek_ensemble_set_state": (ctypes.c_int, [c_p, ctypes.c_int, c_p, ctypes.c_int]),
        "ek_ensemble_get_state": (ctypes.c_int, [c_p, ctypes.c_int, c_p, ctypes.c_int]),
        "ek_ensemble_run": (ctypes.c_int, [c_p, ctypes.c_int, ctypes.c_int]),
        "ek_ensemble_synchronize": (ctypes.c_int, [c_p]),
        "ek_ensemble_time": (ctypes.c_int, [c_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]),
        "ek_ensemble_dt_history": (ctypes.c_int, [c_p, ctypes.c_int, c_p, ctypes.c_int]),
        "ek_ensemble_totals": (ctypes.c_int, [c_p, c_p]),
        "ek_ensemble_info": (ctypes.c_int, [c_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_longlong)]),
        "ek_ensemble_stream": (ctypes.c_int, [c_p, ctypes.POINTER(c_p)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def selftest_bounded_wait(limit_us: int = 2000):
    """Run the step kernels' bounded mbarrier wait on a barrier that never
    completes; returns (expired, elapsed_us): every wait must give up after
    about limit_us and the kernel must return (no hang)."""
    L = load_library()
    expired, elapsed = ctypes.c_int(), ctypes.c_double()
    _check(L.ek_selftest_bounded_wait(int(limit_us), ctypes.byref(expired), ctypes.byref(elapsed)),
           "selftest_bounded_wait")
    return bool(expired.value), elapsed.value


def measure_fma_rate(precision: int) -> float:
    """CUDA-core FMA throughput of the current device in TFLOP/s (2 FLOPs per
    FMA): FP64 for EK_PREC_FP64, FP32 otherwise."""
    L = load_library()
    t = ctypes.c_double()
    _check(L.ek_measure_fma_rate(int(precision), ctypes.byref(t)), "measure_fma_rate")
    return t.value


def _check(status: int, what: str, allow=()):
    if status != EK_OK and status not in allow:
        L = load_library()
        raise EkError(status, "%s: %s (%s)" % (what, L.ek_status_string(status).decode(),
                                               L.ek_last_error().decode()))
    return status


def params_from_ini(text: str, **overrides) -> Params:
    """ConfigMap + HydroParams semantics (C++ front end of the library)."""
    L = load_library()
    p = Params()
    b = text.encode()
    _check(L.ek_params_from_ini(b, len(b), ctypes.byref(p)), "params_from_ini")
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def write_vtk(params: Params, U: np.ndarray, step: int = 0, debug_name: str = "",
              layout: int = EK_LAYOUT_LEFT) -> str:
    """Write a host state as the reference's VTK file (save_VTK_2D/3D,
    IO_VTK.cpp:24-400) into params.output_dir; returns the file name."""
    L = load_library()
    Uc = np.ascontiguousarray(U, dtype=np.float64)
    _check(L.ek_write_vtk(ctypes.byref(params), Uc.ctypes.data, layout, step, debug_name.encode()),
           "write_vtk")
    return vtk_filename(params, step, debug_name)


def vtk_filename(params: Params, step: int = 0, debug_name: str = "") -> str:
    stem = params.output_prefix + ("_" + debug_name if debug_name else "")
    return "%s/%s_%07d.vti" % (params.output_dir or "./", stem, step)


class Solver:
    """One GPU solver: the SolverBase interface over the C ABI."""

    def __init__(self, params: Params):
        L = load_library()
        self._L = L
        self.params = params.copy()
        h = ctypes.c_void_p()
        _check(L.ek_solver_create(ctypes.byref(self.params), ctypes.byref(h)), "ek_solver_create")
        self._h = h
        self.last_status = EK_OK

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.ek_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- state -------------------------------------------------------------
    def set_state(self, U: np.ndarray, layout: int = EK_LAYOUT_LEFT):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.size != int(np.prod(self.params.shape)):
            raise ValueError("state has %d values, expected shape %s" % (U.size, self.params.shape))
        _check(self._L.ek_solver_set_state(self._h, U.ctypes.data, layout), "set_state")

    def get_state(self, layout: int = EK_LAYOUT_LEFT, out: np.ndarray | None = None) -> np.ndarray:
        """Current state: shape (nbvar, ksize, jsize, isize) for LayoutLeft,
        (isize, jsize, ksize, nbvar) for LayoutRight; out: a C-contiguous
        float64 array of that size to fill (e.g. in pinned host memory)."""
        shp = self.params.shape
        if out is None:
            U = np.empty(shp if layout == EK_LAYOUT_LEFT else shp[::-1], dtype=np.float64)
        else:
            if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != int(np.prod(shp)):
                raise ValueError("out must be a C-contiguous float64 array of %d values" % int(np.prod(shp)))
            U = out
        _check(self._L.ek_solver_get_state(self._h, U.ctypes.data, layout), "get_state")
        return U

    def set_gravity_field(self, G, layout: int = EK_LAYOUT_LEFT):
        """Static gravity field (hydro, [gravity] enabled): shape (dim, ksize,
        jsize, isize) for LayoutLeft, (isize, jsize, ksize, dim) for
        LayoutRight; None returns to the uniform params.gravity."""
        if G is None:
            _check(self._L.ek_solver_set_gravity_field(self._h, None, layout), "set_gravity_field")
            return
        G = np.ascontiguousarray(G, dtype=np.float64)
        want = self.params.dim * int(np.prod(self.params.shape[1:]))
        if G.size != want:
            raise ValueError("gravity field has %d values, expected %d" % (G.size, want))
        _check(self._L.ek_solver_set_gravity_field(self._h, G.ctypes.data, layout), "set_gravity_field")

    # -- SolverBase --------------------------------------------------------
    def compute_dt(self) -> float:
        d = ctypes.c_double()
        _check(self._L.ek_solver_compute_dt(self._h, ctypes.byref(d)), "compute_dt")
        return d.value

    def next_iteration(self, allow_nonfinite: bool = False):
        allow = (EK_ERR_NONFINITE,) if allow_nonfinite else ()
        self.last_status = _check(self._L.ek_solver_next_iteration(self._h), "next_iteration", allow)

    def run(self, nsteps: int, allow_nonfinite: bool = False) -> int:
        done = ctypes.c_int()
        allow = (EK_ERR_NONFINITE,) if allow_nonfinite else ()
        self.last_status = _check(self._L.ek_solver_run(self._h, nsteps, ctypes.byref(done)), "run", allow)
        return done.value

    def finished(self) -> bool:
        f = ctypes.c_int()
        _check(self._L.ek_solver_finished(self._h, ctypes.byref(f)), "finished")
        return bool(f.value)

    def _time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _check(self._L.ek_solver_time(self._h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it)), "time")
        return t.value, dt.value, it.value

    @property
    def m_t(self) -> float:
        return self._time()[0]

    @property
    def m_dt(self) -> float:
        return self._time()[1]

    @property
    def m_iteration(self) -> int:
        return self._time()[2]

    def dt_history(self) -> np.ndarray:
        n = self.m_iteration
        out = np.empty(n, dtype=np.float64)
        if n:
            _check(self._L.ek_solver_dt_history(self._h, out.ctypes.data, n), "dt_history")
        return out

    def totals(self) -> np.ndarray:
        out = np.empty(3, dtype=np.float64)
        _check(self._L.ek_solver_totals(self._h, out.ctypes.data), "totals")
        return out

    def save_restart(self, path: str, times_saved: int = 0):
        """Write a restart file of the current state, m_t and the output counter."""
        _check(self._L.ek_solver_save_restart(self._h, path.encode(), times_saved), "save_restart")

    def load_restart(self, path: str, reset_time: bool = False) -> int:
        """init_restart: restore the state and m_t from a restart file, start
        at iteration 0; returns the saved output counter (m_times_saved)."""
        n = ctypes.c_int(0)
        _check(self._L.ek_solver_load_restart(self._h, path.encode(), int(reset_time), ctypes.byref(n)),
               "load_restart")
        return n.value

    def save_vtk(self, step: int = 0, debug_name: str = "") -> str:
        """save_solution with VTK output: the current state in the reference's
        file format; step is the output counter (m_times_saved)."""
        _check(self._L.ek_solver_save_vtk(self._h, step, debug_name.encode()), "save_vtk")
        return vtk_filename(self.params, step, debug_name)

    def device_state(self):
        ptr, nbytes = ctypes.c_void_p(), ctypes.c_size_t()
        _check(self._L.ek_solver_device_state(self._h, ctypes.byref(ptr), ctypes.byref(nbytes)), "device_state")
        return ptr.value, nbytes.value

    def synchronize(self):
        _check(self._L.ek_solver_synchronize(self._h), "synchronize")

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        _check(self._L.ek_solver_launch_count(self._h, ctypes.byref(n)), "launch_count")
        return n.value

    # -- timing ------------------------------------------------------------
    def stream(self) -> int:
        """cudaStream_t of the solver (e.g. for torch.cuda.ExternalStream)."""
        p = ctypes.c_void_p()
        _check(self._L.ek_solver_stream(self._h, ctypes.byref(p)), "stream")
        return p.value or 0

    def set_profiling(self, enable: bool = True):
        _check(self._L.ek_solver_set_profiling(self._h, int(enable)), "set_profiling")

    def kernel_time(self, kernel: int = 0):
        """(total ms, launches) of one step kernel since profiling was enabled."""
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        _check(self._L.ek_solver_kernel_time(self._h, kernel, ctypes.byref(ms), ctypes.byref(n)), "kernel_time")
        return ms.value, n.value

    def hlld_repairs(self) -> int:
        """Tiles recomputed by the mixed HLLD form's repair kernel (faces with
        ill-conditioned FP32 star states solved in FP64) since the state was
        set; 0 for the other forms."""
        n = ctypes.c_longlong()
        _check(self._L.ek_solver_hlld_repairs(self._h, ctypes.byref(n)), "hlld_repairs")
        return n.value


class Ensemble:
    """Independent Hydro_Muscl_2D runs stepped together by one persistent
    kernel per step (optionally replayed from a CUDA graph)."""

    def __init__(self, params_list):
        L = load_library()
        self._L = L
        self.params = [p.copy() for p in params_list]
        arr = (Params * len(self.params))(*self.params)
        h = ctypes.c_void_p()
        _check(L.ek_ensemble_create(arr, len(self.params), ctypes.byref(h)), "ek_ensemble_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.ek_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.params)

    def set_state(self, i: int, U: np.ndarray, layout: int = EK_LAYOUT_LEFT):
        U = np.ascontiguousarray(U, dtype=np.float64)
        if U.size != int(np.prod(self.params[i].shape)):
            raise ValueError("instance %d: state has %d values, expected %s" % (i, U.size, self.params[i].shape))
        _check(self._L.ek_ensemble_set_state(self._h, i, U.ctypes.data, layout), "ensemble set_state")

    def get_state(self, i: int) -> np.ndarray:
        U = np.empty(self.params[i].shape, dtype=np.float64)
        _check(self._L.ek_ensemble_get_state(self._h, i, U.ctypes.data, EK_LAYOUT_LEFT), "ensemble get_state")
        return U

    def run(self, nsteps: int, graph: bool = True):
        _check(self._L.ek_ensemble_run(self._h, nsteps, int(graph)), "ensemble run")

    def synchronize(self):
        _check(self._L.ek_ensemble_synchronize(self._h), "ensemble synchronize")

    def time(self, i: int):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        _check(self._L.ek_ensemble_time(self._h, i, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it)), "time")
        return t.value, dt.value, it.value

    def dt_history(self, i: int) -> np.ndarray:
        n = self.time(i)[2]
        out = np.empty(n, dtype=np.float64)
        if n:
            _check(self._L.ek_ensemble_dt_history(self._h, i, out.ctypes.data, n), "dt_history")
        return out

    def totals(self) -> np.ndarray:
        out = np.empty((len(self.params), 2), dtype=np.float64)
        _check(self._L.ek_ensemble_totals(self._h, out.ctypes.data), "totals")
        return out

    def info(self):
        c, t, g, l = ctypes.c_longlong(), ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
        _check(self._L.ek_ensemble_info(self._h, ctypes.byref(c), ctypes.byref(t), ctypes.byref(g),
                                        ctypes.byref(l)), "info")
        return {"cells": c.value, "tiles": t.value, "grid": g.value, "launches": l.value}

    def stream(self) -> int:
        p = ctypes.c_void_p()
        _check(self._L.ek_ensemble_stream(self._h, ctypes.byref(p)), "stream")
        return p.value or 0


class SolverFactory:
    """Name -> solver registry, as the reference's SolverFactory
    (shared/SolverFactory.h:72-116, SolverFactory.cpp:18-22)."""

    _registry = {
        "Hydro_Muscl_2D": Solver,
        "Hydro_Muscl_3D": Solver,
        "MHD_Muscl_2D": Solver,
        "MHD_Muscl_3D": Solver,
    }

    @classmethod
    def register(cls, name: str, creator):
        cls._registry[name] = creator

    @classmethod
    def names(cls):
        return sorted(cls._registry)

    @classmethod
    def create(cls, name: str, params: Params) -> Solver:
        if name not in cls._registry:
            raise EkError(EK_ERR_INVALID, "%s: is not recognized as a valid application name key. "
                          "Valid solver names are: %s" % (name, ", ".join(cls.names())))
        return cls._registry[name](params)
