"""ek_mhd3d_step_noalloc: the MHD_Muscl_3D step on a static device scratch.

The entry point allocates no device memory, for host codes that keep every
byte of device memory in their own pool and cannot hand the library a trace
buffer: its compact-trace temporary lives in a fixed-size file-scope device
array.  The GPU tests call it through the C ABI on caller-owned device arrays
(allocated here with torch, as a host code's own pool would):
* two calls in a row against two steps of the solver entry point
  (ek_solver_next_iteration) from the same state.  Both run the same kernels,
  so the interiors and the time steps agree to the last bit; the tolerance is
  written as 0 for the bitwise build and 1e-13 relative for the FMA build;
* two calls in a row of the bitwise build against two steps of the oracle
  (the reference algorithm's CPU restatement): equal bit for bit;
* a non-finite dt of an asynchronous call (no dt pointer) is reported by the
  next call that asks for its dt.
The input's ghost cells are filled with NaN: the step maps ghost positions to
interior cells through the boundary conditions and never reads them.

The CPU tests check the host-side rejections, which happen before any device
call.  This module is collected last so that it runs both alone and after the
other GPU tests in one process.
"""

import ctypes

import numpy as np
import pytest

import eko
import euler_kokkos_gb300 as ek
from euler_kokkos_gb300 import problems as P
from helpers import interior, load_golden

EK_OK, EK_ERR_INVALID, EK_ERR_UNSUPPORTED = 0, 1, 2
EK_ERR_NONFINITE = ek.EK_ERR_NONFINITE
SCRATCH_BYTES = 64 << 20
TOL = {1: 0.0, 0: 1e-13}


def _lib():
    L = ek.load_library()
    f = L.ek_mhd3d_step_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ek.Params), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                  ctypes.POINTER(ctypes.c_double), ctypes.c_void_p]
    return L


def _step_noalloc(L, p, a, b, t):
    dt = ctypes.c_double(0.0)
    st = L.ek_mhd3d_step_noalloc(ctypes.byref(p), ctypes.c_void_p(a), ctypes.c_void_p(b), t,
                                 ctypes.byref(dt), None)
    assert st == EK_OK, L.ek_last_error().decode()
    return dt.value


def _decks():
    return {
        "orszag_tang_16": P.orszag_tang_3d(n=16, nsteps=2),
        "random_mixedbc_20x14x9": P.smooth_random(dim=3, mhd=True, nx=20, ny=14, nz=9, seed=7,
                                                  bc=(1, 2, 3, 3, 2, 1), nsteps=2),
    }


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [1, 0])
@pytest.mark.parametrize("deck", sorted(_decks()))
def test_two_noalloc_steps_match_solver_steps(deck, exact):
    import torch

    ini, U0 = _decks()[deck]
    p = ek.params_from_ini(ini, exact_fp=exact)
    gw = p.ghost_width

    # solver entry point: two steps from U0
    with ek.SolverFactory.create(p.solver_name, p) as s:
        s.set_state(U0)
        s.next_iteration()
        U1, t1 = s.get_state(), s.m_t
        s.next_iteration()
        U2 = s.get_state()
        dts = s.dt_history()

    # no-alloc entry point: caller-owned device arrays, ghosts of the input NaN
    L = _lib()
    h = np.full_like(U0, np.nan)
    h[:, gw:-gw, gw:-gw, gw:-gw] = U0[:, gw:-gw, gw:-gw, gw:-gw]
    torch.cuda.set_device(0)
    A = torch.from_numpy(h).to("cuda")
    B = torch.zeros_like(A)
    torch.cuda.synchronize()
    dt0 = _step_noalloc(L, p, A.data_ptr(), B.data_ptr(), 0.0)
    V1 = B.cpu().numpy()
    dt1 = _step_noalloc(L, p, B.data_ptr(), A.data_ptr(), 0.0 + dt0)
    V2 = A.cpu().numpy()

    tol = TOL[exact]
    assert abs(dt0 - dts[0]) <= tol * dts[0] and abs(dt1 - dts[1]) <= tol * dts[1], (dt0, dt1, dts)
    assert abs((0.0 + dt0) - t1) <= tol * t1
    for mine, ref in ((V1, U1), (V2, U2)):
        a, b = interior(mine, gw, 3), interior(ref, gw, 3)
        assert np.all(np.isfinite(a))
        err = np.max(np.abs(a - b)) / np.max(np.abs(b))
        assert err <= tol, err


def _device_state(U0, gw):
    import torch

    h = np.full_like(U0, np.nan)
    h[:, gw:-gw, gw:-gw, gw:-gw] = U0[:, gw:-gw, gw:-gw, gw:-gw]
    torch.cuda.set_device(0)
    A = torch.from_numpy(h).to("cuda")
    B = torch.zeros_like(A)
    torch.cuda.synchronize()
    return A, B


@pytest.mark.gpu
@pytest.mark.parametrize("deck", sorted(_decks()))
def test_two_noalloc_steps_match_the_oracle_bitwise(deck):
    ini, U0 = _decks()[deck]
    p = ek.params_from_ini(ini, exact_fp=1)
    gw = p.ghost_width
    o = eko.Oracle(eko.params_from_ini(ini), U0)
    o.next_iteration()
    O1, odt0 = o.state(), o.dt
    o.next_iteration()
    O2, odt1 = o.state(), o.dt
    o.close()

    L = _lib()
    A, B = _device_state(U0, gw)
    dt0 = _step_noalloc(L, p, A.data_ptr(), B.data_ptr(), 0.0)
    V1 = B.cpu().numpy()
    dt1 = _step_noalloc(L, p, B.data_ptr(), A.data_ptr(), 0.0 + dt0)
    V2 = A.cpu().numpy()
    assert dt0 == odt0 and dt1 == odt1, (dt0, dt1, odt0, odt1)
    assert np.array_equal(interior(V1, gw, 3), interior(O1, gw, 3))
    assert np.array_equal(interior(V2, gw, 3), interior(O2, gw, 3))


@pytest.mark.gpu
def test_asynchronous_nonfinite_dt_is_reported_by_the_next_synchronous_call():
    # the reference's low-beta MHD blast divides 0/0 in its first step: the
    # third step's dt is not positive (fixture written by the reference)
    g = load_golden("mhdblast3d_10_nan")
    assert not (g["dts"][2] > 0)
    p = ek.params_from_ini(str(g["ini"]), exact_fp=1)
    L = _lib()
    A, B = _device_state(g["U0"], p.ghost_width)
    C = A.clone()
    dt0 = _step_noalloc(L, p, A.data_ptr(), B.data_ptr(), 0.0)  # finite, synchronous
    assert dt0 == g["dts"][0]
    f = L.ek_mhd3d_step_noalloc
    # two asynchronous steps; the second one's dt is not positive
    assert f(ctypes.byref(p), ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(C.data_ptr()), dt0, None, None) == EK_OK
    assert f(ctypes.byref(p), ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(A.data_ptr()), 0.0, None, None) == EK_OK
    dt = ctypes.c_double(0.0)
    st = f(ctypes.byref(p), ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()), 0.0, ctypes.byref(dt), None)
    assert st == EK_ERR_NONFINITE and "earlier call" in L.ek_last_error().decode()
    # reported once: the next synchronous call reports only its own step
    st = f(ctypes.byref(p), ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(A.data_ptr()), 0.0, ctypes.byref(dt), None)
    assert st == EK_ERR_NONFINITE and "not finite and positive" in L.ek_last_error().decode()
    # a finite step afterwards is clean
    A2, B2 = _device_state(g["U0"], p.ghost_width)
    assert _step_noalloc(L, p, A2.data_ptr(), B2.data_ptr(), 0.0) == dt0


def _trace_bytes(p):
    # 48 FP64 values per trace cell (47 and a spare); trace cells: 32-cell
    # blocks along x
    return 48 * 8 * 32 * ((p.nx + 2 + 31) // 32) * (p.ny + 2) * (p.nz + 2)


def test_rejects_grid_beyond_the_static_scratch():
    L = _lib()
    ini, _ = P.smooth_random(dim=3, mhd=True, nx=51, ny=51, nz=51, seed=1, nsteps=1)
    p = ek.params_from_ini(ini)
    assert _trace_bytes(p) > SCRATCH_BYTES - 512
    # the size check comes before any device call; the pointers are never used
    st = L.ek_mhd3d_step_noalloc(ctypes.byref(p), ctypes.c_void_p(1 << 40), ctypes.c_void_p(1 << 41), 0.0,
                                 None, None)
    assert st == EK_ERR_INVALID
    assert "static scratch" in L.ek_last_error().decode()
    # a 50^3 interior fits: the call passes the size check (and fails only
    # later where there is no GPU)
    ini, _ = P.smooth_random(dim=3, mhd=True, nx=50, ny=50, nz=50, seed=1, nsteps=1)
    q = ek.params_from_ini(ini)
    assert _trace_bytes(q) <= SCRATCH_BYTES - 512
    if not __import__("conftest").gpu_available():
        st = L.ek_mhd3d_step_noalloc(ctypes.byref(q), ctypes.c_void_p(1 << 40), ctypes.c_void_p(1 << 41), 0.0,
                                     None, None)
        assert st != EK_ERR_INVALID, L.ek_last_error().decode()


def test_rejects_bad_calls_before_any_device_work():
    L = _lib()
    ini, _ = P.orszag_tang_3d(n=16, nsteps=1)
    p = ek.params_from_ini(ini)
    a, b = ctypes.c_void_p(1 << 40), ctypes.c_void_p(1 << 41)
    cases = [
        (p.copy(precision=1), a, b, 0.0, EK_ERR_UNSUPPORTED),        # FP64 arrays only
        (p, a, a, 0.0, EK_ERR_INVALID),                               # in place
        (p, a, ctypes.c_void_p((1 << 40) + 4096), 0.0, EK_ERR_INVALID),  # overlapping
        (p, a, b, 2e30, EK_ERR_INVALID),                              # t >= tEnd
        (p, None, b, 0.0, EK_ERR_INVALID),                            # null input
    ]
    for q, x, y, t, want in cases:
        assert L.ek_mhd3d_step_noalloc(ctypes.byref(q), x, y, t, None, None) == want
    hydro_ini, _ = P.smooth_random(dim=3, mhd=False, nx=8, seed=1, nsteps=1)
    q = ek.params_from_ini(hydro_ini)
    assert L.ek_mhd3d_step_noalloc(ctypes.byref(q), a, b, 0.0, None, None) == EK_ERR_UNSUPPORTED
