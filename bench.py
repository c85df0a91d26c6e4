"""Benchmark: Mcell-updates/s of the unsplit MUSCL-Hancock step on one GB300.

Headline workload (the 3D MHD Orszag-Tang configuration, 256^3):
MHD_Muscl_3D, HLLD + constrained transport, slope_type 2, CFL 0.8, periodic
boundaries, seeded 1e-3 noise in v_z.  A "step" is one full time step (CFL
dt, trace, fluxes, emfs, update and CT update) of the whole grid.  ``value``
is the mixed-FP32 form; the FP64 drop-in is measured on the same workload
beside it, and the two forms are compared after the configuration's 100
steps (L1 / L-inf error, dt sequence, max |div B|).  The 3D hydro blast, the
2D implode (FP64), the low-beta MHD blast, 2D MHD Orszag-Tang and the
Kelvin-Helmholtz ensemble are measured under ``workloads``.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the
workload on its own GPU (the path has no exchange between ranks); the
slowest rank's time is used and ``value`` is the sum over ranks.
``--impl reference`` times the reference algorithm's CPU restatement
(oracle/) on the host cores instead (rank 0 only).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s on 1 GB300: mixed-FP32 vs FP64 at stated L1 err; % of HBM BW"
UNIT = "Mcell-updates/s"
PEAKS_FALLBACK = {"hbm_gbs": 6800.0}

# algorithmic bytes per cell-update: one read and one write of U
BYTES_PER_CELL = {
    ("hydro2d", "fp64"): 2 * 4 * 8,
    ("hydro3d", "mixed"): 2 * 5 * 4,
    ("hydro3d", "fp64"): 2 * 5 * 8,
    ("mhd3d", "mixed"): 2 * (5 * 4 + 3 * 8),
    ("mhd3d", "fp64"): 2 * 8 * 8,
    ("mhd2d", "mixed"): 2 * (5 * 4 + 3 * 8),
    ("mhd2d", "fp64"): 2 * 8 * 8,
}

HEADLINE = "3D MHD Orszag-Tang %d^3 on [0,1]^3, MHD_Muscl_3D, HLLD + CT, slope_type 2, CFL 0.8, periodic"

# the kernels of one step: ek_solver_kernel_time ids and names
KERNEL_NAMES = {
    "hydro3d": ((0, "hydro3d_step"),),
    "hydro2d": ((0, "hydro2d_step"),),
    "mhd3d": ((2, "mhd_dt_kernel"), (1, "mhd_trace_kernel"), (0, "mhd_update_kernel"), (3, "mhd_repair_kernel")),
    "mhd2d": ((2, "mhd2d_dt_kernel"), (0, "mhd2d_step_kernel"), (3, "mhd2d_repair_kernel")),
}

# DRAM bytes (read + write) per interior cell of one launch of each kernel,
# from ncu captures of the same kernels on 192^3 / 2048^2 cases (the summaries
# are in profiles/); a launch's traffic on the bench workload is this figure
# times its interior cells (these kernels' traffic grows with the cells).
TRAFFIC_PER_CELL = {
    ("hydro3d", "mixed"): {"hydro3d_step": 38.0},   # 159.0 + 109.9 MB / 7.08 M cells
    ("hydro3d", "fp64"): {"hydro3d_step": 78.2},    # 306.3 + 247.4 MB / 7.08 M cells
    ("mhd3d", "mixed"): {"mhd_dt_kernel": 46.0,      # 323 + 3 MB / 7.08 M cells (first step only)
                         "mhd_trace_kernel": 243.0,  # 375.4 + 1345.0 MB / 7.08 M cells
                         "mhd_update_kernel": 345.8,  # 2125.8 + 321.4 MB / 7.08 M cells
                         # with no tile listed (the Orszag-Tang steps) the
                         # repair kernel reads the list head only
                         "mhd_repair_kernel": 0.0},
    ("mhd2d", "mixed"): {"mhd2d_step_kernel": 78.1,  # 186.4 + 141.0 MB / 4.19 M cells
                         "mhd2d_repair_kernel": 0.0},
}

# Floating-point operations per cell-update of the reference algorithm
# (implementationVersion 0, in its own expression order), counted by kind by
# the op-counting build of the oracle (oracle/ek_opcount.cpp through
# eko.count_ops) over the first two steps of the named case, the CFL
# reduction included.  "flops" = add/sub + mul + div + sqrt, one each;
# "other" = min/max + fabs/copysign + negation + comparison.
FLOPS_PER_CELL = {
    "hydro3d": {"flops": 886.945, "other": 196.479, "counted_on": "3D blast 256^3, HLLC, minmod"},
    "mhd3d": {"flops": 3415.651, "other": 591.732, "counted_on": "3D Orszag-Tang 128^3, HLLD, MC"},
    "mhd2d": {"flops": 1692.266, "other": 308.399, "counted_on": "2D Orszag-Tang 1024^2, HLLD, MC"},
    "hydro2d": {"flops": 469.653, "other": 116.702, "counted_on": "2D Kelvin-Helmholtz 128^2, HLLC, MC"},
}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                for n, v in zip(names, f[5:9]):
                    if v.lower() in ("active", "1"):
                        reasons.add(n)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cells_of(p):
    return p.nx * p.ny * (p.nz if p.dim == 3 else 1)


def ghost_cells_of(p):
    return p.isize * p.jsize * (p.ksize if p.dim == 3 else 1)


def time_device_run(ek, s, steps, sync):
    """K steps on the solver's stream, CUDA events on that stream."""
    import torch

    st = torch.cuda.ExternalStream(s.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sync()
    n0 = s.launch_count()
    e0.record(st)
    done = s.run(steps)
    e1.record(st)
    sync()
    return e0.elapsed_time(e1), done, s.launch_count() - n0


def measure_workload(ek, kind, prec, ini, U0, steps, warmup, sync, profile=True):
    p = ek.params_from_ini(ini, precision=prec)
    with ek.Solver(p) as s:
        s.set_state(U0)
        s.run(warmup)
        s.synchronize()
        ms, done, launches = time_device_run(ek, s, steps, sync)
        out = {"ms": ms, "steps": done, "launches": launches}
        if profile:
            # kernel durations (CUDA events around every launch, same stream)
            s.set_profiling(True)
            s.run(steps)
            s.synchronize()
            k = {i: s.kernel_time(i) for i in range(4)}
            out["kernels"] = {i: (v[0] / v[1] if v[1] else None, v[1]) for i, v in k.items()}
            s.set_profiling(False)
        # tiles the mixed HLLD form's repair kernel recomputed (warm-up, timed
        # and profiled steps)
        out["hlld_repaired_tiles"] = s.hlld_repairs()
        out["U"] = s.get_state()
        out["totals"] = s.totals()
        out["iteration"] = s.m_iteration
    out["cells"] = cells_of(p)
    out["ghost_cells"] = ghost_cells_of(p)
    return out


def divb_inner(U, gw, margin, dx, dy, dz):
    """max |div B| (FP64, on the host) of the cells at least `margin` cells
    inside the interior of a 3D MHD state (face B at the left faces, U[5:8]),
    one z-plane at a time."""
    s = slice(gw + margin, U.shape[3] - gw - margin)
    sp = slice(gw + margin + 1, U.shape[3] - gw - margin + 1)
    out = 0.0
    for k in range(gw + margin, U.shape[1] - gw - margin):
        d = ((U[5, k, s, sp] - U[5, k, s, s]) / dx + (U[6, k, sp, s] - U[6, k, s, s]) / dy +
             (U[7, k + 1, s, s] - U[7, k, s, s]) / dz)
        out = max(out, float(np.abs(d).max()))
    return out


def e2e_measure(ek, prec, ini, U0, steps):
    """Reference-facing loop through the C ABI with host buffers in pinned
    memory: set_state (FP64 host array -> device, converted there), one
    next_iteration per step (the dt read back each step, as the reference's
    reduction does), get_state (device -> FP64 host array)."""
    import torch

    p = ek.params_from_ini(ini, precision=prec)
    h_in = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    h_in[...] = U0
    h_out = torch.empty(U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    with ek.Solver(p) as s:
        s.set_state(h_in)  # warm the paths once (allocation, module load)
        s.next_iteration()
        s.get_state(out=h_out)
        s.synchronize()
        t0 = time.perf_counter()
        s.set_state(h_in)
        for _ in range(steps):
            s.next_iteration()
        s.get_state(out=h_out)
        dt = time.perf_counter() - t0
    cells = cells_of(p)
    return {
        "value": cells * steps / dt / 1e6,
        "unit": UNIT,
        "steps": steps,
        "h2d_bytes_per_step": int(round(h_in.nbytes / steps)),
        "d2h_bytes_per_step": int(round(h_out.nbytes / steps)) + 8,
        "wall_s": dt,
        "path": "ek_solver_set_state + next_iteration x K + ek_solver_get_state (pinned host FP64 arrays%s)" %
                (", converted on the device" if prec == ek.EK_PREC_MIXED else ""),
    }, h_out


def oracle_rate(ini, U0, nsteps):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import eko

    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    t0 = time.perf_counter()
    done = len(o.run(nsteps))
    dt = time.perf_counter() - t0
    o.close()
    return cells_of(p) * done / dt / 1e6, dt, eko.num_threads()


def ensure_oracle():
    lib = os.path.join(ROOT, "oracle", "_build", "libek_oracle.so")
    if not os.path.exists(lib):
        env = dict(os.environ, EK_SKIP_REF="1")
        subprocess.run(["sh", os.path.join(ROOT, "oracle", "build.sh")], check=True, env=env,
                       stdout=subprocess.DEVNULL)


def cpu_sample(make, n_full, label, seconds=15.0, probe_n=48, min_n=64):
    """Oracle on a bounded sample of a workload: make(n, nsteps) -> (ini, U0);
    the workload's own grid when the host can do at least 3 steps of it in
    about `seconds`, else a smaller grid of the same problem, with as many
    steps as fit."""
    ensure_oracle()
    ini, U0 = make(probe_n, 2)
    r, _, _ = oracle_rate(ini, U0, 2)
    n = n_full
    while n > min_n and r * 1e6 * seconds / n ** 3 < 3:
        n //= 2
    steps = max(3, min(50, int(r * 1e6 * seconds / n ** 3)))
    ini, U0 = make(n, steps)
    rate, dt, cores = oracle_rate(ini, U0, steps)
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%s %d^3%s, %d steps (oracle/ek_oracle.c, FP64, OpenMP, %d threads, %.1f s)" %
                      (label, n, "" if n == n_full else " (bounded sample of the %d^3 workload)" % n_full,
                       steps, cores, dt)}


def ensemble_workload(ek, P, args, sync, maxt, world, fp32_tflops=None):
    """The batched Kelvin-Helmholtz ensemble: args.ens_n instances with grids
    from {64,96,128,192,256}^2, own shear / density ratio / dt each, FP32 with
    FP64 totals, one persistent kernel per step replayed from a CUDA graph."""
    import torch

    cases = P.kh_ensemble(n_inst=args.ens_n, nsteps=10 ** 6)
    params = [ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED) for ini, _ in cases]
    with ek.Ensemble(params) as e:
        for i, (_, U0) in enumerate(cases):
            e.set_state(i, U0)
        info = e.info()
        e.run(args.ens_steps, graph=True)  # capture, instantiate and warm up
        e.synchronize()
        st = torch.cuda.ExternalStream(e.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sync()
        l0 = e.info()["launches"]
        e0.record(st)
        e.run(args.ens_steps, graph=True)  # replay
        e1.record(st)
        sync()
        ms = maxt(e0.elapsed_time(e1))
        launches = e.info()["launches"] - l0
        tot = e.totals()
        t_last = [e.time(i)[0] for i in (0, len(cases) // 2, len(cases) - 1)]
    cells = info["cells"]
    value = cells * args.ens_steps / (ms / 1e3) / 1e6 * world
    # CPU reference on a bounded sample: the first instances, a few steps each
    cpu = None
    if not args.no_cpu:
        ensure_oracle()
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import eko

        # every instance, one after another (one problem per run, as the
        # reference), as many steps each as fit in about 10 s
        t0 = time.perf_counter()
        done_cells = 0
        nsamp = 2
        for ini, U0 in cases:
            p = eko.params_from_ini(ini)
            o = eko.Oracle(p, U0)
            done_cells += p.nx * p.ny * len(o.run(nsamp))
            o.close()
        probe = time.perf_counter() - t0
        nsamp = max(2, min(args.ens_steps, int(2 * 10.0 / max(probe, 1e-3))))
        t0 = time.perf_counter()
        done_cells = 0
        for ini, U0 in cases:
            p = eko.params_from_ini(ini)
            o = eko.Oracle(p, U0)
            done_cells += p.nx * p.ny * len(o.run(nsamp))
            o.close()
        dt = time.perf_counter() - t0
        cpu = {"value": done_cells / dt / 1e6, "unit": UNIT, "cores": eko.num_threads(), "kind": "port",
               "sample": "all %d instances x %d steps, one after another (%.1f s)" % (len(cases), nsamp, dt)}
    return {
        "value": value, "unit": UNIT, "dtype": "f32", "instances": len(cases), "interior_cells": cells,
        "steps": args.ens_steps, "ms_per_step": ms / args.ens_steps, "tiles_per_step": info["tiles"],
        "persistent_grid": info["grid"], "gpu_launches": launches, "cuda_graph": True,
        "fp64_total_mass_first": float(tot[0, 0]), "t_end_samples": t_last,
        "cpu_baseline": cpu,
        "flop": None if not fp32_tflops else {
            "per_cell": FLOPS_PER_CELL["hydro2d"]["flops"], "counted_on": FLOPS_PER_CELL["hydro2d"]["counted_on"],
            "achieved_tflops": FLOPS_PER_CELL["hydro2d"]["flops"] * value * 1e6 / 1e12,
            "peak_tflops": fp32_tflops,
            "frac": FLOPS_PER_CELL["hydro2d"]["flops"] * value * 1e6 / 1e12 / fp32_tflops / world},
        "config": "%d x Hydro_Muscl_2D Kelvin-Helmholtz, N in {64,96,128,192,256}^2, shear U[0.2,1], "
                  "density ratio U[1.5,3], periodic x / reflecting y, HLLC, MC, CFL 0.8, own dt" % len(cases),
    }


def run_reference(args):
    """--impl reference: the reference algorithm's CPU restatement (the
    reference's own build cannot be compiled on the GPU host: Kokkos is not
    available offline), all host threads, on the headline workload (3D MHD
    Orszag-Tang) and metric; each step a bounded sample of that workload."""
    from euler_kokkos_gb300 import problems as P

    ensure_oracle()
    n_full = args.n
    # probe the host rate to keep the whole run within a few minutes
    ini, U0 = P.orszag_tang_3d(n=32, nsteps=2)
    r, _, cores = oracle_rate(ini, U0, 2)
    n = n_full
    while n > 64 and (args.steps + args.warmup) * n ** 3 / (r * 1e6) > 150:
        n //= 2
    ini, U0 = P.orszag_tang_3d(n=n, nsteps=args.steps + args.warmup)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import eko

    p = eko.params_from_ini(ini)
    o = eko.Oracle(p, U0)
    o.run(args.warmup)
    t0 = time.perf_counter()
    done = len(o.run(args.steps))
    dt = time.perf_counter() - t0
    o.close()
    cells = p.nx * p.ny * p.nz
    value = cells * done / dt / 1e6
    sample = "3D MHD Orszag-Tang %d^3%s, %d timed steps after %d warm-up, FP64" % (
        n, "" if n == n_full else " (bounded sample of the %d^3 workload)" % n_full, done, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": done, "warmup": args.warmup, "ms_per_step": dt * 1e3 / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 3D MHD Orszag-Tang)",
        "config": {"workload": HEADLINE % n,
                   "engine": "oracle/ek_oracle.c (CPU restatement of the reference step), OpenMP"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="grid of the headline (3D MHD Orszag-Tang) and the 3D blast")
    ap.add_argument("--fp64-steps", type=int, default=20, help="timed steps of the FP64 forms")
    ap.add_argument("--err-steps", type=int, default=100,
                    help="steps after which the mixed form is compared with FP64 (the configuration's run length)")
    ap.add_argument("--side-steps", type=int, default=20, help="timed steps of the mixed side workloads")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-blast", action="store_true")
    ap.add_argument("--no-implode", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-mhd2d", action="store_true")
    ap.add_argument("--mhd2d-n", type=int, default=4096)
    ap.add_argument("--no-mhd-blast", action="store_true")
    ap.add_argument("--mhd-blast-n", type=int, default=512,
                    help="grid of the low-beta MHD blast (512, the configured grid: its FP64 runs take about a minute)")
    ap.add_argument("--mhd-blast-steps", type=int, default=30)
    ap.add_argument("--ens-n", type=int, default=512)
    ap.add_argument("--ens-steps", type=int, default=200)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch

    from euler_kokkos_gb300.replicas import Replicas

    torch.cuda.set_device(local)
    rep = Replicas()
    world = rep.world
    barrier = rep.barrier
    maxt = rep.max

    def sync():
        torch.cuda.synchronize()
        barrier()

    import euler_kokkos_gb300 as ek
    from euler_kokkos_gb300 import problems as P

    peaks, peak_kind = load_peaks()
    hbm = float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]))

    # CUDA-core FMA rates of this GPU (TFLOP/s, 2 FLOPs per FMA), the
    # denominators of the FLOP roofline
    fma_peak = {"mixed": ek.measure_fma_rate(ek.EK_PREC_MIXED), "fp64": ek.measure_fma_rate(ek.EK_PREC_FP64)}

    def rate(meas):
        return meas["cells"] * meas["steps"] / (maxt(meas["ms"]) / 1e3) / 1e6 * world

    def flop_roofline(meas, key):
        """The step against both ceilings: HBM (algorithmic bytes at the measured
        copy rate) and CUDA-core FLOPs (the reference's op count at the FMA rate
        measured above), whole-step time."""
        fl = FLOPS_PER_CELL.get(key[0])
        if not fl or not meas["ms"]:
            return {}
        r = meas["cells"] * meas["steps"] / (meas["ms"] / 1e3)  # cell-updates/s
        peak = fma_peak[key[1]]
        bound_hbm = hbm * 1e9 / BYTES_PER_CELL[key]
        bound_flop = peak * 1e12 / fl["flops"]
        return {"flop": {"per_cell": fl["flops"], "other_fp_ops_per_cell": fl["other"],
                         "counted_on": fl["counted_on"], "achieved_tflops": fl["flops"] * r / 1e12,
                         "peak_tflops": peak, "frac": fl["flops"] * r / 1e12 / peak,
                         "peak_source": "CUDA-core FMA rate measured in this run (%s)" %
                                        ("FP64" if key[1] == "fp64" else "FP32")},
                "bound_gcell_s": {"hbm": bound_hbm / 1e9, "flop": bound_flop / 1e9},
                "frac_of_min_bound": r / min(bound_hbm, bound_flop)}

    def roofline(meas, key):
        """HBM roofline of the whole step (every launch of the step) and, beside
        it, of each kernel: achieved = algorithmic bytes per cell-update x cells
        / device time (CUDA events on the solver's stream); traffic = ncu DRAM
        bytes per cell (profiles/) x cells, per step."""
        cells = meas["cells"]
        ms_step = meas["ms"] / meas["steps"]
        algo = BYTES_PER_CELL[key]
        achieved = algo * cells / (ms_step / 1e3) / 1e9
        names = KERNEL_NAMES[key[0]]
        tr = TRAFFIC_PER_CELL.get(key, {})
        kernels = {}
        ktot = sum(v[0] for v in meas["kernels"].values() if v[0])
        for i, name in names:
            kms, kn = meas["kernels"].get(i, (None, 0))
            if not kms:
                continue
            kernels[name] = {"ms_per_launch": kms, "launches_per_step": kn / meas["steps"],
                             "share": kms / ktot if ktot else None,
                             "traffic_per_cell": tr.get(name)}
        dom = max(kernels, key=lambda k: kernels[k]["ms_per_launch"]) if kernels else None
        # DRAM bytes per step: each kernel's traffic per launch times its
        # launches per step (the CFL kernel of the first step only amortises)
        step_tr = None
        if tr and all(n in tr for n in kernels):
            step_tr = sum(tr[n] * kernels[n]["launches_per_step"] for n in kernels)
        nl = sum(k["launches_per_step"] for k in kernels.values())
        out = {"bound": "hbm", "scope": ("whole step (%.2f launches per step)" % nl) if kernels else "whole step",
               "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
               "traffic": step_tr * cells if step_tr is not None else None,
               "traffic_per_cell": step_tr,
               "algorithmic_bytes_per_cell": algo, "ms_per_step": ms_step, "peak_source": peak_kind,
               "kernels": kernels}
        if dom:
            kms = kernels[dom]["ms_per_launch"]
            ach = algo * cells / (kms / 1e3) / 1e9
            out["dominant_kernel"] = {"name": dom, "achieved": ach, "frac": ach / hbm, "kernel_ms": kms,
                                      "traffic": tr[dom] * cells if dom in tr else None}
        out.update(flop_roofline(meas, key))
        return out

    # --- headline: 3D MHD Orszag-Tang, mixed FP32 vs the FP64 drop-in -------
    n = args.n
    ini, U0 = P.orszag_tang_3d(n=n, nsteps=10 ** 6)
    with ClockSampler(local) as clk:
        mixed = measure_workload(ek, "mhd3d", ek.EK_PREC_MIXED, ini, U0, args.steps, args.warmup, sync)
    clocks = clk.summary()
    mixed.pop("U")
    fp64 = measure_workload(ek, "mhd3d", ek.EK_PREC_FP64, ini, U0, args.fp64_steps, args.warmup, sync)
    fp64.pop("U")
    value, v64 = rate(mixed), rate(fp64)
    ms_mixed = maxt(mixed["ms"])

    # accuracy after the configuration's run length: both forms from U0
    gw = 3
    runs = {}
    for name, prec in (("mixed", ek.EK_PREC_MIXED), ("fp64", ek.EK_PREC_FP64)):
        with ek.Solver(ek.params_from_ini(ini, precision=prec)) as s:
            s.set_state(U0)
            s.run(args.err_steps)
            Uf = s.get_state()
            runs[name] = (Uf[:, gw:-gw, gw:-gw, gw:-gw].copy(), s.dt_history(), s.totals())
            del Uf
    (am, dm, tm), (af, df, tf) = runs["mixed"], runs["fp64"]
    nerr = min(len(dm), len(df))

    def l1(v):
        return float(np.abs(am[v] - af[v]).sum() / np.abs(af[v]).sum())

    def linf(v):
        return float(np.abs(am[v] - af[v]).max() / np.abs(af[v]).max())

    # the magnetic field as a vector: component errors against the field's scale
    bl1 = sum(float(np.abs(am[v] - af[v]).sum()) for v in (5, 6, 7)) / \
        sum(float(np.abs(af[v]).sum()) for v in (5, 6, 7))
    blinf = max(float(np.abs(am[v] - af[v]).max()) for v in (5, 6, 7)) / \
        max(float(np.abs(af[v]).max()) for v in (5, 6, 7))
    accuracy = {
        "after_steps": nerr,
        "l1_rel_err_mixed_vs_fp64": {"rho": l1(0), "E": l1(1), "B": bl1},
        "linf_rel_err_mixed_vs_fp64": {"rho": linf(0), "E": linf(1), "B": blinf},
        "B_note": "B as a vector: sum (max) of |B - B_fp64| over the components over sum (max) of |B_fp64|",
        "max_rel_dt_diff": float(np.abs(dm[:nerr] / df[:nerr] - 1).max()),
        "max_divB": {"mixed": float(tm[2]), "fp64": float(tf[2])},
        "target": "L1 rho <= 1e-5 relative; div B at FP64 round-off",
    }
    del runs, am, af

    workloads = {}

    # --- 3D hydro blast (C2) --------------------------------------------------
    if not args.no_blast:
        ini_b, U0_b = P.blast_3d(n=n, nsteps=10 ** 6)
        bm = measure_workload(ek, "hydro3d", ek.EK_PREC_MIXED, ini_b, U0_b, args.side_steps, 3, sync)
        b64 = measure_workload(ek, "hydro3d", ek.EK_PREC_FP64, ini_b, U0_b, args.fp64_steps, 3, sync)
        with ek.Solver(ek.params_from_ini(ini_b, precision=ek.EK_PREC_FP64)) as s64:
            s64.set_state(U0_b)
            s64.run(bm["iteration"])
            bb = s64.get_state()[0, 2:-2, 2:-2, 2:-2]
        ab = bm["U"][0, 2:-2, 2:-2, 2:-2]
        vb, vb64 = rate(bm), rate(b64)
        e2e_b64 = e2e_measure(ek, ek.EK_PREC_FP64, ini_b, U0_b, args.fp64_steps)[0] if rank == 0 else None
        workloads["hydro_blast_%d" % n] = {
            "value_mixed": vb, "value_fp64": vb64, "unit": UNIT, "mixed_over_fp64": vb / vb64,
            "ms_per_step_mixed": bm["ms"] / bm["steps"], "ms_per_step_fp64": b64["ms"] / b64["steps"],
            "l1_rel_err_rho_mixed_vs_fp64": float(np.abs(ab - bb).sum() / np.abs(bb).sum()),
            "error_after_steps": bm["iteration"],
            "roofline_mixed": roofline(bm, ("hydro3d", "mixed")),
            "roofline_fp64": roofline(b64, ("hydro3d", "fp64")),
            "e2e_fp64": e2e_b64,
            "config": "Hydro_Muscl_3D blast %d^3, HLLC, minmod, CFL 0.7, outflow, 1%% density noise" % n,
        }
        del bm, b64, ab, bb, U0_b

    # --- 2D implode FP64 (C1) -------------------------------------------------
    if not args.no_implode:
        ini_i, U0_i = P.implode_2d(n=256, nsteps=100)
        im = measure_workload(ek, "hydro2d", ek.EK_PREC_FP64, ini_i, U0_i, 100, 3, sync)
        vi = rate(im)
        e2e_i = e2e_measure(ek, ek.EK_PREC_FP64, ini_i, U0_i, 100)[0] if rank == 0 else None
        cpu_i = None
        if rank == 0 and not args.no_cpu:
            ensure_oracle()
            ri, dti, cores = oracle_rate(ini_i, U0_i, 100)
            cpu_i = {"value": ri, "unit": UNIT, "cores": cores, "kind": "port",
                     "sample": "the whole configuration: 2D implode 256^2, 100 steps (%.2f s)" % dti}
        workloads["hydro_implode2d_256"] = {
            "value_fp64": vi, "unit": UNIT, "steps": im["steps"], "ms_per_step_fp64": im["ms"] / im["steps"],
            "roofline_fp64": roofline(im, ("hydro2d", "fp64")),
            "e2e_fp64": e2e_i, "cpu_baseline": cpu_i,
            "config": "Hydro_Muscl_2D implode 256^2, HLLC, minmod, CFL 0.8, reflecting walls, 100 steps, FP64",
        }
        del im

    # --- 3D MHD low-beta blast (C5) -------------------------------------------
    if not args.no_mhd_blast:
        # low-beta MHD blast with a small transverse field (the configured field
        # along x alone makes the reference's HLLD divide 0/0 in the first
        # step); mixed vs FP64 rate, and both forms' states after the
        # configured steps for the error and div B
        nb = args.mhd_blast_n
        ini_b, U0_b = P.mhd_blast_3d(n=nb, nsteps=10 ** 6, by_ratio=0.1)
        mb = measure_workload(ek, "mhd3d", ek.EK_PREC_MIXED, ini_b, U0_b, args.side_steps, 3, sync)
        mb64 = measure_workload(ek, "mhd3d", ek.EK_PREC_FP64, ini_b, U0_b, max(5, args.fp64_steps // 4), 3,
                                sync, profile=False)
        mb.pop("U"), mb64.pop("U")
        res, inner = {}, {}
        pb = ek.params_from_ini(ini_b)
        for name, prec in (("mixed", ek.EK_PREC_MIXED), ("fp64", ek.EK_PREC_FP64)):
            with ek.Solver(ek.params_from_ini(ini_b, precision=prec)) as s:
                s.set_state(U0_b)
                s.run(args.mhd_blast_steps)
                Ub = s.get_state()
                res[name] = (Ub[:2, 3:-3, 3:-3, 3:-3].copy(), s.totals(), s.dt_history())
                inner[name] = divb_inner(Ub, 3, 4, pb.dx, pb.dy, pb.dz)
                if name == "mixed":
                    repaired = s.hlld_repairs()
                del Ub
            sync()
        (ab, totb, dtb), (bb, totb64, dtb64) = res["mixed"], res["fp64"]
        l1b = [float(np.abs(ab[v] - bb[v]).sum() / np.abs(bb[v]).sum()) for v in (0, 1)]
        linfb = [float(np.abs(ab[v] - bb[v]).max() / np.abs(bb[v]).max()) for v in (0, 1)]
        del res, ab, bb, U0_b
        vb, vb64 = rate(mb), rate(mb64)
        workloads["mhd_blast_lowbeta_%d" % nb] = {
            "value_mixed": vb, "value_fp64": vb64, "unit": UNIT, "mixed_over_fp64": vb / vb64,
            "ms_per_step_mixed": mb["ms"] / mb["steps"], "ms_per_step_fp64": mb64["ms"] / mb64["steps"],
            "error_after_steps": len(dtb),
            "l1_rel_err_rho_E_mixed_vs_fp64": l1b, "linf_rel_err_rho_E_mixed_vs_fp64": linfb,
            "max_rel_dt_diff": float(np.abs(dtb / dtb64 - 1).max()),
            "hlld_repaired_tiles": {"error_run": repaired, "timed_runs": mb["hlld_repaired_tiles"],
                                    "note": "tiles recomputed by the repair kernel (faces with ill-conditioned "
                                            "FP32 HLLD star states solved in FP64)"},
            "max_divB_mixed": float(totb[2]), "max_divB_fp64": float(totb64[2]),
            "max_divB_inner_mixed": inner["mixed"], "max_divB_inner_fp64": inner["fp64"],
            "divB_note": "max over all interior cells, and over the cells 4 or more cells inside "
                         "(the outflow fill copies face B like cell values, BoundariesFunctors.h:814-831, "
                         "so the boundary cells hold the rounding size of each form's face-B changes)",
            "roofline_mixed": roofline(mb, ("mhd3d", "mixed")),
            "config": "MHD_Muscl_3D low-beta blast %d^3, B = (10, 1, 0)/sqrt(4 pi), p 0.1 / 10 in r 0.1, "
                      "0.5%% density noise, HLLD + CT, slope_type 2, CFL 0.8, outflow" % nb,
        }
        del mb, mb64

    if not args.no_mhd2d:
        n2 = args.mhd2d_n
        ini_2, U0_2 = P.orszag_tang_2d(n=n2, nsteps=10 ** 6)
        m2 = measure_workload(ek, "mhd2d", ek.EK_PREC_MIXED, ini_2, U0_2, args.side_steps, 3, sync)
        m264 = measure_workload(ek, "mhd2d", ek.EK_PREC_FP64, ini_2, U0_2, max(5, args.fp64_steps // 4), 3, sync)
        a2 = m2["U"][0, 0, 3:-3, 3:-3]
        with ek.Solver(ek.params_from_ini(ini_2, precision=ek.EK_PREC_FP64)) as s64:
            s64.set_state(U0_2)
            s64.run(m2["iteration"])
            b2 = s64.get_state()[0, 0, 3:-3, 3:-3]
        v2, v264 = rate(m2), rate(m264)
        workloads["mhd2d_orszag_tang_%d" % n2] = {
            "value_mixed": v2, "value_fp64": v264, "unit": UNIT, "mixed_over_fp64": v2 / v264,
            "ms_per_step_mixed": m2["ms"] / m2["steps"], "ms_per_step_fp64": m264["ms"] / m264["steps"],
            "l1_rel_err_rho_mixed_vs_fp64": float(np.abs(a2 - b2).sum() / np.abs(b2).sum()),
            "hlld_repaired_tiles": m2["hlld_repaired_tiles"],
            "max_divB_mixed": float(m2["totals"][2]), "max_divB_fp64": float(m264["totals"][2]),
            "roofline_mixed": roofline(m2, ("mhd2d", "mixed")),
            "roofline_fp64": roofline(m264, ("mhd2d", "fp64")),
            "config": "MHD_Muscl_2D Orszag-Tang %d^2, HLLD + CT, slope_type 2, CFL 0.8, periodic" % n2,
        }

    if not args.no_ensemble:
        workloads["kh_ensemble_%d" % args.ens_n] = ensemble_workload(ek, P, args, sync, maxt, world, fma_peak["mixed"])

    line = None
    if rank == 0:
        e2e, _ = e2e_measure(ek, ek.EK_PREC_MIXED, ini, U0, args.steps)
        e2e64, _ = e2e_measure(ek, ek.EK_PREC_FP64, ini, U0, args.fp64_steps)
        cpu = None
        if not args.no_cpu:
            cpu = cpu_sample(lambda m, k: P.orszag_tang_3d(n=m, nsteps=k), n, "3D MHD Orszag-Tang",
                             probe_n=32)
        launches = mixed["launches"]
        line = {
            "metric": METRIC,
            "value": value,
            "unit": UNIT,
            "n_gpus": world,
            "steps": mixed["steps"],
            "warmup": args.warmup,
            "ms_per_step": ms_mixed / mixed["steps"],
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic: seeded 3D MHD Orszag-Tang (rho 25/(36 pi), p 5/(12 pi), v = (-sin 2 pi y, "
                    "sin 2 pi x, 1e-3 splitmix noise), face B from A_z)",
            "config": {
                "workload": (HEADLINE % n) + "; mixed FP32 (FP64 face B and CT update, dt, totals, "
                                             "cancellation islands)",
                "grid": [n] * 3,
                "l2_policy": "no flush: the mixed state (%.0f MB) is larger than the 129 MB L2" %
                             ((5 * 4 + 3 * 8) * mixed["ghost_cells"] / 1e6),
                "parallelism": "replicas" if world > 1 else "single GPU",
                "kernels": [k for _, k in KERNEL_NAMES["mhd3d"]],
            },
            "fp64": {
                "value": v64, "unit": UNIT, "steps": fp64["steps"], "ms_per_step": maxt(fp64["ms"]) / fp64["steps"],
                "roofline": roofline(fp64, ("mhd3d", "fp64")),
                "e2e": e2e64,
                "note": "FP64 drop-in (FMA contraction); FP64 FMA rate of this GPU: %.2f TFLOP/s" % fma_peak["fp64"],
            },
            "mixed_over_fp64": value / v64,
            "accuracy": accuracy,
            "hlld_repaired_tiles": mixed["hlld_repaired_tiles"],
            "roofline": roofline(mixed, ("mhd3d", "mixed")),
            "reference_formula_mcell_s": mixed["ghost_cells"] * mixed["steps"] / (ms_mixed / 1e3) / 1e6 * world,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
            "workloads": workloads,
        }
    barrier()
    if line is not None:
        print(json.dumps(line), flush=True)
    rep.close()


if __name__ == "__main__":
    main()
