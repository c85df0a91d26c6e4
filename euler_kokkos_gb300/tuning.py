"""Tuning of the step kernels: tile shapes, resident CTAs per SM, planes per
CTA column.

The tile shapes and register budgets are compile-time parameters of the CUDA
kernels (EK_*_TX/TY and EK_*_MINB_* in csrc/ek_common.cuh); the planes per CTA
column of the 3D kernels is a run-time parameter.  ``python -m
euler_kokkos_gb300.tuning`` builds the library once per candidate set into
``_build/tune/<i>/``, times every kernel family on its workload through the C
ABI (CUDA events around each launch: ek_solver_set_profiling /
ek_solver_kernel_time), keeps the fastest candidate of each family and writes
the choice to ``tuning.json`` beside this file, which build() turns into -D
flags.  The workloads are the benchmark's sizes (3D blast and Orszag-Tang
256^3, 2D Orszag-Tang 4096^2, the 512-instance Kelvin-Helmholtz ensemble):
the best tile depends on the grid.  The objective is the mixed-precision (FP32) kernel time, the
performance form; the FP64 build uses the same shapes.  Run it on the GPU it
tunes for; it needs nvcc and a few minutes.
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING_FILE = os.path.join(HERE, "tuning.json")

# Candidate sets per kernel family; candidate 0 is the built-in default.
CANDIDATES = {
    "hydro2d": [{"EK_H2_TX": "32", "EK_H2_TY": "8"}, {"EK_H2_TX": "32", "EK_H2_TY": "4"}, {"EK_H2_TX": "64", "EK_H2_TY": "4"},
                {"EK_H2_TX": "16", "EK_H2_TY": "16"}, {"EK_H2_TX": "64", "EK_H2_TY": "8"},
                {"EK_H2_TX": "16", "EK_H2_TY": "8"}, {"EK_H2_TX": "32", "EK_H2_TY": "16"}],
    "hydro3d": [{"EK_H3_TX": "32", "EK_H3_TY": "8", "EK_H3_MINB_F32": "4", "EK_H3_MINB_F64": "2"},
                {"EK_H3_TX": "32", "EK_H3_TY": "4", "EK_H3_MINB_F32": "8", "EK_H3_MINB_F64": "4"},
                {"EK_H3_TX": "64", "EK_H3_TY": "4", "EK_H3_MINB_F32": "4", "EK_H3_MINB_F64": "2"},
                {"EK_H3_TX": "16", "EK_H3_TY": "16", "EK_H3_MINB_F32": "4", "EK_H3_MINB_F64": "2"},
                {"EK_H3_TX": "32", "EK_H3_TY": "16", "EK_H3_MINB_F32": "2", "EK_H3_MINB_F64": "1"},
                {"EK_H3_TX": "16", "EK_H3_TY": "16", "EK_H3_MINB_F32": "3", "EK_H3_MINB_F64": "2"},
                {"EK_H3_TX": "16", "EK_H3_TY": "8", "EK_H3_MINB_F32": "8", "EK_H3_MINB_F64": "4"}],
    "mhd_trace": [{"EK_MT_TX": "32", "EK_MT_TY": "4"}, {"EK_MT_TX": "16", "EK_MT_TY": "8"}, {"EK_MT_TX": "32", "EK_MT_TY": "8"},
                  {"EK_MT_TX": "64", "EK_MT_TY": "2"}, {"EK_MT_TX": "16", "EK_MT_TY": "4"},
                  {"EK_MT_TX": "32", "EK_MT_TY": "4", "EK_MT_MINB_F32": "6"}, {"EK_MT_TX": "64", "EK_MT_TY": "4"}],
    "mhd_update": [{"EK_MU_TX": "32", "EK_MU_TY": "8", "EK_MU_MINB_F32": "4"},
                   {"EK_MU_TX": "32", "EK_MU_TY": "4", "EK_MU_MINB_F32": "8"},
                   {"EK_MU_TX": "16", "EK_MU_TY": "8", "EK_MU_MINB_F32": "8"},
                   {"EK_MU_TX": "64", "EK_MU_TY": "4", "EK_MU_MINB_F32": "4"},
                   {"EK_MU_TX": "32", "EK_MU_TY": "16", "EK_MU_MINB_F32": "2"},
                   {"EK_MU_TX": "16", "EK_MU_TY": "16", "EK_MU_MINB_F32": "4"},
                   {"EK_MU_TX": "32", "EK_MU_TY": "8", "EK_MU_MINB_F32": "3"}],
    "mhd2d": [{"EK_M2_TX": "16", "EK_M2_TY": "8"}, {"EK_M2_TX": "32", "EK_M2_TY": "8"}, {"EK_M2_TX": "16", "EK_M2_TY": "16"},
              {"EK_M2_TX": "32", "EK_M2_TY": "4"}, {"EK_M2_TX": "8", "EK_M2_TY": "8"},
              {"EK_M2_TX": "16", "EK_M2_TY": "16", "EK_M2_MINB_F32": "3"},
              {"EK_M2_TX": "16", "EK_M2_TY": "16", "EK_M2_MINB_F32": "4"}],
}
KCHUNKS = (16, 32, 64)


def load_flags():
    """-D flags of the tuned configuration (empty when there is none)."""
    if not os.path.exists(TUNING_FILE):
        return []
    with open(TUNING_FILE) as f:
        cfg = json.load(f)
    flags = ["-D%s=%s" % (k, v) for k, v in sorted(cfg.get("flags", {}).items())]
    if cfg.get("kchunk"):
        flags.append("-DEK_KCHUNK_DEFAULT=%d" % int(cfg["kchunk"]))
    return flags


# ---------------------------------------------------------------------------
# measurement (runs in a child process against one built variant)
# ---------------------------------------------------------------------------
def _kernel_ms(ek, ini, U0, kernels, steps, **over):
    p = ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED, **over)
    with ek.Solver(p) as s:
        s.set_state(U0)
        s.run(3)
        s.synchronize()
        s.set_profiling(True)
        s.run(steps)
        s.synchronize()
        out = {}
        for name, kid in kernels:
            total, n = s.kernel_time(kid)
            out[name] = total / n if n else None
    return out


def _ensemble_ms(ek, P, steps=50):
    import time

    cases = P.kh_ensemble(n_inst=512, nsteps=10 ** 6)
    params = [ek.params_from_ini(ini, precision=ek.EK_PREC_MIXED) for ini, _ in cases]
    with ek.Ensemble(params) as e:
        for i, (_, U0) in enumerate(cases):
            e.set_state(i, U0)
        e.run(steps, graph=True)  # capture and warm up
        e.synchronize()
        t0 = time.perf_counter()
        e.run(steps, graph=True)
        e.synchronize()
        return (time.perf_counter() - t0) * 1e3 / steps


def measure(families):
    import euler_kokkos_gb300 as ek
    from euler_kokkos_gb300 import problems as P

    res = {}
    if "hydro2d" in families:
        # the 2D tile serves the single solver and the ensemble; the batched
        # Kelvin-Helmholtz ensemble is the benchmark that uses it
        res["hydro2d"] = _ensemble_ms(ek, P)
    if "hydro3d" in families:
        ini, U0 = P.blast_3d(n=256, nsteps=10 ** 6)
        res["hydro3d"] = {str(k): _kernel_ms(ek, ini, U0, [("step", 0)], 8, kchunk=k)["step"] for k in KCHUNKS}
    if "mhd_trace" in families or "mhd_update" in families:
        ini, U0 = P.orszag_tang_3d(n=256, nsteps=10 ** 6)
        r = {str(k): _kernel_ms(ek, ini, U0, [("update", 0), ("trace", 1)], 4, kchunk=k) for k in KCHUNKS}
        res["mhd_trace"] = {k: v["trace"] for k, v in r.items()}
        res["mhd_update"] = {k: v["update"] for k, v in r.items()}
    if "mhd2d" in families:
        ini, U0 = P.orszag_tang_2d(n=4096, nsteps=10 ** 6)
        res["mhd2d"] = _kernel_ms(ek, ini, U0, [("step", 0)], 6)["step"]
    return res


# ---------------------------------------------------------------------------
# driver
# ---------------------------------------------------------------------------
def _build_variant(idx, cfg):
    from euler_kokkos_gb300 import build as B

    d = os.path.join(HERE, "_build", "tune", str(idx))
    os.makedirs(d, exist_ok=True)
    flags = []
    for fam in cfg.values():
        flags += ["-D%s=%s" % (k, v) for k, v in fam.items()]
    cmd = [sys.executable, "-c",
           "import sys; sys.path.insert(0, %r); import euler_kokkos_gb300.build as B; "
           "B.BUILD = %r; B.LIB = %r; B.COMMON = B.COMMON + %r; B.build(force=True, tuned=False)"
           % (os.path.dirname(HERE), d, os.path.join(d, "libek_gb300.so"), flags)]
    return subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), os.path.join(d, "libek_gb300.so")


def tune(parallel_builds=3):
    nvar = max(len(c) for c in CANDIDATES.values())
    cfgs = [{fam: c[min(i, len(c) - 1)] for fam, c in CANDIDATES.items()} for i in range(nvar)]
    libs = [None] * nvar
    for start in range(0, nvar, parallel_builds):
        procs = [(i, *_build_variant(i, cfgs[i])) for i in range(start, min(nvar, start + parallel_builds))]
        for i, p, lib in procs:
            out, _ = p.communicate()
            if p.returncode != 0:
                raise RuntimeError("variant %d failed to build:\n%s" % (i, out.decode(errors="replace")))
            libs[i] = lib
    results = []
    for i, lib in enumerate(libs):
        fams = [f for f in CANDIDATES if i < len(CANDIDATES[f])]
        env = dict(os.environ, EK_GB300_LIB=lib)
        r = subprocess.run([sys.executable, "-m", "euler_kokkos_gb300.tuning", "--measure", ",".join(fams)],
                           cwd=os.path.dirname(HERE), env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("variant %d failed to run:\n%s" % (i, r.stdout.decode(errors="replace")))
        results.append(json.loads(r.stdout.decode().strip().splitlines()[-1]))
        print("variant", i, json.dumps(results[-1]), flush=True)
    # best candidate per family; the 3D families also pick the planes per column
    flags, chosen, kchunk_score = {}, {}, {k: 0.0 for k in KCHUNKS}
    for fam, cands in CANDIDATES.items():
        best = None
        for i in range(len(cands)):
            v = results[i][fam]
            t = min(x for x in v.values() if x) if isinstance(v, dict) else v
            if t and (best is None or t < best[0]):
                best = (t, i)
        chosen[fam] = {"candidate": best[1], "ms": best[0], "flags": cands[best[1]],
                       "all_ms": [results[i][fam] for i in range(len(cands))]}
        flags.update(cands[best[1]])
        v = results[best[1]][fam]
        if isinstance(v, dict):
            for k in KCHUNKS:
                kchunk_score[k] += v[str(k)] or 1e30
    kchunk = min(KCHUNKS, key=lambda k: kchunk_score[k])
    cfg = {"flags": flags, "kchunk": kchunk, "families": chosen,
           "tuned_on": _gpu_name(), "date": time.strftime("%Y-%m-%d")}
    with open(TUNING_FILE, "w") as f:
        json.dump(cfg, f, indent=1, sort_keys=True)
    return cfg


def _gpu_name():
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--measure":
        sys.path.insert(0, os.path.dirname(HERE))
        print(json.dumps(measure(sys.argv[2].split(","))))
    else:
        cfg = tune()
        print(json.dumps({k: v for k, v in cfg.items() if k != "families"}, indent=1))
