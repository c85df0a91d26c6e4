"""Build the CUDA library libek_gb300.so (sm_103a) in-tree.

Translation units (compiled in parallel, one -gencode):
  ek_kernels.cu  x2  -- namespace ek_exact (FP64, --fmad=false: bitwise parity)
                        namespace ek_fast  (FP64 with FMA contraction + mixed FP32)
  ek_capi.cu         -- C ABI host implementation
  ek_config.cpp      -- .ini front end
  ek_noalloc.cu      -- the MHD 3D step on a static device scratch (no allocation)
  ek_io.cpp          -- VTK output in the reference's format
and the driver executable _build/ek_main (ek_main.cpp: the reference's main
loop over the C ABI).
Usage: python -m euler_kokkos_gb300.build   (or build() from Python)
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libek_gb300.so")


def main_path() -> str:
    """The driver executable, beside the library."""
    return os.path.join(os.path.dirname(LIB), "ek_main")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I" + CSRC, "-I" + os.path.join(os.path.dirname(HERE), "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".h", ".cpp")) and f != "ek_main.cpp"]


def _units():
    k = os.path.join(CSRC, "ek_kernels.cu")
    return [
        ("ek_kernels_exact.o", k, ["-DEK_NS=ek_exact", "-DEK_EXACT_ONLY", "--fmad=false"]),
        ("ek_kernels_fast.o", k, ["-DEK_NS=ek_fast", "--fmad=true", "--ftz=true",
                                  "--prec-div=false", "--prec-sqrt=false"]),
        ("ek_capi.o", os.path.join(CSRC, "ek_capi.cu"), []),
        ("ek_config.o", os.path.join(CSRC, "ek_config.cpp"), ["-x", "cu"]),
        ("ek_noalloc.o", os.path.join(CSRC, "ek_noalloc.cu"), []),
        ("ek_io.o", os.path.join(CSRC, "ek_io.cpp"), ["-x", "cu"]),
    ]


def _tuned_flags():
    from euler_kokkos_gb300 import tuning

    return tuning.load_flags()


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(main_path()):
        return False
    if os.path.getmtime(os.path.join(CSRC, "ek_main.cpp")) > os.path.getmtime(main_path()):
        return False
    t = os.path.getmtime(LIB)
    srcs = _sources() + [os.path.join(os.path.dirname(HERE), "include", "ek_gb300.h"), __file__]
    tj = os.path.join(HERE, "tuning.json")
    if os.path.exists(tj):
        srcs.append(tj)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build(force: bool = False, verbose: bool = False, tuned: bool = True) -> str:
    """Compile and link the library; tuned: add the tile shapes and register
    budgets chosen by euler_kokkos_gb300.tuning (tuning.json), if any."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    procs = []
    extra_common = _tuned_flags() if tuned else []
    for obj, src, extra in _units():
        cmd = [nvcc, "-c", src, "-o", os.path.join(BUILD, obj)] + ARCH + COMMON + extra_common + extra
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("CUDA build failed:\n" + msg)
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-o", tmp] + ARCH + [os.path.join(BUILD, o) for o, _, _ in _units()]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    # the driver executable, linked against the library beside it
    cxx = shutil.which("g++") or shutil.which("c++")
    cmd = [cxx, "-O2", "-std=c++17", os.path.join(CSRC, "ek_main.cpp"),
           "-I" + os.path.join(os.path.dirname(HERE), "include"), "-L" + os.path.dirname(LIB), "-lek_gb300",
           "-Wl,-rpath,$ORIGIN", "-o", main_path()]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("ek_main link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
