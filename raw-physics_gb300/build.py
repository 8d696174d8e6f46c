"""Build the GB300 extension in place: raw-physics_gb300/librawphys_gb300.so.

Eleven translation units, compiled in parallel:
  csrc/rp_kernels_f32.cu   FP32 build of the persistent step kernels (nvcc, sm_103a)
  csrc/rp_kernels_f64.cu   all-FP64 build, no FMA contraction        (nvcc, sm_103a, -fmad=false)
  csrc/rp_pipe_f32.cu      FP32 build of the phase-major kernels     (nvcc, sm_103a)
  csrc/rp_pipe_f64.cu      all-FP64 phase-major kernels              (nvcc, sm_103a, -fmad=false)
  csrc/rp_noalloc.cu       static device scratch of the no-allocation contact query (nvcc)
  csrc/rp_adjoint.cu       adjoint of the substep                    (nvcc, sm_103a, -fmad=false)
  csrc/rp_host.cpp         runtime + C ABI (include/rp.h)            (host compiler)
  csrc/rp_hull.cpp         hull topology and mass properties        (host compiler)
  csrc/rp_hull_io.cpp      OBJ input and the binary hull cache       (host compiler)
  csrc/rp_shim.cpp         C++-mangled pbd_simulate drop-in          (host compiler)
Host code is compiled with -ffp-contract=off so the set-up arithmetic keeps the reference's FP64
rounding on both x86-64 and aarch64.

    python raw-physics_gb300/build.py [--force]
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librawphys_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDE = ["-I" + os.path.join(HERE, "..", "include"), "-I" + CSRC, "-I" + os.path.join(CUDA_HOME, "include")]

HEADERS = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + [
    os.path.join(HERE, "..", "include", "rp.h"), os.path.join(HERE, "..", "include", "rp_compat.h")]


def _units():
    cu_common = [NVCC, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                 "--diag-suppress=1444", *INCLUDE]
    cxx = ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", *INCLUDE]
    return [
        ("rp_kernels_f32.cu", cu_common),
        ("rp_kernels_f64.cu", cu_common + ["-fmad=false"]),
        ("rp_pipe_f32.cu", cu_common),
        ("rp_pipe_f64.cu", cu_common + ["-fmad=false"]),
        ("rp_noalloc.cu", cu_common),
        ("rp_adjoint.cu", cu_common + ["-fmad=false"]),
        ("rp_host.cpp", cxx),
        ("rp_hull.cpp", cxx),
        ("rp_hull_io.cpp", cxx),
        ("rp_shim.cpp", cxx),
    ]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.exists(s) and os.path.getmtime(s) > t for s in sources)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    jobs, objs = [], []
    for src, cmd in _units():
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + HEADERS):
            jobs.append(cmd + ["-c", path, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if jobs or _stale(LIB, objs):
        run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
