"""Build libcfd2d_gpu.so (and the cfd2d_gpu executable) in-tree for sm_103a.

Host C++ is compiled with g++ and -ffp-contract=off (mesh geometry and region
states must round like the reference's build on x86-64 and AArch64 alike);
device code with nvcc -gencode arch=compute_103a,code=sm_103a. The FP64 kernels
are compiled with -fmad=false, the mixed-precision kernels with FMA.

    python cfd-2d_gb300/build.py [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libcfd2d_gpu.so")
EXE = os.path.join(LIB_DIR, "cfd2d_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


HOST_SOURCES = ["xml.cpp", "mesh.cpp", "task.cpp", "solver.cpp", "solver_adjoint.cpp", "solver_batch.cpp",
                "solver_tiles.cpp", "implicit.cpp", "rkdg.cpp", "capi.cpp"]
# -fmad per translation unit: "false" for the bit-exact FP64 path, "true" for the mixed form
# (with fast math), "fma" for FMA contraction with IEEE division and square root
DEVICE_SOURCES = {"kern_fp64.cu": "false", "kern_common.cu": "false", "kern_mixed.cu": "true",
                  "noalloc.cu": "false", "adjoint.cu": "false", "adjoint_mixed.cu": "true",
                  "implicit.cu": "false", "gmres.cu": "fma", "rkdg.cu": "false"}
HEADERS = ["xml.hpp", "mesh.hpp", "task.hpp", "solver.hpp", "kernels.hpp", "kernels.cuh", "kern_inst.cuh",
           "adjoint.cuh", "adj_inst.cuh", "implicit.hpp", "rkdg.hpp"]


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    ch = cuda_home()
    nvcc = os.path.join(ch, "bin", "nvcc")
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INC, "cfd2d.h")]
    jobs = []
    objs = []
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, s)
        out = os.path.join(OBJ, s + ".o")
        objs.append(out)
        if force or _stale(out, [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", INC, "-I", CSRC, "-I", os.path.join(ch, "include"), "-c", src, "-o", out])
    for s, fmad in DEVICE_SOURCES.items():
        src = os.path.join(CSRC, s)
        out = os.path.join(OBJ, s + ".o")
        objs.append(out)
        if force or _stale(out, [src] + hdrs):
            extra = ["-use_fast_math"] if fmad == "true" else []
            fm = "true" if fmad == "fma" else fmad
            jobs.append([nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", f"-fmad={fm}", *extra, "-Xptxas", "-v",
                         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", INC, "-I", CSRC,
                         "-c", src, "-o", out])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for out in ex.map(lambda c: _run(c, verbose), jobs):
            logs.append(out)
    if jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lcudart", "-ldl"], verbose)
    main_src = os.path.join(CSRC, "main.cpp")
    if os.path.exists(main_src) and (force or _stale(EXE, [main_src, LIB])):
        _run(["g++", "-std=c++17", "-O2", "-I", INC, main_src, "-o", EXE, "-L", LIB_DIR, "-lcfd2d_gpu",
              f"-Wl,-rpath,$ORIGIN"], verbose)
    with open(os.path.join(OBJ, "ptxas.log"), "a") as f:
        for s in logs:
            f.write(s)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
