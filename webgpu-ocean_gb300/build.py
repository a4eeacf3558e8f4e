"""Builds libmpm.so in-tree (webgpu-ocean_gb300/build/libmpm.so) with nvcc.

Each .cu file is compiled in parallel for sm_103a only, then linked into one
shared library with the CUDA runtime linked statically.  Flags that the
bit-exact arithmetic depends on:
  -fmad=false, -Xptxas=--fmad=false   no FMA contraction in device code,
                                 also of packed f32x2 multiplies and adds
  -prec-div=true -prec-sqrt=true  IEEE division (the kernels also use
                                 explicitly rounded intrinsics)
  -Xcompiler -ffp-contract=off  no contraction in host code (scene builders)
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
# MPM_BUILD_DIR places a build elsewhere (tuning sweeps build variants side
# by side); MPM_NVCC_DEFINES adds -D flags, e.g. "MPM_G2P_MIN_BLOCKS=4".
BUILD = os.environ.get("MPM_BUILD_DIR") or os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libmpm.so")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")

SOURCES = ["capi.cu", "capi_batch.cu", "capi_adjoint.cu", "kernels_dispatch.cu",
           "kernels_sorted.cu", "profiler.cu", "noalloc.cu", "adjoint.cu", "render.cu", "sph.cu"]
HEADERS = ["mpm_math.cuh", "mpm_math_x2.cuh", "mpm_internal.h", "sorted_engine.h", "adjoint.h",
           "render_math.cuh", "capi_internal.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xptxas=--fmad=false",
              "-prec-div=true",
              "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
              "-I" + INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _inputs_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    paths.append(os.path.join(INCLUDE, "mpm.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile (if stale) and return the path of libmpm.so."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _inputs_mtime():
        return LIB
    cc = nvcc()
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(obj)
        defines = ["-D" + d for d in os.environ.get("MPM_NVCC_DEFINES", "").split() if d]
        cmd = [cc, *ARCH, *NVCC_FLAGS, *defines, "-c", os.path.join(CSRC, src), "-o", obj]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                            text=True)))
    errors = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src}\n{out}")
        elif ptxas_info or verbose:
            print(out, file=sys.stderr)
    if errors:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call([cc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
