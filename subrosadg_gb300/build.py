"""In-tree build of the GB300 DG library for sm_103a.

    python -m subrosadg_gb300.build [--force] [-v]

libsdg_gpu.so (CUDA kernels + C ABI + host mesh layer) is compiled with nvcc
for sm_103a only, its translation units in parallel (one per kernel family).  Outputs are git-ignored.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "subrosadg_gb300", "csrc")
LIBDIR = os.path.join(ROOT, "subrosadg_gb300", "lib")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd, cwd):
    proc = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return proc


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile libsdg_gpu.so (CUDA kernels + C ABI + host mesh layer)."""
    os.makedirs(LIBDIR, exist_ok=True)
    target = os.path.join(LIBDIR, "libsdg_gpu.so")
    units = ["sdg_variants_tensor.cu", "sdg_variants_tensor_hex.cu", "sdg_variants_dense.cu", "sdg_variants_dense_tet.cu", "sdg_variants_face.cu", "sdg_variants_adjoint_face.cu",
             "sdg_variants_adjoint_tile.cu", "sdg_variants_adjoint_hex.cu", "sdg_variants_adjoint_dense_tet.cu", "sdg_variants_adjoint_dense.cu", "sdg_gpu.cu", "sdg_batch.cu",
             "sdg_adjoint.cu", "sdg_rawbinary.cu",
             "sdg_mesh.cpp", "sdg_noalloc.cu", "sdg_av.cu"]
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".cpp", ".hpp", ".h"))]
    deps.append(os.path.join(ROOT, "include", "sdg_gpu.h"))
    if not force and not _stale(target, deps):
        return target
    nvcc = _nvcc()
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)

    def compile_unit(u):
        obj = os.path.join(objdir, u + ".o")
        cmd = [nvcc, "-std=c++17", GENCODE, "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-O3,-fvisibility=hidden",
               "-c", os.path.join(CSRC, u), "-o", obj]
        if verbose:
            cmd.insert(4, "-Xptxas=-v")
        p = _run(cmd, CSRC)
        if verbose:
            sys.stderr.write(p.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_unit, units))
    _run([nvcc, GENCODE, "-shared", "-Xcompiler", "-fopenmp", "-o", target] + objs + ["-ldl"], CSRC)
    return target


CPP = os.path.join(ROOT, "subrosadg_gb300", "cpp")
DRIVERS = ["periodic_2d_ceuler"]


def build_drivers(force: bool = False) -> list:
    """Compile the C++23 example drivers (cpp/*.cpp over the C++ mirror gpu_solver.hpp) against libsdg_gpu.so."""
    lib = build_library(force=force)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    out = []
    for name in DRIVERS:
        target = os.path.join(LIBDIR, "sdg_" + name)
        deps = [os.path.join(CPP, name + ".cpp"), os.path.join(CPP, "gpu_solver.hpp"), lib,
                os.path.join(ROOT, "include", "sdg_gpu.h")]
        if force or _stale(target, deps):
            _run([cxx, "-std=c++23", "-O2", "-Wall", "-Wextra", "-o", target, os.path.join(CPP, name + ".cpp"),
                  "-L" + LIBDIR, "-lsdg_gpu", "-Wl,-rpath,$ORIGIN"], CPP)
        out.append(target)
    return out


if __name__ == "__main__":
    print("built", build_library(force="--force" in sys.argv, verbose="-v" in sys.argv), *build_drivers())
