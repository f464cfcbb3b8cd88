"""Build recipe of the oracle (test infrastructure only): oracle/liborc.so.

The oracle is the CPU restatement of the reference algorithm that the tests and
the CPU baseline of bench.py check the GPU path against.  It is compiled with
g++ and OpenMP from oracle/sdg_oracle.cpp; no product code calls it.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build(force: bool = False) -> str:
    target = os.path.join(HERE, "liborc.so")
    srcs = [os.path.join(HERE, f) for f in ("sdg_oracle.cpp", "orc_basis.hpp", "orc_physics.hpp")]
    srcs += [os.path.join(ROOT, "subrosadg_gb300", "csrc", "triangle_rules.h"), os.path.join(ROOT, "include", "sdg_gpu.h")]
    if not force and os.path.exists(target) and all(os.path.getmtime(s) <= os.path.getmtime(target) for s in srcs):
        return target
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-o", target, os.path.join(HERE, "sdg_oracle.cpp")]
    proc = subprocess.run(cmd, cwd=HERE, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stderr)
    return target


if __name__ == "__main__":
    print(build(force=True))
