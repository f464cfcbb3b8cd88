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


from concurrent.futures import ThreadPoolExecutor

# liborc.so: the oracle in double (the reference's Real); liborc_ext.so: the same code in long double,
# the extended-precision truth the parity tests measure both the GPU path and the double oracle against.
# -ffp-contract=off keeps the double results identical on x86-64 and aarch64 hosts.
VARIANTS = {"liborc.so": [], "liborc_ext.so": ["-DORC_REAL=long double"]}


def _build_one(target, extra, force):
    srcs = [os.path.join(HERE, f) for f in ("sdg_oracle.cpp", "orc_basis.hpp", "orc_physics.hpp", "build.py")]
    srcs += [os.path.join(ROOT, "subrosadg_gb300", "csrc", f) for f in ("triangle_rules.h", "tetrahedron_rules.h")]
    srcs += [os.path.join(ROOT, "include", "sdg_gpu.h")]
    if not force and os.path.exists(target) and all(os.path.getmtime(s) <= os.path.getmtime(target) for s in srcs):
        return target
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O3", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-fvisibility=hidden",
           "-fvisibility-inlines-hidden", *extra, "-o", target,
           os.path.join(HERE, "sdg_oracle.cpp")]
    proc = subprocess.run(cmd, cwd=HERE, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + proc.stderr)
    return target


def build(force: bool = False) -> str:
    with ThreadPoolExecutor(max_workers=len(VARIANTS)) as ex:
        futs = [ex.submit(_build_one, os.path.join(HERE, name), extra, force) for name, extra in VARIANTS.items()]
        out = [f.result() for f in futs]
    return out[0]


if __name__ == "__main__":
    print(build(force=True))
