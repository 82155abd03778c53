"""Builds the CPU restatement (test infrastructure) as oracle/_build/libpbf_oracle.so.

-ffp-contract=off keeps every a*b+c as two roundings on every host
architecture, which is what makes the FP32 mirror bit-comparable with the
exact-mode CUDA passes.  OpenMP only parallelises independent per-particle
loops; results do not depend on the thread count.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpbf_oracle.so")
SRC = os.path.join(HERE, "pbf_oracle.cpp")
HDR = os.path.join(HERE, "..", "include", "pbf_gb300.h")


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(d) <= os.path.getmtime(LIB) for d in (SRC, HDR)):
        return LIB
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
           "-shared", SRC, "-o", LIB + ".tmp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="-f" in sys.argv))
