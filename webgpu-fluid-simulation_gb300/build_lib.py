"""Builds libpbf_gb300.so (the C ABI + CUDA kernels) in-tree for sm_103a.

Usage: python build_lib.py  (or import and call build()).  The translation
units compile in parallel with nvcc; the float passes are compiled twice,
once with -fmad=false (bit-exact mode) and once with FMA contraction.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libpbf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
UNITS = [
    ("pbf_api.cu", []),
    ("pbf_sort.cu", []),
    ("pbf_passes_fast.cu", []),
    ("pbf_passes_exact.cu", ["-fmad=false"]),
    ("pbf_volume.cu", ["-fmad=false"]),
    ("pbf_scan_static.cu", []),
    ("pbf_learned.cu", []),
    ("pbf_mlp_tc.cu", []),
    ("pbf_seed.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("pbf_render.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "pbf_gb300.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose=False, force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = _sources()
    if not force and not _stale(LIB, deps):
        return LIB
    nvcc = _nvcc()

    def compile_unit(unit):
        src, extra = unit
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [nvcc] + ARCH + COMMON + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
