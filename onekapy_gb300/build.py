"""Build liboneka_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch extension).

    python -m onekapy_gb300.build [--verbose] [--force]

Each translation unit compiles in parallel; the FP64 units are built with
``--fmad=false`` so that no multiply-add is contracted (the reference's
Python/NumPy arithmetic rounds every operation).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "liboneka_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-I", os.path.join(ROOT, "include")]

# translation unit -> extra flags
UNITS = {
    "capi.cu": ["--fmad=false"],
    "chronicle.cu": ["--fmad=false"],
    "realize.cu": ["--fmad=false"],
    "track64.cu": ["--fmad=false"],
    "track32.cu": ["--fmad=true", "--use_fast_math"],
    "probe.cu": ["--fmad=true"],
    "noalloc.cu": ["--fmad=false"],
    "mlp.cu": ["--fmad=true"],
    "gemm_tc.cu": ["--fmad=true"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found (set NVCC or put /usr/local/cuda/bin on PATH)")


def _sources_newer(target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "oneka_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _sources_newer(LIB):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    cc = nvcc()

    def compile_unit(name):
        obj = os.path.join(OBJ_DIR, name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], "-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, sorted(UNITS)))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
