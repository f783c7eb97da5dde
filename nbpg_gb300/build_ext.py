"""Compile libnbpg_gb300.so in-tree with nvcc for sm_103a.

Each .cu translation unit compiles in parallel to an object file under
``nbpg_gb300/_build``; they are then linked into ``nbpg_gb300/_build/libnbpg_gb300.so``.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnbpg_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no floating-point contraction, so that float expressions round as written on every host
# (GCC contracts a * b + c into an FMA by default where the CPU has one, as the Grace host does; the
# popularity-driven alpha of the build, minAlpha + cof * (maxAlpha - minAlpha), would then round
# differently from the restatement it is checked against)
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "-Xcompiler", "-ffp-contract=off",
         f"-I{INCLUDE}"]


def _newest_dep() -> float:
    deps = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max(os.path.getmtime(p) for p in deps) if deps else 0.0


def _compile(src: str, dep_time: float, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), dep_time):
        return obj
    cmd = [NVCC, *ARCH, *FLAGS, "-c", src, "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    dep_time = _newest_dep()
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, dep_time, verbose), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    _build_cli()
    return LIB


CLI = {"nbpg_vamana": ("vamana.cpp", []), "nbpg_fgim": ("vamana.cpp", ["-DNBPG_FGIM"]),
       "nbpg_compgt": ("compgt.cpp", []), "nbpg_pcacompress": ("pcacompress.cpp", []),
       "nbpg_fmtconv": ("fmtconv.cpp", []), "nbpg_hnsw": ("hnsw.cpp", [])}


def _build_cli() -> None:
    """The drop-in executables for the reference's drivers (host C++ over the C ABI)."""
    cxx = os.environ.get("CXX", "g++")
    src_dir = os.path.join(HERE, "cli")
    for exe, (src, defs) in CLI.items():
        out = os.path.join(OUT, exe)
        srcp = os.path.join(src_dir, src)
        deps = [srcp, os.path.join(src_dir, "flags.h"), os.path.join(src_dir, "common.h"), os.path.join(INCLUDE, "nbpg.h"),
                LIB]
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
            continue
        cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", *defs, srcp, f"-I{INCLUDE}", f"-L{OUT}", "-lnbpg_gb300",
               "-Wl,-rpath,$ORIGIN", "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"building {exe} failed:\n{r.stderr}")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
