"""Build recipe for libmontegpu.so (sm_103a) and the CPU oracle.

``python -m casmcode_monte_gb300.build`` compiles every CUDA translation unit in
parallel with nvcc for ``sm_103a`` only and links ``casmcode_monte_gb300/lib/
libmontegpu.so``.  Objects are cached by source modification time.  The oracle
(test infrastructure) is built separately by ``build_oracle()`` with make.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "libmontegpu.so"
SOURCES = ["mg_api.cu", "ising_replay.cu", "ce_api.cu", "ce_noalloc.cu", "ce_pool.cu", "ce_canonical.cu", "ce_nfold.cu", "ce_replay.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code keeps a*b+c unfused (-ffp-contract=off) so results match the reference's
# un-contracted FP64 arithmetic on aarch64 as on x86-64
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(CSRC, "generated"), os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h", ".inc")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


# per-file flags: the pool's device statistics must round exactly like the host code
FILE_FLAGS = {"ce_pool.cu": ["-fmad=false"]}


def _compile(src: str, verbose: bool, extra: list[str]) -> str:
    obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
    srcp = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(srcp), _deps_mtime()) and not extra:
        return obj
    cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(src, []), *extra, "-c", srcp, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if extra and (r.stdout or r.stderr):
        print(r.stdout + r.stderr)
    return obj


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile and link libmontegpu.so; returns its path."""
    os.makedirs(OBJDIR, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, extra), SOURCES))
    out = os.path.join(LIBDIR, LIBNAME)
    if not os.path.exists(out) or any(os.path.getmtime(o) > os.path.getmtime(out) for o in objs):
        cmd = [_nvcc(), *ARCH, "-shared", "--cudart", "static", "-o", out, *objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


def build_oracle(verbose: bool = False) -> str:
    """Build the CPU oracle (test infrastructure) with its Makefile."""
    d = os.path.join(ROOT, "oracle")
    r = subprocess.run(["make", "-C", d], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout)
    return os.path.join(d, "build", "liboracle.so")


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv))
