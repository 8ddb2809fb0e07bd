"""Build recipe of the native library (no cmake, no torch extension machinery).

``build()`` compiles every ``csrc/*.cu`` translation unit for sm_103a in
parallel (one nvcc per unit, objects cached in ``_build/``) and links

  * ``libkblas_gb300.so`` -- the KBLAS-compatible C ABI (include/*.h), and
  * ``libkblas_probe.so`` -- FMA-throughput probes used for roofline peaks.

Both land next to this file (in-tree, git-ignored). Host code is built with
portable flags only, so the same recipe works on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libkblas_gb300.so")
PROBE_LIB = os.path.join(HERE, "libkblas_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", INC, "-I", CSRC] + ARCH

LIB_UNITS = ["runtime.cu", "potrf_posv.cu", "trsm_trmm.cu", "syrk.cu", "gemm_batch.cu", "inverse.cu", "posv_mixed.cu",
             "posv_vbatch.cu", "posv_noalloc.cu", "cxx_overloads.cu"]
PROBE_UNITS = ["probe.cu"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit: str, verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    if not _stale(obj, [src, __file__] + _headers()):
        return obj
    cmd = [nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def _link(objs, out, libs):
    tmp = out + ".tmp%d" % os.getpid()
    cmd = [nvcc(), "-shared", *ARCH, "-o", tmp, *objs, *libs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed for {out}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = [u for u in LIB_UNITS + PROBE_UNITS if os.path.exists(os.path.join(CSRC, u))]
    jobs = jobs or min(len(units), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = dict(zip(units, ex.map(lambda u: _compile(u, verbose), units)))
    lib_objs = [objs[u] for u in LIB_UNITS if u in objs]
    if _stale(LIB, lib_objs):
        _link(lib_objs, LIB, ["-lcublas", "-lcudart"])
    probe_objs = [objs[u] for u in PROBE_UNITS if u in objs]
    if probe_objs and _stale(PROBE_LIB, probe_objs):
        _link(probe_objs, PROBE_LIB, ["-lcudart"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
