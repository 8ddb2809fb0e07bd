"""Build libkblas_phase.so: the library's units compiled with phase_hooks.h
force-included (clock64 phase timers in the persistent POSV kernels). Same
flags and units as the product build; objects in profiling/_obj/, the library
next to this file. Not used by the product, the tests or the benchmark."""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import build as B  # noqa: E402

OBJ = os.path.join(HERE, "_obj")
OUT = os.path.join(HERE, "libkblas_phase.so")


def _compile(unit):
    obj = os.path.join(OBJ, unit.replace(".cu", ".o"))
    cmd = [B.nvcc(), *B.NVCC_FLAGS, "-include", os.path.join(HERE, "phase_hooks.h"), "-c",
           os.path.join(B.CSRC, unit), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr}")
    return obj


def build():
    os.makedirs(OBJ, exist_ok=True)
    with cf.ThreadPoolExecutor(len(B.LIB_UNITS)) as ex:
        objs = list(ex.map(_compile, B.LIB_UNITS))
    r = subprocess.run([B.nvcc(), "-shared", *B.ARCH, "-o", OUT, *objs, "-lcublas", "-lcudart"],
                       capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(r.stderr)
    return OUT


if __name__ == "__main__":
    print(build())
