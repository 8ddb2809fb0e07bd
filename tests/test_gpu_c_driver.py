"""A plain C host program (tests/c_driver/kblas_c_driver.c) drives the library
through its C ABI exactly as a KBLAS caller does -- handle, workspace queries,
padded device matrices, device pointer arrays, info read back -- and checks
every result against the CPU oracle it links. The CPU test compiles and links
it; the GPU tests run it at the n = 32 benchmark shape and at a blocked-path
shape with several right-hand sides."""
import glob
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "c_driver", "kblas_c_driver.c")


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _cudart_dir(home):
    for d in [os.path.join(home, "lib64")] + sorted(glob.glob(os.path.join(home, "targets", "*", "lib"))):
        if os.path.exists(os.path.join(d, "libcudart.so")):
            return d
    pytest.skip("libcudart.so not found next to nvcc")


def build_driver(kb, out_dir):
    """gcc -std=c99 against include/, linking libkblas_gb300.so, the oracle and
    libcudart; returns the executable's path."""
    from oracle import oracle as orc
    kb.build()
    orc.build()
    home = _cuda_home()
    libdir = os.path.join(ROOT, "kblas-gpu_gb300")
    orcdir = os.path.join(ROOT, "oracle")
    rtdir = _cudart_dir(home)
    exe = os.path.join(str(out_dir), "kblas_c_driver")
    cmd = ["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(home, "include"), SRC, "-o", exe,
           "-L", libdir, "-lkblas_gb300", "-L", orcdir, "-loracle", "-L", rtdir, "-lcudart", "-lm",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{orcdir}", f"-Wl,-rpath,{rtdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_c_driver_compiles_and_links(kb, tmp_path):
    exe = build_driver(kb, tmp_path)
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
@pytest.mark.parametrize("args", [
    (1000, 32, 1, 400, 130),   # the uniform n = 32 shape, one right-hand side
    (200, 100, 4, 300, 256),   # blocked / panel orders, four right-hand sides
])
def test_c_driver_runs_against_oracle(kb, gpu, tmp_path, args):
    exe = build_driver(kb, tmp_path)
    r = subprocess.run([exe, *map(str, args)], capture_output=True, text=True, timeout=300)
    out = r.stdout + r.stderr
    print(out)
    assert r.returncode == 0, out
    assert "ALL PASS" in r.stdout, out
    assert r.stdout.count(" PASS ") >= 7, out
