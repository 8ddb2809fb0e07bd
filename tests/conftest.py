"""Shared fixtures: the host bindings, the CPU oracle, and GPU helpers.

Tests marked ``gpu`` run the CUDA library through its C ABI on a GB300;
everything else runs on the CPU (oracle against the LAPACK golden vectors,
library build/exports, host-side logic).
"""
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def load_pkg():
    name = "kblas_gpu_gb300"
    if name in sys.modules:
        return sys.modules[name]
    path = os.path.join(ROOT, "kblas-gpu_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location(
        name, path, submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_workloads():
    name = "kblas_gpu_gb300.workloads"
    if name in sys.modules:
        return sys.modules[name]
    load_pkg()
    path = os.path.join(ROOT, "kblas-gpu_gb300", "workloads.py")
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def kb():
    return load_pkg()


@pytest.fixture(scope="session")
def wl():
    return load_workloads()


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def golden():
    return np.load(os.path.join(ROOT, "tests", "golden", "lapack_golden.npz"))


@pytest.fixture(scope="session")
def gpu(kb):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    kb.build()
    return torch


@pytest.fixture()
def handle(kb, gpu):
    h = kb.Handle()
    yield h
    gpu.cuda.synchronize()
    h.close()
