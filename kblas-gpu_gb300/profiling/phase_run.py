"""Per-phase SM cycles of the mixed-precision POSV panel path, from the
clock64 build (phase_build.py). Runs kblasDposv_batch_mixed_strided on
squared-exponential covariances (nugget 1e-4) and prints one JSON line per
case: the call's event time, its per-SM cycles per system (time x SM clock x
SMs / systems) and, per phase, the cycles and visits per system.

Phases (posv_core.cuh, panel_mixed_posv): stage (scales, FP64 -> FP32 panels),
factor (FP32 panel Cholesky + diagonal-block inverses), solve0 (first FP32
solve, per sweep of up to 4 right-hand sides), residual (FP64 r = b - A x,
per sweep), solve_corr (convergence test + FP32 correction solve, per step),
tail (write-back). Sub-phases of the factorization (chol_panel.cuh,
team_potrf_panel_la): f:diag0, f:rows_trsm, f:trailing, f:invert; inside
f:trailing, warp 0's look-ahead (update and factor of the next diagonal
block) and, timed by warp 1, the trailing update of the other warps.

Run on the GPU:  python kblas-gpu_gb300/profiling/phase_build.py &&
                 python kblas-gpu_gb300/profiling/phase_run.py [batch n nrhs [sqexp|spd]]
(KGB_NO_TC=1 in the environment: FP32 FMA trailing updates instead of the
tensor cores, for comparison.)
"""
import ctypes as C
import importlib.util
import json
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
NAMES = {0: "stage", 1: "factor", 2: "solve0", 3: "residual", 4: "solve_corr", 5: "tail",
         8: "f:diag0", 9: "f:rows_trsm", 10: "f:trailing", 11: "f:invert",
         12: "f:w0_next_block_update", 13: "f:w0_next_block_factor",
         14: "f:w1_trailing_update", 15: "f:w1_before_update"}


def _load(name, path, pkg=False):
    spec = importlib.util.spec_from_file_location(
        name, path, submodule_search_locations=[os.path.dirname(path)] if pkg else None)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def main():
    kb = _load("kblas_gpu_gb300", os.path.join(PKG, "__init__.py"), pkg=True)
    wl = _load("kblas_gpu_gb300.workloads", os.path.join(PKG, "workloads.py"))
    kb.LIB_PATH = os.path.join(HERE, "libkblas_phase.so")
    lib = kb.lib()
    lib.kgb_phase_all.restype = C.c_int
    lib.kgb_phase_all.argtypes = [C.c_void_p, C.c_int]
    batch = int(sys.argv[1]) if len(sys.argv) > 1 else 2000
    n = int(sys.argv[2]) if len(sys.argv) > 2 else 512
    m = int(sys.argv[3]) if len(sys.argv) > 3 else 8
    kind = sys.argv[4] if len(sys.argv) > 4 else "sqexp"
    prop = torch.cuda.get_device_properties(0)
    if kind == "spd":  # A = G G^T + n I (the variable-size benchmark's recipe)
        a = wl.spd_shifted(batch, n, seed=0)
    else:
        a = np.concatenate([wl.sqexp_cov(100, n, seed=k) for k in range((batch + 99) // 100)])[:batch]
    b = wl.rhs_rows(batch, m, n, seed=1)
    A0, B0 = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    A, B = A0.clone(), B0.clone()
    info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    it = torch.zeros_like(info)
    h = kb.Handle()
    lib.kblas_posv_batch_mixed_wsquery(h.ptr, b"R", m, n, batch)
    kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")

    def call():
        kb.check(h.call("kblasDposv_batch_mixed_strided", "R", "L", m, n, A.data_ptr(), n, n * n,
                        B.data_ptr(), m, m * n, batch, info.data_ptr(), it.data_ptr()), "mixed")

    buf = (C.c_ulonglong * 32)()
    for _ in range(2):
        A.copy_(A0)
        B.copy_(B0)
        call()
    A.copy_(A0)
    B.copy_(B0)
    torch.cuda.synchronize()
    lib.kgb_phase_all(buf, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    call()
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    lib.kgb_phase_all(buf, 0)
    itv = it.cpu().numpy()
    clock_hz = 2.07e9  # the maximum SM clock; the benchmark's clock samples show it held
    out = {"batch": batch, "n": n, "nrhs": m, "matrices": kind, "ms": ms,
           "tensor_core_update": os.environ.get("KGB_NO_TC") != "1",
           "per_sm_cycles_per_system": ms * 1e-3 * clock_hz * prop.multi_processor_count / batch,
           "mean_steps": float(itv[itv >= 0].mean()) if (itv >= 0).any() else None,
           "fallbacks": int((itv < 0).sum()), "phases": {}}
    for k, name in NAMES.items():
        if buf[16 + k]:
            out["phases"][name] = {"cycles_per_system": buf[k] / batch,
                                   "visits_per_system": buf[16 + k] / batch}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
