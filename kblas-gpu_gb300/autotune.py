"""Autotuner of the persistent POSV launch shapes (writes csrc/tuning_table.h).

The persistent POSV kernels (plain FP64 and mixed precision) split orders into
eight size classes; per class the table gives the team size (threads per system)
and the systems per work item. A work item is spread over the teams of one
CTA, one system per team, so the useful item size is the number of teams
(256 / team size); the choice that matters is the team size. For each class
this sweeps every team size the kernels accept, times the variable-size POSV
on a batch whose orders are log-uniform over that class, and keeps the fastest.
The chosen table is applied at run time through kblasSetPosvTuning while it
is measured, and written out as a header to be compiled in.

It also tunes the mixed path's conditioning-routing constant (the c of
route_fp64 in csrc/posv_core.cuh, set through kblasSetPosvRouting): on a
uniform batch of n = 64 systems with 4 right-hand sides and condition numbers
log-uniform in [1e2, 1e8] it times the mixed POSV for each candidate c (0 =
no routing) and keeps the fastest; every candidate's results must meet the
backward-error bar (checked on the device: info 0 for all systems).

Run on the GPU:  python kblas-gpu_gb300/autotune.py --out <path>/tuning_table.h
"""
from __future__ import annotations

import argparse
import datetime
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NT = 256                                  # threads per CTA of the persistent kernels
# class upper bounds (last: largest supported order); 64, 96 and 176 are
# about where the factors of 8, 4 and 2 teams per CTA stop fitting in shared
# memory
NMAX = [8, 16, 32, 64, 96, 128, 176, 1024]
CLASS_TOP = [8, 16, 32, 64, 96, 128, 176, 256]  # orders swept per class (last capped at 256)
NCLS = len(NMAX)
CANDIDATES = [                            # team sizes accepted per class (W >= n for n <= 32)
    [8, 16, 32],
    [16, 32],
    [32],
    [32, 64, 128],
    [32, 64, 128, 256],
    [32, 64, 128, 256],
    [64, 128, 256],
    [64, 128, 256],
]


def load_pkg():
    name = "kblas_gpu_gb300"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(HERE, "__init__.py"),
                                                  submodule_search_locations=[HERE])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


class ClassBatch:
    """SPD systems (A = G G^T + n I, one RHS) with orders log-uniform over
    [lo, hi], each in its own slice of one device pool, with pointer arrays."""

    def __init__(self, torch, lo, hi, bytes_target=1.5e9, seed=0, max_batch=200_000):
        rng = np.random.default_rng(seed)
        mean_bytes = 8.0 * np.mean(np.arange(lo, hi + 1, dtype=np.float64) ** 2)
        batch = int(min(max_batch, max(2000, bytes_target / mean_bytes)))
        u = rng.uniform(np.log(lo), np.log(hi + 1), batch)
        ns = np.clip(np.floor(np.exp(u)).astype(np.int32), lo, hi)
        ns.sort()
        self.batch, self.ns = batch, ns
        offs = np.concatenate([[0], np.cumsum(ns.astype(np.int64) ** 2)[:-1]])
        boffs = np.concatenate([[0], np.cumsum(ns.astype(np.int64))[:-1]])
        self.A = torch.empty(int((ns.astype(np.int64) ** 2).sum()), dtype=torch.float64,
                             device="cuda")
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        for n in np.unique(ns):
            sel = np.where(ns == n)[0]
            n = int(n)
            for c0 in range(0, len(sel), 4096):
                s_ = sel[c0:c0 + 4096]
                g = torch.randn((len(s_), n, n), generator=gen, dtype=torch.float64, device="cuda")
                a = g @ g.transpose(1, 2)
                a.diagonal(dim1=1, dim2=2).add_(float(n))
                o0 = int(offs[s_[0]])
                self.A[o0:o0 + len(s_) * n * n].copy_(a.reshape(-1))
        self.A0 = self.A.clone()
        self.B0 = torch.randn(int(ns.sum()), generator=gen, dtype=torch.float64, device="cuda")
        self.B = self.B0.clone()
        self.pA = torch.from_numpy(self.A.data_ptr() + offs * 8).cuda()
        self.pB = torch.from_numpy(self.B.data_ptr() + boffs * 8).cuda()
        self.dn = torch.from_numpy(ns).cuda()
        self.dm = torch.ones(batch, dtype=torch.int32, device="cuda")
        self.dldb = torch.ones(batch, dtype=torch.int32, device="cuda")
        self.info = torch.zeros(batch, dtype=torch.int32, device="cuda")
        self.iter = torch.zeros(batch, dtype=torch.int32, device="cuda")
        self.max_n = int(ns.max())

    def restore(self):
        self.A.copy_(self.A0)
        self.B.copy_(self.B0)


def time_call(torch, kb, h, cb, mixed, reps):
    """Median device time (ms) of one variable-size POSV call over the batch;
    A and B are restored outside the timed region."""
    name = "kblasDposv_vbatch_mixed" if mixed else "kblasDposv_vbatch"
    args = ["R", "L", cb.dm.data_ptr(), cb.dn.data_ptr(), 1, cb.max_n, cb.pA.data_ptr(),
            cb.dn.data_ptr(), cb.pB.data_ptr(), cb.dldb.data_ptr(), cb.batch, cb.info.data_ptr()]
    if mixed:
        args.append(cb.iter.data_ptr())
    stream = torch.cuda.current_stream()
    times = []
    for r in range(reps + 2):
        cb.restore()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = h.call(name, *args)
        e1.record(stream)
        e1.synchronize()
        if st != 1:
            raise RuntimeError(f"{name} returned {st}")
        if r >= 2:
            times.append(e0.elapsed_time(e1))
    if int((cb.info != 0).sum()) != 0:
        raise RuntimeError("tuning batch produced non-zero info")
    return float(np.median(times))


ROUTE_CANDIDATES = [0.0, 4.0, 8.0, 16.0, 32.0, 64.0, 128.0]


class CondBatch:
    """Uniform strided batch of n = 64 SPD systems A = Q diag(l) Q^T (Q from
    the QR of a Gaussian matrix, l geometric with cond log-uniform in
    [1e2, 1e8]) and 4 right-hand sides."""

    def __init__(self, torch, batch=20_000, n=64, m=4, seed=7):
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        q, _ = torch.linalg.qr(torch.randn((batch, n, n), generator=gen, dtype=torch.float64,
                                           device="cuda"))
        lc = torch.rand(batch, generator=gen, dtype=torch.float64, device="cuda") * 6 + 2
        t = torch.linspace(0, 1, n, dtype=torch.float64, device="cuda")
        lam = torch.pow(10.0, -lc[:, None] * t[None, :])
        a = (q * lam[:, None, :]) @ q.transpose(1, 2)
        self.A0 = (0.5 * (a + a.transpose(1, 2))).contiguous()
        self.B0 = torch.randn((batch, n, m), generator=gen, dtype=torch.float64, device="cuda")
        self.A, self.B = self.A0.clone(), self.B0.clone()
        self.info = torch.zeros(batch, dtype=torch.int32, device="cuda")
        self.iter = torch.zeros(batch, dtype=torch.int32, device="cuda")
        self.batch, self.n, self.m = batch, n, m


def time_route(torch, kb, h, cb, reps):
    stream = torch.cuda.current_stream()
    times = []
    for r in range(reps + 2):
        cb.A.copy_(cb.A0)
        cb.B.copy_(cb.B0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = h.call("kblasDposv_batch_mixed_strided", "R", "L", cb.m, cb.n, cb.A.data_ptr(), cb.n,
                    cb.n * cb.n, cb.B.data_ptr(), cb.m, cb.n * cb.m, cb.batch,
                    cb.info.data_ptr(), cb.iter.data_ptr())
        e1.record(stream)
        e1.synchronize()
        if st != 1:
            raise RuntimeError(f"kblasDposv_batch_mixed_strided returned {st}")
        if r >= 2:
            times.append(e0.elapsed_time(e1))
    if int((cb.info != 0).sum()) != 0:
        raise RuntimeError("routing batch produced non-zero info")
    return float(np.median(times))


def tune_route(torch, kb, reps=5, log=print):
    """Returns {"route_c": best, "ms": {c: ms}}."""
    h = kb.Handle(stream=torch.cuda.current_stream().cuda_stream)
    cb = CondBatch(torch)
    res = {}
    try:
        kb.lib().kblas_posv_batch_mixed_wsquery(h.ptr, b"R", cb.m, cb.n, cb.batch)
        kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")
        for c in ROUTE_CANDIDATES:
            kb.check(kb.lib().kblasSetPosvRouting(c), "kblasSetPosvRouting")
            res[c] = time_route(torch, kb, h, cb, reps)
            log(f"route c {c:g}: {res[c]:.3f} ms")
    finally:
        kb.lib().kblasSetPosvRouting(-1.0)
        torch.cuda.synchronize()
        h.close()
    return {"route_c": min(res, key=res.get), "ms": res}


def set_table(kb, mixed, ts, spi):
    C = __import__("ctypes")
    arr = lambda v: (C.c_int * NCLS)(*v)
    st = kb.lib().kblasSetPosvTuning(1 if mixed else 0, arr(NMAX), arr(ts), arr(spi))
    if st != 1:
        raise RuntimeError(f"kblasSetPosvTuning rejected ts={ts} spi={spi}")


def tune(torch, kb, reps=5, log=print):
    """Returns {form: {"ts": [...], "spi": [...], "ms": {class: {ts: ms}}}}."""
    h = kb.Handle(stream=torch.cuda.current_stream().cuda_stream)
    out = {}
    batches = []
    for c in range(NCLS):
        lo = 1 if c == 0 else CLASS_TOP[c - 1] + 1
        batches.append(ClassBatch(torch, lo, CLASS_TOP[c], seed=c))
    try:
        for form in ("mixed", "plain"):
            mixed = form == "mixed"
            best_ts = [8, 16, 32, 32, 64, 128, 128, 256]
            best_spi = [NT // t for t in best_ts]
            ms_table = {}
            for c in range(NCLS):
                cb = batches[c]
                res = {}
                for ts in CANDIDATES[c]:
                    trial_ts, trial_spi = list(best_ts), list(best_spi)
                    trial_ts[c], trial_spi[c] = ts, NT // ts
                    set_table(kb, mixed, trial_ts, trial_spi)
                    # the scratch per CTA depends on the table
                    kb.lib().kblas_posv_vbatch_wsquery(h.ptr, cb.max_n, cb.batch)
                    kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")
                    res[ts] = time_call(torch, kb, h, cb, mixed, reps)
                    log(f"{form} class {c} (n {1 if c == 0 else CLASS_TOP[c - 1] + 1}.."
                        f"{CLASS_TOP[c]}, {cb.batch} systems) ts {ts}: {res[ts]:.3f} ms")
                ts = min(res, key=res.get)
                best_ts[c], best_spi[c] = ts, NT // ts
                ms_table[c] = res
            out[form] = {"ts": best_ts, "spi": best_spi, "ms": ms_table}
    finally:
        kb.lib().kblasSetPosvTuning(1, None, None, None)
        kb.lib().kblasSetPosvTuning(0, None, None, None)
        torch.cuda.synchronize()
        h.close()
    return out


def header_text(result, device_name):
    stamp = datetime.date.today().isoformat()
    lines = [
        "// tuning_table.h -- per-size-class launch shapes of the persistent POSV",
        "// kernels: class upper bound on n, team size (threads per system) and",
        "// systems per work item. Written by kblas-gpu_gb300/autotune.py from",
        f"// measurements on {device_name} ({stamp}): per class, the team size with",
        "// the shortest variable-size POSV over orders log-uniform in the class.",
        "#pragma once",
        "",
        "// {nmax}, {team size}, {systems per item}",
    ]
    route = result.get("route")
    if route:
        lines.append("// conditioning routing constant of the mixed path (route_fp64): the")
        lines.append("// fastest mixed POSV on n = 64, 4 RHS, cond 1e2..1e8 (ms per call: "
                     + ", ".join(f"c {k:g}: {v:.3f}" for k, v in route["ms"].items()) + ")")
        lines.append(f"#define KGB_TUNE_ROUTE_C {float(route['route_c']):.1f}f")
        lines.append("")
    for form, tag in (("mixed", "MIXED"), ("plain", "PLAIN")):
        r = result[form]
        lines.append(f"#define KGB_TUNE_{tag}_NMAX {{{', '.join(map(str, NMAX))}}}")
        lines.append(f"#define KGB_TUNE_{tag}_TS {{{', '.join(map(str, r['ts']))}}}")
        lines.append(f"#define KGB_TUNE_{tag}_SPI {{{', '.join(map(str, r['spi']))}}}")
        lines.append("")
    lines.append("// measured ms per call, class: {team size: ms}")
    for form in ("mixed", "plain"):
        for c, res in result[form]["ms"].items():
            txt = ", ".join(f"{k}: {v:.3f}" for k, v in res.items())
            lines.append(f"//   {form} class {c}: {txt}")
    return "\n".join(lines) + "\n"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "csrc", "tuning_table.h"))
    ap.add_argument("--json", default=None)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args()
    import torch
    kb = load_pkg()
    kb.lib()
    result = tune(torch, kb, reps=args.reps)
    result["route"] = tune_route(torch, kb, reps=args.reps)
    text = header_text(result, torch.cuda.get_device_name(0))
    with open(args.out, "w") as f:
        f.write(text)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(result, f, indent=1, default=str)
    print(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
