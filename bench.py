"""Benchmark: batched POSV solves/s at backward error <= 10 n eps64, mixed
precision vs plain FP64, on GB300.

Workload (one "step" = one pass of the variable-size POSV over the batch):
100,000 SPD systems, n = floor(exp(U[ln 8, ln 257))) (8..256), A = G G^T + n I
with G ~ N(0, 1), one right-hand side b ~ N(0, 1), pointer-array storage
(each matrix n x n column-major, lda = n), every 100th system made indefinite
by flipping the sign of one eigenvalue (exercises the info codes and the FP64
fallback). Seeded synthetic data (seed 0), generated on the GPU.

Reported: ``value`` = mixed-precision solves/s with the inputs resident in HBM
(device time of the library call, CUDA events on the launching stream);
``fp64_form`` = the plain FP64 variable-size POSV on the same batch; ``e2e`` =
the same metric through the C ABI with pinned host buffers, the host->device
copy of A and B and the device->host copy of X and info inside the timed
region. Accuracy is checked against the CPU oracle on a sample (+ every
indefinite system) outside the timed region.

``--impl reference`` times the reference path's CPU implementation (LAPACK
DPOTRF + DPOTRS looped over the batch with all host threads -- the C oracle,
a restatement of LAPACK) on a bounded sample of the same workload.
"""
import argparse
import importlib.util
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched POSV solves/s at backward err ≤10·n·eps64: mixed-prec vs plain FP64"
EPS64 = 2.0 ** -53
E2E_CHUNKS = 16
LINK_PROBE_REPS = 5  # plain host->device copies of the matrix pool after the e2e steps
WORKLOAD = ("variable-size DPOSV: 100000 SPD systems, n log-uniform integer 8..256, "
            "A = G G^T + n I, 1 RHS, pointer arrays, 1% indefinite (one eigenvalue flipped)")


def load_pkg():
    import __graft_entry__ as g
    return g._pkg(), g._workloads()


def shard_mod():
    import importlib
    load_pkg()
    return importlib.import_module("kblas_gpu_gb300.shard")


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


# ----------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------
class VWorkload:
    """Variable-size POSV batch resident on the GPU."""

    def __init__(self, torch, wl, batch=100_000, nmin=8, nmax=256, seed=0, indef_every=100,
                 shard=(0, 1)):
        dev = "cuda"
        self.torch = torch
        rank, world = shard
        ns_all = wl.vbatch_sizes(batch, nmin, nmax, seed=seed)
        # this rank's contiguous range, balanced by work (no data exchange)
        lo, hi = shard_mod().shard_range(ns_all, rank, world)
        mine = np.arange(lo, hi)
        self.gidx = mine
        self.ns = ns_all[mine].astype(np.int32)
        self.batch = len(mine)
        self.indef = np.where(self.gidx % indef_every == 0)[0]  # local indices
        is_indef = np.zeros(self.batch, bool)
        is_indef[self.indef] = True
        # pool layout: SPD systems first, grouped by n (contiguous per order),
        # then the indefinite ones in one trailing region, restored between
        # steps with one copy (the FP64 fallback writes its partial factor)
        order = np.lexsort((self.ns, is_indef))
        sizes = self.ns.astype(np.int64) ** 2
        offs = np.zeros(self.batch, np.int64)
        offs[order] = np.concatenate([[0], np.cumsum(sizes[order])[:-1]])
        self.offs = offs
        self.pool_elems = int(sizes.sum())
        self.indef_lo = int(offs[self.indef].min()) if len(self.indef) else self.pool_elems
        self.A = torch.empty(self.pool_elems, dtype=torch.float64, device=dev)
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        for grp in (False, True):
            for n in np.unique(self.ns[is_indef == grp]):
                sel = np.where((self.ns == n) & (is_indef == grp))[0]
                sel = sel[np.argsort(offs[sel])]  # contiguous run in the pool
                n = int(n)
                for c0 in range(0, len(sel), 2048):
                    s_ = sel[c0:c0 + 2048]
                    g = torch.randn((len(s_), n, n), generator=gen, dtype=torch.float64, device=dev)
                    a = g @ g.transpose(1, 2)
                    a.diagonal(dim1=1, dim2=2).add_(float(n))
                    if grp:
                        # flip one eigenvalue (numpy on the host: ~1% of the batch)
                        an = a.cpu().numpy()
                        w_, v_ = np.linalg.eigh(an)
                        k = torch.randint(0, n, (len(s_),), generator=gen, device=dev).cpu().numpy()
                        ar = np.arange(len(s_))
                        vk = v_[ar, :, k]
                        wk = w_[ar, k]
                        an = an - 2.0 * wk[:, None, None] * vk[:, :, None] * vk[:, None, :]
                        an = 0.5 * (an + an.transpose(0, 2, 1))
                        a = torch.from_numpy(an).to(dev)
                    o0 = int(offs[s_[0]])
                    self.A[o0:o0 + len(s_) * n * n].copy_(a.reshape(-1))  # symmetric: col-major == row-major
                    del g, a
        self.A0_indef = self.A[self.indef_lo:].clone()
        bsz = self.ns.astype(np.int64)
        self.boffs = np.concatenate([[0], np.cumsum(bsz)[:-1]])
        self.B0 = torch.randn(int(bsz.sum()), generator=gen, dtype=torch.float64, device=dev)
        self.B = self.B0.clone()
        base = self.A.data_ptr()
        self.pA = torch.from_numpy(base + self.offs * 8).to(dev)
        self.pB = torch.from_numpy(self.B.data_ptr() + self.boffs * 8).to(dev)
        self.dn = torch.from_numpy(self.ns).to(dev)
        self.dm = torch.ones(self.batch, dtype=torch.int32, device=dev)
        self.dlda = self.dn.clone()
        self.dldb = torch.ones(self.batch, dtype=torch.int32, device=dev)
        self.info = torch.zeros(self.batch, dtype=torch.int32, device=dev)
        self.iter = torch.zeros(self.batch, dtype=torch.int32, device=dev)
        self.max_n = int(self.ns.max())

    def restore(self, full=False):
        if full:
            self.A.copy_(self.A_pristine)
        elif self.indef_lo < self.pool_elems:
            self.A[self.indef_lo:].copy_(self.A0_indef)
        self.B.copy_(self.B0)

    def keep_pristine(self):
        self.A_pristine = self.A.clone()

    # algorithmic units
    def flops_useful(self, nrhs=1):
        n = self.ns.astype(np.float64)
        potrf = n ** 3 / 3 + n ** 2 / 2 + n / 6  # reference testing/flops.h POTRF
        potrs = 2 * nrhs * n ** 2
        return float((potrf + potrs).sum())

    def alg_bytes(self, nrhs=1):
        n = self.ns.astype(np.float64)
        return float((8 * n * (n + 1) + 16 * n * nrhs).sum())


def call_vbatch(kb, h, w, mixed):
    name = "kblasDposv_vbatch_mixed" if mixed else "kblasDposv_vbatch"
    args = ["R", "L", w.dm.data_ptr(), w.dn.data_ptr(), 1, w.max_n, w.pA.data_ptr(),
            w.dlda.data_ptr(), w.pB.data_ptr(), w.dldb.data_ptr(), w.batch, w.info.data_ptr()]
    if mixed:
        args.append(w.iter.data_ptr())
    st = h.call(name, *args)
    if st != 1:
        raise RuntimeError(f"{name} returned {st}")


# ----------------------------------------------------------------------------
# clocks sampling (nvidia-smi during the timed region)
# ----------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows = []
        self.p = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[3:7]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# measurement helpers
# ----------------------------------------------------------------------------
def timed_steps(torch, fn, before, steps, warmup, stream):
    """Warm-up, then `steps` timed calls; `before` runs outside the events."""
    for _ in range(warmup):
        before()
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        before()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    return times


def measure_fp64_peak(kb, torch):
    """Live FP64 FMA throughput of this GPU (the denominator of every FP64-pipe
    fraction): libkblas_probe.so's kblas_probe_fma (csrc/probe.cu) runs one
    CTA per SM of 512 threads (16 warps), each thread ILP = 4 independent
    chains of `iters` dependent FMAs; one warm-up launch and one launch timed
    with CUDA events per repeat, best of 3 repeats. Returns the record."""
    p = kb.probe_lib()
    scratch = torch.zeros(1 << 20, dtype=torch.float64, device="cuda")
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    threads, iters, ilp, repeats = 512, 4096, 4, 3
    times = []
    for _ in range(repeats):
        times.append(float(p.kblas_probe_fma(64, nsm, threads, iters, ilp, scratch.data_ptr())))
    flop = 2.0 * nsm * threads * iters * ilp
    best = max(flop / (ms * 1e-3) / 1e12 for ms in times)
    # the same chains on 32, 16 and 8 lanes of each warp: the time barely
    # moves, i.e. a predicated-off lane still costs its FP64 issue slot
    lanes = {str(a): float(p.kblas_probe_fma64_lanes(nsm, threads, iters, a, scratch.data_ptr()))
             for a in (32, 16, 8)}
    return {"peak_tflops_measured_live": best,
            "predicated_lanes_probe_ms": lanes,
            "probe": {"kernel": "fma_chain_kernel<double, 4> (csrc/probe.cu)", "blocks": nsm,
                      "threads_per_block": threads, "ilp_chains_per_thread": ilp,
                      "fma_per_chain": iters, "flop_per_launch": flop, "repeats": repeats,
                      "kernel_ms": [round(x, 4) for x in times], "statistic": "best of repeats"}}


def accuracy_check(orc, w, torch, sample=1500, seed=0):
    """Backward error of a random sample of systems + all indefinite ones
    (info exactness), CPU oracle."""
    rng = np.random.default_rng(seed)
    pick = np.unique(np.concatenate([rng.choice(w.batch, min(sample, w.batch), replace=False),
                                     w.indef]))
    info = w.info.cpu().numpy()
    Xh = w.B.cpu().numpy()
    Bh = w.B0.cpu().numpy()
    As, Xs, Bs, ns = [], [], [], []
    for i in pick:
        n = int(w.ns[i])
        As.append(w.A_pristine[w.offs[i]:w.offs[i] + n * n].cpu().numpy().reshape(n, n).copy())
        Xs.append(Xh[w.boffs[i]:w.boffs[i] + n].reshape(n, 1).copy())
        Bs.append(Bh[w.boffs[i]:w.boffs[i] + n].reshape(n, 1).copy())
        ns.append(n)
    ms = [1] * len(pick)
    # reference info codes
    refA = [a.copy() for a in As]
    refB = [b.copy() for b in Bs]
    info_ref = orc.posv_vbatch(ms, ns, refA, ns, refB, [1] * len(pick))
    info_ok = bool(np.array_equal(info[pick], info_ref))
    good = [k for k in range(len(pick)) if info_ref[k] == 0]
    eta = orc.backward_error_r_vbatch([1] * len(good), [ns[k] for k in good], [As[k] for k in good],
                                      [ns[k] for k in good], [Xs[k] for k in good], [1] * len(good),
                                      [Bs[k] for k in good], [1] * len(good))
    ratio = eta / np.array([10 * ns[k] * EPS64 for k in good])
    # forward error against the oracle's FP64 solution (refB now holds it)
    fwd = np.array([np.abs(Xs[k] - refB[k]).max() / max(float(np.abs(refB[k]).max()), 1e-300)
                    for k in good])
    return {"checked": int(len(pick)), "info_exact": info_ok,
            "max_eta_over_10n_eps": float(ratio.max()) if len(ratio) else 0.0,
            "max_forward_rel_err_vs_oracle": float(fwd.max()) if len(fwd) else 0.0,
            "all_within_bound": bool((ratio <= 1.0).all()),
            "indefinite_checked": int(len(w.indef))}


class CpuSample:
    """Systems drawn from the benchmark's n distribution, solved the way the
    reference testers time the CPU path: LAPACK dpotrf + dpotrs per system,
    OpenMP over the batch, all host threads. The LAPACK is the host's
    optimized one (scipy's, one thread per call) when scipy is importable,
    else the oracle's C restatement. A pool of distinct systems is generated
    once; each timed chunk solves fresh copies of systems drawn from it
    (copies made outside the timer)."""

    POOL = 8000
    CHUNK = 8000

    def __init__(self, orc, wl, seed=0):
        self.orc = orc
        self.nth = os.cpu_count() or 1
        lp = orc.host_lapack()
        self.lapack = lp is not None
        self.solver = lp[2] if lp else "FP64 POTRF+POTRS, C restatement of LAPACK"
        ns = wl.vbatch_sizes(100_000, 8, 256, seed=seed)
        rng = np.random.default_rng(seed + 1)
        self.rng = rng
        self.pool = []
        for i in rng.choice(len(ns), self.POOL, replace=False):
            n = int(ns[i])
            g = rng.standard_normal((n, n))
            self.pool.append((np.ascontiguousarray(g @ g.T + n * np.eye(n)),
                              rng.standard_normal((n, 1)), n))

    def time(self, k):
        """Seconds to solve k systems (chunks of fresh copies)."""
        total, done = 0.0, 0
        while done < k:
            c = min(self.CHUNK, k - done)
            pick = self.rng.integers(0, self.POOL, c)
            As = [self.pool[i][0].copy() for i in pick]
            Bs = [self.pool[i][1].copy() for i in pick]
            nn = [self.pool[i][2] for i in pick]
            t0 = time.perf_counter()
            if self.lapack:
                self.orc.lapack_posv1_vbatch(nn, As, nn, Bs, nthreads=self.nth)
            else:
                self.orc.posv_vbatch([1] * c, nn, As, nn, Bs, [1] * c, nthreads=self.nth)
            total += time.perf_counter() - t0
            done += c
        return total

    def size_for(self, seconds):
        dt = self.time(2000)
        return int(min(5_000_000, max(2000, 2000 * seconds / max(dt, 1e-3))))

    def describe(self, k, dt):
        return (f"{k} systems drawn from the same n distribution (pool of {self.POOL} distinct, "
                f"{self.solver}, OpenMP over the batch, {self.nth} threads), {dt:.1f} s")


def cpu_baseline(orc, wl, seconds_target=15.0, seed=0):
    """The CPU path timed on one bounded sample of the workload."""
    cs = CpuSample(orc, wl, seed)
    k = cs.size_for(seconds_target)
    dt = cs.time(k)
    return {"value": k / dt, "unit": "solves/s", "cores": cs.nth, "kind": "port",
            "sample": cs.describe(k, dt)}


def read_traffic():
    """DRAM traffic per launch of the persistent mixed kernel, from the
    committed ncu summary (null when absent)."""
    path = os.path.join(ROOT, "profiles", "posv_vbatch_mixed_n8-256.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def run_reference(args):
    """The reference path's CPU implementation on the host cores: every step
    solves its own bounded sample of the workload (sized so that the whole run
    takes about a minute); the value is the median rate over the steps."""
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    kb, wl = load_pkg()
    from oracle import oracle as orc
    orc.build()
    cs = CpuSample(orc, wl)
    k = cs.size_for(max(1.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cs.time(k)
    dts = [cs.time(k) for _ in range(args.steps)]
    v = float(np.median([k / dt for dt in dts]))
    line = {"metric": METRIC, "value": v, "unit": "solves/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.median(dts)) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "step": f"one sample of {k} systems per step"},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cs.nth, "kind": "port",
                             "sample": cs.describe(k, float(np.sum(dts)))},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ----------------------------------------------------------------------------
# the other configurations of the path (one JSON line each, --workload NAME)
# ----------------------------------------------------------------------------
def _flops_potrf(n):
    return n ** 3 / 3.0 + n ** 2 / 2.0 + n / 6.0  # reference testing/flops.h POTRF


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _roof(fp64_peak, flops, bytes_, ms, peaks):
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    gbs = bytes_ / (ms * 1e-3) / 1e9
    tf = flops / (ms * 1e-3) / 1e12
    return {"roofline": {"bound": "fp64 pipe (no FP64 tensor path on this part)",
                         "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": tf / fp64_peak, "traffic": None,
                         "peak_source": "FP64 FMA chains measured live in this run (fp64_pipe)"},
            "hbm": {"achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm}}


class Ctx:
    """What the configuration runners share: the package, the oracle, one
    handle on the current stream, the peaks."""

    def __init__(self, args, torch, kb, wl, orc, h, stream, fp64_probe, peaks):
        self.args, self.torch, self.kb, self.wl, self.orc = args, torch, kb, wl, orc
        self.h, self.stream = h, stream
        self.fp64 = fp64_probe
        self.fp64_peak = fp64_probe["peak_tflops_measured_live"]
        self.peaks = peaks
        self.rng = np.random.default_rng(1)

    def steps(self, k=None):
        return k if k is not None else self.args.steps


def _cpu_time(fn, make, seconds):
    """Repeat fn(*make()) (inputs made outside the timer) for about `seconds`;
    returns (calls, time)."""
    spent, reps = 0.0, 0
    while spent < seconds or reps == 0:
        inp = make()
        t0 = time.perf_counter()
        fn(*inp)
        spent += time.perf_counter() - t0
        reps += 1
    return reps, spent


def cfg_potrf_potrs_n32(c, cpu_seconds=3.0):
    """DPOTRF + DPOTRS, 10000 x n = 32, strided, one RHS. One timed step runs
    REPS back-to-back POTRF + POTRS pairs, each on its own copy of the batch
    (REPS x 82 MB, larger than L2), inside one CUDA event pair."""
    torch, kb, h, orc, wl = c.torch, c.kb, c.h, c.orc, c.wl
    batch, n, reps = 10_000, 32, c.args.reps
    a = wl.spd_shifted(batch, n, seed=0)
    b = wl.rhs_rows(batch, 1, n, seed=0)
    A0, B0 = _dev(torch, a), _dev(torch, b)
    As = A0.unsqueeze(0).repeat(reps, 1, 1, 1)
    Bs = B0.unsqueeze(0).repeat(reps, 1, 1, 1)
    info = torch.zeros(reps, batch, dtype=torch.int32, device="cuda")
    s2 = n * n

    def step():
        for r in range(reps):
            kb.check(c.h.call("kblasDpotrf_batch_strided", "L", n, As[r].data_ptr(), n, s2, batch,
                              info[r].data_ptr()), "potrf")
            kb.check(c.h.call("kblasDpotrs_batch_strided", "R", "L", 1, n, As[r].data_ptr(), n,
                              s2, Bs[r].data_ptr(), 1, n, batch), "potrs")

    def restore():
        As.copy_(A0.unsqueeze(0).expand_as(As))
        Bs.copy_(B0.unsqueeze(0).expand_as(Bs))

    with ClockSampler(0) as clk:
        t = timed_steps(torch, step, restore, c.steps(), c.args.warmup, c.stream)
    ms_step = float(np.mean(t))
    ms = ms_step / reps  # one POTRF + POTRS pair over the batch
    X = Bs[reps - 1].cpu().numpy()
    pick = c.rng.choice(batch, 500, replace=False)
    eta = orc.backward_error_r(a[pick], X[pick], b[pick], 1, n)
    la = a[pick].copy()
    info_ref = orc.potrf_batch(la, n)
    L_ = As[reps - 1].cpu().numpy()
    fac = max(orc.lower_rel_diff(L_[i], la[k], n) for k, i in enumerate(pick[:100]))
    flops = batch * (_flops_potrf(n) + 2.0 * n * n)
    bytes_ = batch * (8.0 * n * (n + 1) + 16.0 * n)
    # CPU: the host LAPACK (dpotrf + dpotrs per matrix, OpenMP over the batch)
    ca, cb = a[:2000].copy(), b[:2000].reshape(2000, 1, n).copy()
    lp = orc.host_lapack()
    if lp:
        k, dt = _cpu_time(lambda x, y: orc.lapack_posv_batch(x, y), lambda: (ca.copy(), cb.copy()),
                          cpu_seconds)
        solver = lp[2]
    else:
        k, dt = _cpu_time(lambda x, y: orc.posv_batch(x, y, 1, n),
                          lambda: (ca.copy(), b[:2000].copy()), cpu_seconds)
        solver = "FP64 POTRF+POTRS, C restatement of LAPACK"
    d = {"metric": "batched DPOTRF+DPOTRS solves/s (n=32)", "value": batch / (ms * 1e-3),
         "unit": "solves/s", "ms_per_step": ms_step, "ms_per_call_pair": ms,
         "fp64_gflops": flops / (ms * 1e-3) / 1e9,
         "accuracy": {"checked": 500, "max_eta_over_10n_eps": float(eta.max() / (10 * n * EPS64)),
                      "max_factor_rel_diff_vs_oracle": float(fac),
                      "info_exact": bool(np.array_equal(info[reps - 1].cpu().numpy()[pick],
                                                        info_ref))},
         "gpu_launches": 2 * reps * c.steps(), "clocks": clk.summary(),
         "cpu_baseline": {"value": 2000 * k / dt, "unit": "solves/s", "cores": os.cpu_count(),
                          "kind": "port",
                          "sample": f"2000 systems x {k} passes ({solver}, OpenMP over the batch)"},
         "config": {"workload": "DPOTRF + DPOTRS, 10000 x n=32, strided, lda=32, 1 RHS, "
                                "A = G G^T + 32 I",
                    "timing": f"{reps} back-to-back POTRF+POTRS pairs per step, each on its own "
                              f"copy of the batch ({reps * a.nbytes / 1e9:.1f} GB, larger than "
                              f"L2), one CUDA event pair; value from the mean step"}}
    d.update(_roof(c.fp64_peak, flops, bytes_, ms, c.peaks))
    return d


def cfg_trsm_trmm_syrk_n64(c, cpu_seconds=3.0):
    torch, kb, h, orc, wl = c.torch, c.kb, c.h, c.orc, c.wl
    batch, n = 20_000, 64
    L_ = wl.lower_tri(batch, n, seed=0, upper_fill=0.0)
    Bm = wl.general(batch, n, n, seed=1)
    Cs = wl.spd_shifted(batch, n, seed=2)
    Am = wl.general(batch, n, n, seed=3)
    dL, dB0, dC0, dA = _dev(torch, L_), _dev(torch, Bm), _dev(torch, Cs), _dev(torch, Am)
    dB, dC = dB0.clone(), dC0.clone()
    s2 = n * n
    res = {}
    pL = torch.from_numpy(dL.data_ptr() + np.arange(batch, dtype=np.int64) * s2 * 8).cuda()
    pB = torch.from_numpy(dB.data_ptr() + np.arange(batch, dtype=np.int64) * s2 * 8).cuda()
    pA = torch.from_numpy(dA.data_ptr() + np.arange(batch, dtype=np.int64) * s2 * 8).cuda()
    pC = torch.from_numpy(dC.data_ptr() + np.arange(batch, dtype=np.int64) * s2 * 8).cuda()
    ops = {
        "trsm_strided": lambda: h.call("kblasDtrsm_batch_strided", "L", "L", "N", "N", n, n, 1.0,
                                       dL.data_ptr(), n, s2, dB.data_ptr(), n, s2, batch),
        "trmm_strided": lambda: h.call("kblasDtrmm_batch_strided", "L", "L", "N", "N", n, n, 1.0,
                                       dL.data_ptr(), n, s2, dB.data_ptr(), n, s2, batch),
        "syrk_strided": lambda: h.call("kblasDsyrk_batch_strided", "L", "N", n, n, -1.0,
                                       dA.data_ptr(), n, s2, 1.0, dC.data_ptr(), n, s2, batch),
        "trsm_array": lambda: h.call("kblasDtrsm_batch", "L", "L", "N", "N", n, n, 1.0,
                                     pL.data_ptr(), n, pB.data_ptr(), n, batch),
        "trmm_array": lambda: h.call("kblasDtrmm_batch", "L", "L", "N", "N", n, n, 1.0,
                                     pL.data_ptr(), n, pB.data_ptr(), n, batch),
        "syrk_array": lambda: h.call("kblasDsyrk_batch", "L", "N", n, n, -1.0, pA.data_ptr(), n,
                                     1.0, pC.data_ptr(), n, batch),
    }
    with ClockSampler(0) as clk:
        for name, fn in ops.items():
            def call(fn=fn, name=name):
                kb.check(fn(), name)
            restore = (lambda: dC.copy_(dC0)) if name.startswith("syrk") else (lambda: dB.copy_(dB0))
            t = timed_steps(torch, call, restore, c.steps(), c.args.warmup, c.stream)
            ms = float(np.mean(t))
            if name.startswith("syrk"):
                flops = batch * n * n * (n + 1.0)
                bytes_ = batch * (8.0 * n * n + 16.0 * n * (n + 1) / 2)
            else:
                flops = batch * float(n) * n * n
                bytes_ = batch * (8.0 * n * (n + 1) / 2 + 16.0 * n * n)
            res[name] = {"ms": ms, "gflops": flops / (ms * 1e-3) / 1e9,
                         "gbs": bytes_ / (ms * 1e-3) / 1e9,
                         "fp64_frac": flops / (ms * 1e-3) / 1e12 / c.fp64_peak}
    # accuracy on a sample against the oracle (strided forms)
    pick = c.rng.choice(batch, 200, replace=False)
    dB.copy_(dB0)
    kb.check(ops["trsm_strided"](), "trsm")
    X = dB.cpu().numpy()[pick]
    ref = Bm[pick].copy()
    orc.trsm_batch("L", "L", "N", "N", n, n, 1.0, L_[pick].copy(), ref)
    trsm_err = float(np.abs(X - ref).max() / np.abs(ref).max())
    dB.copy_(dB0)
    kb.check(ops["trmm_strided"](), "trmm")
    X = dB.cpu().numpy()[pick]
    ref = Bm[pick].copy()
    orc.trmm_batch("L", "L", "N", "N", n, n, 1.0, L_[pick].copy(), ref)
    trmm_err = float(np.abs(X - ref).max() / np.abs(ref).max())
    dC.copy_(dC0)
    kb.check(ops["syrk_strided"](), "syrk")
    Cg = dC.cpu().numpy()[pick]
    Cr = Cs[pick].copy()
    orc.syrk_batch("L", "N", n, n, -1.0, Am[pick].copy(), 1.0, Cr)
    low = np.tril(np.ones((n, n), bool)).T  # column-major lower = upper of the stored array
    syrk_err = float(np.abs((Cg - Cr)[:, low]).max() / np.abs(Cr[:, low]).max())
    # CPU: the oracle's TRSM (C restatement of BLAS xTRSM), OpenMP over the batch
    cl, cb = L_[:2000].copy(), Bm[:2000]
    k, dt = _cpu_time(lambda x, y: orc.trsm_batch("L", "L", "N", "N", n, n, 1.0, x, y),
                      lambda: (cl, cb.copy()), cpu_seconds)
    ms = res["trsm_strided"]["ms"]
    d = {"metric": "batched DTRSM GFLOP/s (64x64, strided; TRMM/SYRK in ops)",
         "value": res["trsm_strided"]["gflops"], "unit": "GFLOP/s", "ms_per_step": ms,
         "ops": res,
         "accuracy": {"trsm_rel_err_vs_oracle": trsm_err, "trmm_rel_err_vs_oracle": trmm_err,
                      "syrk_rel_err_vs_oracle": syrk_err},
         "gpu_launches": 6 * c.steps(), "clocks": clk.summary(),
         "cpu_baseline": {"value": 2000 * k * float(n) ** 3 / dt / 1e9, "unit": "GFLOP/s",
                          "cores": os.cpu_count(), "kind": "port",
                          "sample": f"DTRSM L,L,N,N 64x64, 2000 matrices x {k} passes (oracle's "
                                    f"C restatement of BLAS xTRSM, OpenMP over the batch)"},
         "config": {"workload": "DTRSM / DTRMM L,L,N,N 64x64 and DSYRK L,N 64x64, 20000 "
                                "matrices, strided and pointer-array; value from the mean step"}}
    d.update(_roof(c.fp64_peak, batch * float(n) ** 3,
                   batch * (8.0 * n * (n + 1) / 2 + 16.0 * n * n), ms, c.peaks))
    return d


def cfg_posv_mixed(c, which, cpu_seconds=4.0):
    """Mixed vs plain FP64 uniform DPOSV: the n = 64 conditioned batch with 4
    RHS, or the n = 512 covariances with 8 RHS."""
    torch, kb, h, orc, wl = c.torch, c.kb, c.h, c.orc, c.wl
    if which == "mixed_posv_n64":
        batch, n, m = min(50_000, c.args.batch), 64, 4
        a, cond = wl.spd_cond(batch, n, seed=0)
        desc = (f"mixed vs FP64 DPOSV, {batch} x n=64, cond log-uniform 1e2..1e8 (Q diag Q^T), "
                "4 RHS, strided")
    else:
        # --batch below 2000 shrinks the batch (whole hundreds), for profiler captures
        batch, n, m = max(100, min(2_000, c.args.batch) // 100 * 100), 512, 8
        a = np.concatenate([wl.sqexp_cov(100, n, seed=k) for k in range(batch // 100)])
        desc = (f"mixed vs FP64 DPOSV, {batch} x n=512 squared-exponential covariances, "
                "l ~ U[0.05, 0.3], nugget 1e-4, 8 RHS, strided")
    b = wl.rhs_rows(batch, m, n, seed=1)
    A0, B0 = _dev(torch, a), _dev(torch, b)
    A, B = A0.clone(), B0.clone()
    info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    it = torch.zeros(batch, dtype=torch.int32, device="cuda")
    kb.lib().kblas_posv_batch_mixed_wsquery(h.ptr, b"R", m, n, batch)
    kb.lib().kblas_posv_batch_strided_wsquery(h.ptr, b"R", m, n, batch)
    kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")

    def restore():
        A.copy_(A0)
        B.copy_(B0)

    def mixed():
        kb.check(h.call("kblasDposv_batch_mixed_strided", "R", "L", m, n, A.data_ptr(), n, n * n,
                        B.data_ptr(), m, m * n, batch, info.data_ptr(), it.data_ptr()), "mixed")

    def fp64():
        kb.check(h.call("kblasDposv_batch_strided", "R", "L", m, n, A.data_ptr(), n, n * n,
                        B.data_ptr(), m, m * n, batch, info.data_ptr()), "posv")

    with ClockSampler(0) as clk:
        tm = timed_steps(torch, mixed, restore, c.steps(), c.args.warmup, c.stream)
    Xm, itm, infom = B.cpu().numpy(), it.cpu().numpy(), info.cpu().numpy()
    status = h.device_status()
    tf = timed_steps(torch, fp64, restore, max(2, c.steps() // 2), 2, c.stream)
    Xf, infof = B.cpu().numpy(), info.cpu().numpy()
    ms_m, ms_f = float(np.mean(tm)), float(np.mean(tf))
    ok = infof == 0
    pick = np.where(ok)[0]
    pick = pick[c.rng.choice(len(pick), min(len(pick), 400), replace=False)]
    eta_m = orc.backward_error_r(a[pick], Xm[pick], b[pick], m, n)
    eta_f = orc.backward_error_r(a[pick], Xf[pick], b[pick], m, n)
    fwd = np.abs(Xm[pick] - Xf[pick]).max(axis=(1, 2)) / np.abs(Xf[pick]).max(axis=(1, 2))
    ref_a, ref_b = a[pick].copy(), b[pick].copy()
    info_o = orc.posv_batch(ref_a, ref_b, m, n)
    den = np.abs(ref_b).max(axis=(1, 2))
    fwd_om = np.abs(Xm[pick] - ref_b).max(axis=(1, 2)) / den
    fwd_of = np.abs(Xf[pick] - ref_b).max(axis=(1, 2)) / den
    flops = batch * (_flops_potrf(n) + 2.0 * m * n * n)
    # CPU: host LAPACK dpotrf + dpotrs per system (B as n x m, LAPACK's layout)
    ns = min(batch, 2000 if n <= 64 else 200)
    ca = a[:ns].copy()
    # b[k][i][r] = B(r, i); LAPACK solves A Y = B^T with Y n x m column-major:
    # [k][r][i] = B(r, i)
    cbt = np.ascontiguousarray(b[:ns].transpose(0, 2, 1))
    lp = orc.host_lapack()
    if lp:
        k, dt = _cpu_time(lambda x, y: orc.lapack_posv_batch(x, y), lambda: (ca.copy(), cbt.copy()),
                          cpu_seconds)
        solver = lp[2]
    else:
        k, dt = _cpu_time(lambda x, y: orc.posv_batch(x, y, m, n), lambda: (ca.copy(), b[:ns].copy()),
                          cpu_seconds)
        solver = "FP64 POTRF+POTRS, C restatement of LAPACK"
    d = {"metric": f"batched POSV solves/s (n={n}, {m} RHS): mixed-prec vs plain FP64",
         "value": batch / (ms_m * 1e-3), "unit": "solves/s", "ms_per_step": ms_m,
         "fp64_form": {"value": batch / (ms_f * 1e-3), "unit": "solves/s", "ms_per_step": ms_f,
                       "max_eta_over_10n_eps": float(eta_f.max() / (10 * n * EPS64))},
         "mixed_over_fp64": ms_f / ms_m,
         "accuracy": {"checked": int(len(pick)),
                      "max_eta_over_10n_eps": float(eta_m.max() / (10 * n * EPS64)),
                      "all_within_bound": bool((eta_m <= 10 * n * EPS64).all()),
                      "max_forward_rel_diff_vs_fp64": float(fwd.max()),
                      "max_forward_rel_err_vs_oracle": float(fwd_om.max()),
                      "fp64_form_max_forward_rel_err_vs_oracle": float(fwd_of.max()),
                      "oracle_info_equal": bool(np.array_equal(info_o, infom[pick])),
                      "info_equal_to_fp64_form": bool(np.array_equal(infom, infof))},
         "refinement": {"mean_steps": float(itm[itm >= 0].mean()) if (itm >= 0).any() else None,
                        "fallback_systems": int((itm < 0).sum()),
                        "fallback_codes": {str(k_): int((itm == k_).sum()) for k_ in (-1, -2, -3, -4)
                                           if (itm == k_).any()}},
         "device_status": int(status),
         "gpu_launches": c.steps(), "clocks": clk.summary(),
         "cpu_baseline": {"value": ns * k / dt, "unit": "solves/s", "cores": os.cpu_count(),
                          "kind": "port",
                          "sample": f"{ns} systems x {k} passes ({solver}, OpenMP over the batch)"},
         "config": {"workload": desc, "timing": "value from the mean step"}}
    d.update(_roof(c.fp64_peak, flops, batch * (8.0 * n * (n + 1) + 16.0 * n * m), ms_f, c.peaks))
    d["roofline"]["note"] = "roofline of the FP64 form (the mixed form uses FP32 + FP64)"
    return d


def cfg_inverse_n64(c):
    torch, kb, h, orc, wl = c.torch, c.kb, c.h, c.orc, c.wl
    batch, n = 20_000, 64
    a = wl.spd_shifted(batch, n, seed=0)
    Lh = a.copy()
    orc.potrf_batch(Lh, n)
    A0, L0 = _dev(torch, a), _dev(torch, Lh)
    W_ = A0.clone()
    info = torch.zeros(batch, dtype=torch.int32, device="cuda")
    fl = {"trtri": n ** 3 / 3.0, "lauum": n ** 3 / 3.0, "potri": 2 * n ** 3 / 3.0, "poti": n ** 3}
    res = {}
    for op in ("trtri", "lauum", "potri", "poti"):
        src = A0 if op == "poti" else L0
        flags = ("L", "N") if op == "trtri" else ("L",)

        def fn(op=op, flags=flags):
            kb.check(h.call(f"kblasD{op}_batch_strided", *flags, n, W_.data_ptr(), n, n * n,
                            batch, info.data_ptr()), op)
        t = timed_steps(torch, fn, lambda src=src: W_.copy_(src), c.steps(), c.args.warmup,
                        c.stream)
        ms = float(np.mean(t))
        res[op] = {"ms": ms, "gflops": batch * fl[op] / (ms * 1e-3) / 1e9,
                   "fp64_frac": batch * fl[op] / (ms * 1e-3) / 1e12 / c.fp64_peak}
    pick = c.rng.choice(batch, 200, replace=False)
    W_.copy_(A0)
    kb.check(h.call("kblasDpoti_batch_strided", "L", n, W_.data_ptr(), n, n * n, batch,
                    info.data_ptr()), "poti")
    got = W_.cpu().numpy()[pick]
    ref = a[pick].copy()
    orc.poti_batch(ref, n)
    low = np.triu(np.ones((n, n), bool))
    err = float(np.abs((got - ref)[:, low]).max() / np.abs(ref[:, low]).max())
    cs = a[:2000]
    k, dt = _cpu_time(lambda x: orc.poti_batch(x, n), lambda: (cs.copy(),), 3.0)
    ms = res["poti"]["ms"]
    d = {"metric": "batched DPOTI inverses/s (n=64; TRTRI/LAUUM/POTRI in ops)",
         "value": batch / (ms * 1e-3), "unit": "inverses/s", "ms_per_step": ms, "ops": res,
         "accuracy": {"poti_rel_err_vs_oracle": err},
         "gpu_launches": c.steps(),
         "cpu_baseline": {"value": 2000 * k / dt, "unit": "inverses/s", "cores": os.cpu_count(),
                          "kind": "port", "sample": f"POTI, 2000 matrices x {k} passes"},
         "config": {"workload": "DTRTRI / DLAUUM / DPOTRI / DPOTI, 20000 x n=64, strided, "
                                "lower, A = G G^T + 64 I"}}
    d.update(_roof(c.fp64_peak, batch * fl["poti"], batch * 16.0 * n * (n + 1) / 2, ms, c.peaks))
    return d


def make_ctx(args, torch, kb, wl, orc, h, stream):
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    return Ctx(args, torch, kb, wl, orc, h, stream, measure_fp64_peak(kb, torch), peaks)


CONFIGS = {
    "potrf_potrs_n32": cfg_potrf_potrs_n32,
    "trsm_trmm_syrk_n64": cfg_trsm_trmm_syrk_n64,
    "mixed_posv_n64": lambda c: cfg_posv_mixed(c, "mixed_posv_n64"),
    "posv_n512": lambda c: cfg_posv_mixed(c, "posv_n512"),
    "inverse_n64": cfg_inverse_n64,
    "gemm_vbatch": lambda c: run_gemm_vbatch(c),
}


def run_workload(args):
    """One configuration besides the variable-size headline, as its own JSON
    line."""
    import torch
    torch.cuda.set_device(0)
    kb, wl = load_pkg()
    from oracle import oracle as orc
    orc.build()
    stream = torch.cuda.current_stream()
    h = kb.Handle(stream=stream.cuda_stream)
    c = make_ctx(args, torch, kb, wl, orc, h, stream)
    d = CONFIGS[args.workload](c)
    line = {"metric": d.pop("metric"), "value": d.pop("value"), "unit": d.pop("unit"), "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": d.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "fp64_pipe": c.fp64}
    line.update(d)
    print(json.dumps(line))
    return 0


def run_gemm_vbatch(c):
    """Batched DGEMM (uniform 64^3, beside cuBLAS through torch.bmm, which is
    what the reference's uniform GEMM calls) and the variable-size DGEMM /
    DSYRK / DTRSM, sizes uniform in 16..128, pointer arrays."""
    args, torch, kb, wl, orc, h, stream = c.args, c.torch, c.kb, c.wl, c.orc, c.h, c.stream
    fp64_peak, peaks, rng = c.fp64_peak, c.peaks, c.rng
    res = {}
    # uniform: 20000 x 64x64x64, C := A B + C (--batch below 20000 shrinks both
    # parts, for profiler captures)
    batch, n = min(20_000, args.batch), 64
    A = torch.randn(batch, n, n, dtype=torch.float64, device="cuda")
    B = torch.randn(batch, n, n, dtype=torch.float64, device="cuda")
    C0 = torch.randn(batch, n, n, dtype=torch.float64, device="cuda")
    C = C0.clone()
    s2 = n * n

    def ours():
        kb.check(h.call("kblasDgemm_batch_strided", "N", "N", n, n, n, 1.0, A.data_ptr(), n, s2,
                        B.data_ptr(), n, s2, 1.0, C.data_ptr(), n, s2, batch), "gemm")

    def cublas():
        # column-major C = A B + C is row-major C^T = B^T A^T + C^T: same bytes, same flops
        C.baddbmm_(B, A)

    flops_u = 2.0 * batch * n ** 3
    for name, fn in (("dgemm_uniform_64", ours), ("cublas_bmm_uniform_64", cublas)):
        t = timed_steps(torch, fn, lambda: C.copy_(C0), args.steps, args.warmup, stream)
        ms = float(np.mean(t))
        res[name] = {"ms": ms, "gflops": flops_u / (ms * 1e-3) / 1e9,
                     "fp64_frac": flops_u / (ms * 1e-3) / 1e12 / fp64_peak}
    C.copy_(C0)
    ours()
    ref = torch.baddbmm(C0, B, A)
    uni_err = float(((C - ref).abs().max() / ref.abs().max()).item())

    # variable size
    vb = min(20_000, args.batch)
    ms_ = rng.integers(16, 129, vb).astype(np.int32)
    ns_ = rng.integers(16, 129, vb).astype(np.int32)
    ks_ = rng.integers(16, 129, vb).astype(np.int32)
    mx = 128

    def pool(rows, cols):
        sizes = rows.astype(np.int64) * cols
        offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
        buf = torch.randn(int(sizes.sum()), dtype=torch.float64, device="cuda")
        ptrs = torch.from_numpy(buf.data_ptr() + offs * 8).cuda()
        return buf, ptrs, offs

    Ab, pA, oA = pool(ms_, ks_)
    Bb, pB, oB = pool(ks_, ns_)
    Cb0, pC, oC = pool(ms_, ns_)
    Cb = Cb0.clone()
    pC = torch.from_numpy(Cb.data_ptr() + oC * 8).cuda()
    dm, dn, dk = (torch.from_numpy(v).cuda() for v in (ms_, ns_, ks_))

    def vgemm():
        kb.check(h.call("kblasDgemm_vbatch", "N", "N", dm.data_ptr(), dn.data_ptr(), dk.data_ptr(),
                        mx, mx, mx, 1.0, pA.data_ptr(), dm.data_ptr(), pB.data_ptr(),
                        dk.data_ptr(), 1.0, pC.data_ptr(), dm.data_ptr(), vb), "gemm_vbatch")

    # SYRK: C_i (m_i x m_i) := -A_i A_i^T + C_i with A_i = the m_i x k_i GEMM operand;
    # TRSM: L_i X = B, L_i the leading m_i x m_i block of C_i made well conditioned
    Sb0, pS, oS = pool(ms_, ms_)
    Sb = Sb0.clone()
    pS = torch.from_numpy(Sb.data_ptr() + oS * 8).cuda()
    Lb = Sb0.clone()
    # diagonally dominant lower triangles: scale the pool, then add 2 on the diagonals
    Lb.mul_(0.1)
    diag_idx = np.concatenate([o + np.arange(m) * (m + 1) for o, m in zip(oS, ms_)])
    Lb[torch.from_numpy(diag_idx).cuda()] += 2.0
    pL = torch.from_numpy(Lb.data_ptr() + oS * 8).cuda()
    Xb0, pX, oX = pool(ms_, ns_)
    Xb = Xb0.clone()
    pX = torch.from_numpy(Xb.data_ptr() + oX * 8).cuda()

    def vsyrk():
        kb.check(h.call("kblasDsyrk_vbatch", "L", "N", dm.data_ptr(), dk.data_ptr(), mx, mx, -1.0,
                        pA.data_ptr(), dm.data_ptr(), 1.0, pS.data_ptr(), dm.data_ptr(), vb),
                 "syrk_vbatch")

    def vtrsm():
        kb.check(h.call("kblasDtrsm_vbatch", "L", "L", "N", "N", dm.data_ptr(), dn.data_ptr(), mx,
                        mx, 1.0, pL.data_ptr(), dm.data_ptr(), pX.data_ptr(), dm.data_ptr(), vb),
                 "trsm_vbatch")

    fl = {"dgemm_vbatch": float(2.0 * (ms_.astype(np.float64) * ns_ * ks_).sum()),
          "dsyrk_vbatch": float((ms_.astype(np.float64) * (ms_ + 1) * ks_).sum()),
          "dtrsm_vbatch": float((ms_.astype(np.float64) ** 2 * ns_).sum())}
    with ClockSampler(0) as clk:
        for name, fn, rst in (("dgemm_vbatch", vgemm, lambda: Cb.copy_(Cb0)),
                              ("dsyrk_vbatch", vsyrk, lambda: Sb.copy_(Sb0)),
                              ("dtrsm_vbatch", vtrsm, lambda: Xb.copy_(Xb0))):
            t = timed_steps(torch, fn, rst, args.steps, args.warmup, stream)
            ms = float(np.mean(t))
            res[name] = {"ms": ms, "gflops": fl[name] / (ms * 1e-3) / 1e9,
                         "fp64_frac": fl[name] / (ms * 1e-3) / 1e12 / fp64_peak}
    # accuracy of the variable-size GEMM on a sample against the oracle
    Cb.copy_(Cb0)
    vgemm()
    Ch, Ah, Bh, C0h = Cb.cpu().numpy(), Ab.cpu().numpy(), Bb.cpu().numpy(), Cb0.cpu().numpy()
    worst = 0.0
    for i in rng.choice(vb, 100, replace=False):
        m, nn, k = int(ms_[i]), int(ns_[i]), int(ks_[i])
        a = Ah[oA[i]:oA[i] + m * k].reshape(1, k, m).copy()
        b = Bh[oB[i]:oB[i] + k * nn].reshape(1, nn, k).copy()
        c = C0h[oC[i]:oC[i] + m * nn].reshape(1, nn, m).copy()
        orc.gemm_batch("N", "N", m, nn, k, 1.0, a, b, 1.0, c, nthreads=1)
        got = Ch[oC[i]:oC[i] + m * nn].reshape(1, nn, m)
        worst = max(worst, float(np.abs(got - c).max() / np.abs(c).max()))
    # CPU baseline: the oracle's DGEMM over a sample of the variable-size batch
    sample = rng.choice(vb, 400, replace=False)
    t0 = time.perf_counter()
    done_fl = 0.0
    while time.perf_counter() - t0 < 3.0:
        for i in sample[:40]:
            m, nn, k = int(ms_[i]), int(ns_[i]), int(ks_[i])
            a = Ah[oA[i]:oA[i] + m * k].reshape(1, k, m)
            b = Bh[oB[i]:oB[i] + k * nn].reshape(1, nn, k)
            c = C0h[oC[i]:oC[i] + m * nn].reshape(1, nn, m).copy()
            orc.gemm_batch("N", "N", m, nn, k, 1.0, a, b, 1.0, c, nthreads=1)
            done_fl += 2.0 * m * nn * k
    cpu_gf = done_fl / (time.perf_counter() - t0) / 1e9
    ms = res["dgemm_vbatch"]["ms"]
    ex = {"ops": res,
          "accuracy": {"uniform_rel_err_vs_cublas": uni_err, "vbatch_rel_err_vs_oracle": worst},
          "gpu_launches": 5 * args.steps, "clocks": clk.summary(),
          "cpu_baseline": {"value": cpu_gf, "unit": "GFLOP/s", "cores": 1, "kind": "port",
                           "sample": "oracle DGEMM (scalar C loops) on 40 of the variable-size "
                                     "products, repeated for 3 s, one thread"},
          "config": {"workload": f"DGEMM N,N: uniform {batch} x 64^3 strided (and cuBLAS via "
                                 f"torch.baddbmm beside it); variable-size DGEMM / DSYRK L,N / "
                                 f"DTRSM L,L,N,N over {vb} matrices, m, n, k uniform in 16..128, "
                                 f"pointer arrays, sizes in device arrays"}}
    bytes_ = 8.0 * float((ms_.astype(np.float64) * ks_ + ks_ * ns_ + 2.0 * ms_ * ns_).sum())
    ex.update(_roof(fp64_peak, fl["dgemm_vbatch"], bytes_, ms, peaks))
    ex.update({"metric": "variable-size batched DGEMM GFLOP/s (m, n, k in 16..128)",
               "value": res["dgemm_vbatch"]["gflops"], "unit": "GFLOP/s", "ms_per_step": ms})
    return ex


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--batch", type=int, default=100_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--reps", type=int, default=100,
                    help="potrf_potrs_n32: POTRF + POTRS pairs per step, each on its own copy "
                         "of the 82 MB batch (fewer for profiler captures)")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the other configurations after the variable-size headline")
    ap.add_argument("--workload", default="vbatch",
                    choices=["vbatch", "potrf_potrs_n32", "trsm_trmm_syrk_n64", "mixed_posv_n64",
                             "posv_n512", "inverse_n64", "gemm_vbatch"])
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "vbatch":
        return run_workload(args)

    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    kb, wl = load_pkg()
    from oracle import oracle as orc
    orc.build()
    kb.lib()
    stream = torch.cuda.current_stream()
    h = kb.Handle(stream=stream.cuda_stream)
    # weak scaling: the global batch holds --batch systems per rank, split into
    # contiguous work-balanced ranges
    w = VWorkload(torch, wl, batch=args.batch * world, shard=(rank, world))
    w.keep_pristine()
    kb.lib().kblas_posv_vbatch_wsquery(h.ptr, w.max_n, w.batch)
    kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- mixed precision, inputs resident in HBM ----
    barrier()
    with ClockSampler(local) as clk:
        t_mixed = timed_steps(torch, lambda: call_vbatch(kb, h, w, True), lambda: w.restore(),
                              args.steps, args.warmup, stream)
    barrier()
    acc_mixed = accuracy_check(orc, w, torch)
    it = w.iter.cpu().numpy()
    info = w.info.cpu().numpy()
    x_mixed = w.B.cpu()
    # ---- plain FP64 ----
    t_fp64 = timed_steps(torch, lambda: call_vbatch(kb, h, w, False), lambda: w.restore(full=True),
                         max(2, args.steps // 2), 2, stream)
    acc_fp64 = accuracy_check(orc, w, torch)
    w.restore(full=True)
    # ---- end to end through the C ABI with pinned host buffers ----
    hA = torch.empty(w.pool_elems, dtype=torch.float64, pin_memory=True)
    hB = torch.empty(w.B0.numel(), dtype=torch.float64, pin_memory=True)
    hX = torch.empty_like(hB, pin_memory=True)
    hinfo_all = torch.empty(w.batch, dtype=torch.int32, pin_memory=True)
    hA.copy_(w.A_pristine)
    hB.copy_(w.B0)

    # The batch is split into E2E_CHUNKS pieces that are contiguous in the
    # matrix pool (equal bytes); the host->device copy of piece k+1 runs on a
    # copy stream while piece k is solved on the handle's stream -- the usual
    # way to feed a GPU library from host memory, through the same C ABI call.
    order = np.argsort(w.offs, kind="stable")
    nbytes = w.ns[order].astype(np.int64) ** 2
    cum = np.cumsum(nbytes)
    cuts = [0] + [int(np.searchsorted(cum, cum[-1] * k / E2E_CHUNKS)) + 1
                  for k in range(1, E2E_CHUNKS)] + [w.batch]
    chunks = []
    for lo, hi in zip(cuts[:-1], cuts[1:]):
        if hi <= lo:
            continue
        idx = order[lo:hi]
        it_ = torch.from_numpy(idx).to("cuda")
        a_lo = int(w.offs[idx[0]])
        a_hi = int(w.offs[idx[-1]]) + int(w.ns[idx[-1]]) ** 2
        c = {"n": len(idx), "a": (a_lo, a_hi), "max_n": int(w.ns[idx].max()),
             "pA": w.pA[it_], "pB": w.pB[it_], "dn": w.dn[it_], "dm": w.dm[it_],
             "dldb": w.dldb[it_], "info": torch.zeros(len(idx), dtype=torch.int32, device="cuda"),
             "iter": torch.zeros(len(idx), dtype=torch.int32, device="cuda"),
             "hinfo": hinfo_all[lo:hi],
             "ev": torch.cuda.Event()}
        kb.lib().kblas_posv_vbatch_wsquery(h.ptr, c["max_n"], c["n"])
        chunks.append(c)
    kb.check(h.allocate_workspace(), "kblasAllocateWorkspace")
    copy_stream = torch.cuda.Stream()
    ev_b = torch.cuda.Event()
    # per step: the duration of the host->device copies alone (copy stream) and
    # the host time spent issuing the step, so that a slow step can be told
    # apart -- slow copies, slow solves, or a host thread that stalled between
    # two of the step's 35 calls while the GPU waited for the next one
    h2d_events, host_ms = [], []

    def e2e_body(s, timing):
        copy_stream.wait_stream(s)
        eh = None
        if timing:
            eh = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            h2d_events.append(eh)
        with torch.cuda.stream(copy_stream):
            if eh:
                eh[0].record(copy_stream)
            w.B.copy_(hB, non_blocking=True)
            ev_b.record(copy_stream)
            for c in chunks:
                a_lo, a_hi = c["a"]
                w.A[a_lo:a_hi].copy_(hA[a_lo:a_hi], non_blocking=True)
                c["ev"].record(copy_stream)
            if eh:
                eh[1].record(copy_stream)
        s.wait_event(ev_b)
        for c in chunks:
            s.wait_event(c["ev"])
            st = h.call("kblasDposv_vbatch_mixed", "R", "L", c["dm"].data_ptr(), c["dn"].data_ptr(),
                        1, c["max_n"], c["pA"].data_ptr(), c["dn"].data_ptr(), c["pB"].data_ptr(),
                        c["dldb"].data_ptr(), c["n"], c["info"].data_ptr(), c["iter"].data_ptr())
            if st != 1:
                raise RuntimeError(f"kblasDposv_vbatch_mixed returned {st}")
        with torch.cuda.stream(s):
            hX.copy_(w.B, non_blocking=True)
            for c in chunks:
                c["hinfo"].copy_(c["info"], non_blocking=True)

    def e2e_step():
        t0 = time.perf_counter()
        e2e_body(stream, True)
        host_ms.append((time.perf_counter() - t0) * 1e3)

    xm = x_mixed.numpy()

    def e2e_results():
        torch.cuda.synchronize()
        e2e_info = np.zeros(w.batch, dtype=np.int32)
        for c, (lo, hi) in zip(chunks, [(a, b) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]):
            e2e_info[order[lo:hi]] = c["hinfo"].numpy()
        return {"info_equal": bool(np.array_equal(e2e_info, info)),
                "max_rel_diff_x": float(np.abs(hX.numpy() - xm).max() / np.abs(xm).max())}

    t_e2e_eager = timed_steps(torch, e2e_step, lambda: None, args.steps, args.warmup, stream)
    torch.cuda.synchronize()
    h2d_ms = [a.elapsed_time(b) for a, b in h2d_events[-args.steps:]]
    host_issue_ms = host_ms[-args.steps:]
    check_eager = e2e_results()
    # the host link alone: the same host->device copy of the matrix pool with
    # no solve running, repeated; its spread is the link's, not the solver's
    link_ms = []
    for _ in range(LINK_PROBE_REPS):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(copy_stream):
            e0.record(copy_stream)
            w.A.copy_(hA, non_blocking=True)
            e1.record(copy_stream)
        e1.synchronize()
        link_ms.append(e0.elapsed_time(e1))

    def agrees(chk):
        return chk is not None and chk["info_equal"] and chk["max_rel_diff_x"] <= 1e-10

    t_e2e, e2e_check = t_e2e_eager, check_eager
    h2d = w.pool_elems * 8 + w.B0.numel() * 8
    d2h = w.B0.numel() * 8 + w.batch * 4

    # ---- roofline of the persistent kernel ----
    sh = shard_mod()
    ms_mixed = sh.max_over_ranks(float(np.mean(t_mixed)))
    ms_fp64 = sh.max_over_ranks(float(np.mean(t_fp64)))
    # mean step, the statistic of `value` (median, min and max beside it)
    ms_e2e = sh.max_over_ranks(float(np.mean(t_e2e)))
    total_batch = int(sh.sum_over_ranks(w.batch))
    v_mixed = total_batch / (ms_mixed * 1e-3)
    v_fp64 = total_batch / (ms_fp64 * 1e-3)
    # an end-to-end run whose results differ from the resident run's (info
    # codes, or X beyond rounding of the summation order) has no rate
    e2e_valid = agrees(e2e_check)
    v_e2e = total_batch / (ms_e2e * 1e-3) if e2e_valid else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    ab = w.alg_bytes()
    achieved = ab / (ms_mixed * 1e-3) / 1e9
    fp64_rec = measure_fp64_peak(kb, torch)
    fp64_peak = fp64_rec["peak_tflops_measured_live"]
    steps_arr = it[(info == 0) & (it >= 0)]
    fp64_flops_refine = float((2.0 * w.ns.astype(np.float64) ** 2 *
                               np.where(it >= 0, it + 1, 0)).sum())
    useful = w.flops_useful()
    line = {
        "metric": METRIC, "value": v_mixed, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mixed,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 (FP32 factor, FP64 residual + update, FP64 fallback)",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "systems_per_gpu": w.batch,
                   "l2": "inputs (%.1f GB) larger than L2, no flush" % (w.pool_elems * 8 / 1e9),
                   "timing": "CUDA events around the library call per step; RHS and indefinite "
                             "matrices restored between steps outside the events"},
        "fp64_form": {"value": v_fp64, "unit": "solves/s", "ms_per_step": ms_fp64,
                      "accuracy": acc_fp64},
        "mixed_over_fp64": v_mixed / v_fp64,
        "accuracy": acc_mixed,
        "refinement": {"mean_steps": float(steps_arr.mean()) if len(steps_arr) else None,
                       "fallback_systems": int((it < 0).sum()),
                       "info_positive": int((info > 0).sum())},
        "gflops_useful": useful / (ms_mixed * 1e-3) / 1e9,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": read_traffic(),
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "note": "algorithmic bytes over the event-timed call. The persistent "
                             "mixed kernel binds on neither HBM nor tensor cores: it is "
                             "latency-bound (team barriers, dependent FMA chains, L2 round "
                             "trips); ncu: DRAM throughput 1.7%, FP64 pipe 19%, FP32 7%, "
                             "tensor 0.6% (profiles/posv_vbatch_mixed_n8-256.txt). The FP64 form's "
                             "fraction of the FP64 pipe is in fp64_pipe"},
        "fp64_pipe": {"peak_tflops_measured_live": fp64_peak, "probe": fp64_rec["probe"],
                      "refinement_fp64_tflops": fp64_flops_refine / (ms_mixed * 1e-3) / 1e12,
                      "fp64_form_tflops": useful / (ms_fp64 * 1e-3) / 1e12,
                      "fp64_form_frac": useful / (ms_fp64 * 1e-3) / 1e12 / fp64_peak},
        "e2e": {"value": v_e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e,
                "ms_step_stats": {"mean": ms_e2e, "median": float(np.median(t_e2e)),
                                  "min": float(np.min(t_e2e)), "max": float(np.max(t_e2e))},
                "host_link_gbs": h2d / (ms_e2e * 1e-3) / 1e9,
                "valid": e2e_valid,
                "per_step_ms": [round(x, 3) for x in t_e2e],
                "per_step_h2d_copy_ms": [round(x, 3) for x in h2d_ms],
                "per_step_host_issue_ms": [round(x, 3) for x in host_issue_ms],
                "host_link_probe_ms": [round(x, 3) for x in link_ms],
                "host_link_probe": "the same host->device copy of the matrix pool (pinned, "
                                   "%.2f GB) with no solve running, %d times after the e2e steps"
                                   % (w.pool_elems * 8 / 1e9, LINK_PROBE_REPS),
                "pipeline": f"{len(chunks)} pieces: host->device copy of piece k+1 overlaps "
                            f"the solve of piece k (copy stream + handle stream)",
                "vs_resident_run": e2e_check},
        # per call: vb_count, vb_plan, vb_scatter, the panel-path and the
        # register-path persistent kernels
        "gpu_launches": 5 * args.steps,
        "clocks": clk.summary(),
    }
    line["device_status"] = h.device_status()
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(orc, wl)
    if rank == 0 and not args.headline_only:
        # the other configurations of the path, each with its own value,
        # accuracy against the oracle, roofline and CPU baseline
        del w
        torch.cuda.empty_cache()
        c = make_ctx(args, torch, kb, wl, orc, h, stream)
        c.fp64 = fp64_rec
        c.fp64_peak = fp64_peak
        line["configs"] = {}
        for name in ("potrf_potrs_n32", "trsm_trmm_syrk_n64", "mixed_posv_n64", "posv_n512"):
            t0 = time.perf_counter()
            line["configs"][name] = CONFIGS[name](c)
            line["configs"][name]["wall_s"] = round(time.perf_counter() - t0, 1)
            torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line))
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
