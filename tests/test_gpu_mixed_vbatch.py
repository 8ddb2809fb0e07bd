"""GPU parity of the mixed-precision POSV (uniform) and the variable-size POSV
(plain FP64 and mixed) against the CPU oracle.

Bar (per system): normwise backward error <= 10 n eps64 for every system of
every form, info codes identical to the oracle's (LAPACK DPOTRF), B left
unchanged by a failed system, A unchanged when the mixed path converged
(iter >= 0) and holding the FP64 factor when it fell back (iter < 0).
"""
import ctypes

import numpy as np
import pytest

from gpu_util import ptr_array, to_dev

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -53


def alloc_ws(kb, h, query, *args):
    getattr(kb.lib(), query)(h.ptr, *args)
    assert h.allocate_workspace() == 1


def run_uniform_mixed(gpu, kb, h, a, b, m, n, form="strided"):
    batch = a.shape[0]
    lda, ldb = a.shape[2], b.shape[2]
    alloc_ws(kb, h, "kblas_posv_batch_mixed_wsquery", b"R", m, n, batch)
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    it = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        st = h.call("kblasDposv_batch_mixed_strided", "R", "L", m, n, da.data_ptr(), lda,
                    a.shape[1] * lda, db.data_ptr(), ldb, b.shape[1] * ldb, batch, info.data_ptr(),
                    it.data_ptr())
    else:
        pa, pb = ptr_array(gpu, da), ptr_array(gpu, db)
        st = h.call("kblasDposv_batch_mixed", "R", "L", m, n, pa.data_ptr(), lda, pb.data_ptr(),
                    ldb, batch, info.data_ptr(), it.data_ptr())
    assert st == 1, st
    gpu.cuda.synchronize()
    return da.cpu().numpy(), db.cpu().numpy(), info.cpu().numpy(), it.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 5, 8, 9, 16, 17, 24, 32, 33, 40, 64, 65, 100, 128, 129, 200, 256])
@pytest.mark.parametrize("m", [1, 4, 6])
def test_mixed_uniform_wellconditioned(gpu, handle, kb, wl, orc, n, m):
    batch = 70 if n <= 64 else 5
    lda, ldb = n + 1, m + 1
    a = wl.spd_shifted(batch, n, seed=n * 7 + m, ld=lda)
    b = wl.rhs_rows(batch, m, n, seed=n + 3 * m, ld=ldb)
    A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n,
                                       form="strided" if (n + m) % 2 else "array")
    assert (info == 0).all()
    assert (it >= 0).all(), it  # these systems converge without the FP64 fallback
    assert np.array_equal(A, a), "A must be unchanged after a converged refinement"
    assert np.array_equal(X[:, :, m:], b[:, :, m:])
    eta = orc.backward_error_r(a, X, b, m, n)
    assert eta.max() <= 10 * n * EPS64, (eta.max(), 10 * n * EPS64)


def test_mixed_illconditioned_cond_1e2_to_1e8(gpu, handle, kb, wl, orc):
    """cond(A) log-uniform in [1e2, 1e8], 4 RHS (the mixed-precision benchmark
    recipe): every system reaches the FP64 backward-error bar, through
    refinement or the FP64 fallback; the forward error tracks cond * eps."""
    n, m, batch = 64, 4, 96
    a, cond = wl.spd_cond(batch, n, seed=3)
    b = wl.rhs_rows(batch, m, n, seed=4)
    A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n)
    assert (info == 0).all()
    eta = orc.backward_error_r(a, X, b, m, n)
    assert eta.max() <= 10 * n * EPS64, eta.max()
    ref_a, ref_b = a.copy(), b.copy()
    orc.posv_batch(ref_a, ref_b, m, n)
    fwd = np.abs(X - ref_b).max(axis=(1, 2)) / np.abs(ref_b).max(axis=(1, 2))
    assert (fwd <= 100 * n * cond * EPS64).all()
    # systems that took the FP64 path hold an FP64 factor of A in A (checked
    # by its backward error: the factor itself is as ill-conditioned as A)
    fb = np.where(it < 0)[0]
    for s in fb:
        assert orc.factor_backward_error(a[s], A[s], n) <= 10 * n * EPS64
    conv = np.where(it >= 0)[0]
    assert np.array_equal(A[conv], a[conv])
    # the well-conditioned part converges in a few steps; the worst part is
    # routed to FP64 by the conditioning estimate before any refinement
    assert (it[cond < 1e3] >= 0).all()
    assert (it[cond > 1e7] == -4).any()


def test_mixed_routing_off_and_on(gpu, handle, kb, wl, orc):
    """kblasSetPosvRouting(0) turns the conditioning routing off (no iter -4;
    the refinement's cost-model exit alone sends systems to FP64); a large
    constant routes every system; each one meets the bar either way."""
    n, m, batch = 64, 4, 96
    a, cond = wl.spd_cond(batch, n, seed=13)
    b = wl.rhs_rows(batch, m, n, seed=14)
    L = kb.lib()
    try:
        counts = {}
        for c in (0.0, 1e6):
            assert L.kblasSetPosvRouting(c) == 1
            A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n)
            assert (info == 0).all()
            eta = orc.backward_error_r(a, X, b, m, n)
            assert eta.max() <= 10 * n * EPS64, (c, eta.max())
            counts[c] = int((it == -4).sum())
            if c == 0.0:
                assert (it[cond < 1e4] >= 0).all()
            else:
                # every system whose FP32 pivots passed (-1 otherwise) is routed
                assert set(np.unique(it).tolist()) <= {-1, -4}, np.unique(it)
        assert counts[0.0] == 0
        assert counts[1e6] > 0
    finally:
        assert L.kblasSetPosvRouting(-1.0) == 1
    assert L.kblasSetPosvRouting(float("nan")) == kb.KBLAS_Error_WrongInput


@pytest.mark.parametrize("n", [150, 300])
@pytest.mark.parametrize("m", [2, 3, 5, 7])
def test_mixed_panel_path_several_rhs_covariance(gpu, handle, kb, wl, orc, n, m):
    """Panel path with 4- and 8-warp teams and 2..4 right-hand sides per
    sweep (the sweep that solves them all at once), on squared-exponential
    covariances (nugget 1e-4, cond up to ~1e6), which take several refinement
    steps: every system meets the bar and stays close to the FP64 solution."""
    batch = 6
    a = wl.sqexp_cov(batch, n, seed=n + m)
    b = wl.rhs_rows(batch, m, n, seed=5 * m + 1)
    # the refinement sweeps are what this test exercises: no conditioning
    # routing to FP64 (with it, most of these systems take the FP64 path)
    assert kb.lib().kblasSetPosvRouting(0.0) == 1
    try:
        A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n,
                                           form="strided" if m % 2 else "array")
    finally:
        assert kb.lib().kblasSetPosvRouting(-1.0) == 1
    assert (info == 0).all()
    eta = orc.backward_error_r(a, X, b, m, n)
    assert eta.max() <= 10 * n * EPS64, eta.max()
    assert (it >= 1).all(), it  # refinement steps were taken (correction solves ran)
    assert np.array_equal(A, a)
    ref_a, ref_b = a.copy(), b.copy()
    orc.posv_batch(ref_a, ref_b, m, n)
    fwd = np.abs(X - ref_b).max(axis=(1, 2)) / np.abs(ref_b).max(axis=(1, 2))
    assert (fwd <= 1e-4).all(), fwd.max()


@pytest.mark.parametrize("n", [8, 16, 24])
def test_mixed_register_path_illconditioned_many_rhs(gpu, handle, kb, wl, orc, n):
    """Register path (several systems share a warp) with cond up to 1e8 and 4
    right-hand sides: systems fall back to FP64 after different numbers of
    converged right-hand sides, so the systems of one warp resume the FP64
    solve at different rows; every system must still meet the bar."""
    m, batch = 4, 512
    a, cond = wl.spd_cond(batch, n, seed=21 + n)
    b = wl.rhs_rows(batch, m, n, seed=22 + n)
    A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n)
    assert (info == 0).all()
    eta = orc.backward_error_r(a, X, b, m, n)
    assert eta.max() <= 10 * n * EPS64, eta.max()
    assert (it < 0).any() and (it >= 0).any()


def test_mixed_indefinite_info_exact(gpu, handle, kb, wl, orc):
    n, m, batch = 48, 2, 40
    a = wl.spd_shifted(batch, n, seed=11)
    bad = [3, 17, 18, 39]
    for s in bad:
        a[s] = wl.flip_one_eigenvalue(a[s], n, seed=s)
    b = wl.rhs_rows(batch, m, n, seed=12)
    A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n)
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, n)
    assert np.array_equal(info, info_ref)
    assert (info_ref[bad] > 0).all()
    for s in bad:
        assert it[s] == -1
        assert np.array_equal(X[s], b[s]), "B of a non-SPD system was modified"
    good = [s for s in range(batch) if s not in bad]
    eta = orc.backward_error_r(a[good], X[good], b[good], m, n)
    assert eta.max() <= 10 * n * EPS64


def test_mixed_needs_workspace(gpu, handle, kb, wl):
    n, m, batch = 32, 1, 8
    a = to_dev(gpu, wl.spd_shifted(batch, n))
    b = to_dev(gpu, wl.rhs_rows(batch, m, n))
    info = gpu.zeros(batch, dtype=gpu.int32, device="cuda")
    st = handle.call("kblasDposv_batch_mixed_strided", "R", "L", m, n, a.data_ptr(), n, n * n,
                     b.data_ptr(), m, n * m, batch, info.data_ptr(), None)
    assert st == kb.KBLAS_InsufficientWorkspace


# --------------------------------------------------------------------------
# variable size
# --------------------------------------------------------------------------

def make_vbatch(wl, sizes, ms, seed, indefinite=()):
    As, Bs = [], []
    for i, (n, m) in enumerate(zip(sizes, ms)):
        lda = n + (i % 3)
        ldb = max(1, m) + (i % 2)
        a = wl.spd_shifted(1, n, seed=seed + i, ld=lda)[0] if n > 0 else np.zeros((0, max(lda, 1)))
        if i in indefinite and n > 1:
            a = wl.flip_one_eigenvalue(a, n, seed=i)
        b = wl.rhs_rows(1, m, n, seed=seed + 7 * i, ld=ldb)[0] if n > 0 else np.zeros((0, ldb))
        As.append(np.ascontiguousarray(a))
        Bs.append(np.ascontiguousarray(b))
    return As, Bs


def upload_vbatch(gpu, As, Bs):
    """Each matrix in its own device allocation; device pointer arrays."""
    dA = [gpu.from_numpy(x.reshape(-1).copy() if x.size else np.zeros(1)).cuda() for x in As]
    dB = [gpu.from_numpy(x.reshape(-1).copy() if x.size else np.zeros(1)).cuda() for x in Bs]
    pa = gpu.tensor([t.data_ptr() for t in dA], dtype=gpu.int64, device="cuda")
    pb = gpu.tensor([t.data_ptr() for t in dB], dtype=gpu.int64, device="cuda")
    return dA, dB, pa, pb


def run_vbatch(gpu, kb, h, As, Bs, ns, ms, mixed, graph=False):
    batch = len(ns)
    ldas = [a.shape[1] if a.ndim == 2 and a.shape[0] else max(1, n) for a, n in zip(As, ns)]
    ldbs = [b.shape[1] if b.ndim == 2 and b.shape[0] else 1 for b in Bs]
    max_n, max_m = max(ns), max(ms)
    kb.lib().kblas_posv_vbatch_wsquery(h.ptr, max_n, batch)
    assert h.allocate_workspace() == 1
    dA, dB, pa, pb = upload_vbatch(gpu, As, Bs)
    dn = gpu.tensor(ns, dtype=gpu.int32, device="cuda")
    dm = gpu.tensor(ms, dtype=gpu.int32, device="cuda")
    dlda = gpu.tensor(ldas, dtype=gpu.int32, device="cuda")
    dldb = gpu.tensor(ldbs, dtype=gpu.int32, device="cuda")
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    it = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    name = "kblasDposv_vbatch_mixed" if mixed else "kblasDposv_vbatch"
    args = ["R", "L", dm.data_ptr(), dn.data_ptr(), max_m, max_n, pa.data_ptr(), dlda.data_ptr(),
            pb.data_ptr(), dldb.data_ptr(), batch, info.data_ptr()]
    if mixed:
        args.append(it.data_ptr())
    if graph:
        s = gpu.cuda.Stream()
        h.set_stream(s.cuda_stream)
        g = gpu.cuda.CUDAGraph()
        with gpu.cuda.graph(g, stream=s):
            assert h.call(name, *args) == 1
        g.replay()
        gpu.cuda.synchronize()
        h.set_stream(0)
    else:
        assert h.call(name, *args) == 1
    gpu.cuda.synchronize()
    Aout = [t.cpu().numpy()[: a.size].reshape(a.shape) for t, a in zip(dA, As)]
    Bout = [t.cpu().numpy()[: b.size].reshape(b.shape) for t, b in zip(dB, Bs)]
    return Aout, Bout, info.cpu().numpy(), it.cpu().numpy()


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_vbatch_mixed_sizes(gpu, handle, kb, wl, orc, mixed):
    rng = np.random.default_rng(5)
    batch = 300
    ns = list(wl.vbatch_sizes(batch, 1, 256, seed=9))
    ns[0], ns[1], ns[2] = 1, 256, 33
    ms = [int(x) for x in rng.integers(0, 4, batch)]
    ms[3] = 0
    indef = {7, 50, 51, 120, 299}
    As, Bs = make_vbatch(wl, ns, ms, seed=100, indefinite=indef)
    Aout, Bout, info, it = run_vbatch(gpu, kb, handle, As, Bs, ns, ms, mixed)
    # oracle
    refA = [a.copy() for a in As]
    refB = [b.copy() for b in Bs]
    ldas = [a.shape[1] for a in As]
    ldbs = [b.shape[1] for b in Bs]
    info_ref = orc.posv_vbatch(ms, ns, refA, ldas, refB, ldbs)
    assert np.array_equal(info, info_ref), np.where(info != info_ref)
    assert all(info_ref[i] > 0 for i in indef if ns[i] > 1)
    good = [i for i in range(batch) if info_ref[i] == 0 and ms[i] > 0]
    eta = orc.backward_error_r_vbatch([ms[i] for i in good], [ns[i] for i in good],
                                      [As[i] for i in good], [ldas[i] for i in good],
                                      [Bout[i] for i in good], [ldbs[i] for i in good],
                                      [Bs[i] for i in good], [ldbs[i] for i in good])
    lim = np.array([10 * ns[i] * EPS64 for i in good])
    assert (eta <= lim).all(), (eta / lim).max()
    for i in range(batch):
        if info_ref[i] > 0:
            assert np.array_equal(Bout[i], Bs[i])
        if mixed and info_ref[i] == 0 and it[i] >= 0:
            assert np.array_equal(Aout[i], As[i])
        if not mixed or it[i] < 0:
            if info_ref[i] == 0:
                assert orc.factor_backward_error(As[i], Aout[i], ns[i]) <= 10 * ns[i] * EPS64
    if mixed:
        ok = [i for i in range(batch) if info_ref[i] == 0]
        assert (it[ok] >= 0).mean() > 0.95  # well-conditioned: refinement, not fallback


def test_vbatch_argument_info_codes(gpu, handle, kb, wl):
    ns = [8, -1, 5, 300, 6, 4]
    ms = [1, 1, -2, 1, 1, 9]
    As, Bs = make_vbatch(wl, [max(n, 0) if n <= 256 else 8 for n in ns], [max(m, 0) for m in ms], seed=1)
    batch = len(ns)
    dA, dB, pa, pb = upload_vbatch(gpu, As, Bs)
    ldas = [8, 1, 5, 300, 5, 4]   # system 4: lda < n
    ldbs = [1, 1, 1, 1, 1, 9]
    kb.lib().kblas_posv_vbatch_wsquery(handle.ptr, 256, batch)
    assert handle.allocate_workspace() == 1
    T = lambda v: gpu.tensor(v, dtype=gpu.int32, device="cuda")
    dn, dm, dla, dlb = T(ns), T(ms), T(ldas), T(ldbs)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    st = handle.call("kblasDposv_vbatch", "R", "L", dm.data_ptr(), dn.data_ptr(), 8, 256,
                     pa.data_ptr(), dla.data_ptr(), pb.data_ptr(), dlb.data_ptr(), batch,
                     info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    got = list(info.cpu().numpy())
    assert got == [0, -5, -4, -7, -9, -6], got


def test_vbatch_graph_capture_replay(gpu, handle, kb, wl, orc):
    batch = 64
    ns = list(wl.vbatch_sizes(batch, 8, 96, seed=2))
    ms = [1] * batch
    As, Bs = make_vbatch(wl, ns, ms, seed=300)
    Aout, Bout, info, it = run_vbatch(gpu, kb, handle, As, Bs, ns, ms, True, graph=True)
    assert (info == 0).all() and (it >= 0).all()
    ldas = [a.shape[1] for a in As]
    ldbs = [b.shape[1] for b in Bs]
    eta = orc.backward_error_r_vbatch(ms, ns, As, ldas, Bout, ldbs, Bs, ldbs)
    assert (eta <= np.array([10 * n * EPS64 for n in ns])).all()


@pytest.mark.parametrize("tc", [True, False], ids=["tensor_core", "ffma"])
def test_vbatch_mixed_large_orders_tensor_core_kernel(gpu, handle, kb, wl, orc, monkeypatch, tc):
    """A variable-size batch whose largest order exceeds 256 runs the kernel
    with the tensor-core trailing update (orders 177.. on whole-CTA teams);
    with KGB_NO_TC=1 the kernel without it. Both meet the bar on the same
    batch, with 1..6 right-hand sides (residual sweeps over 1..4 at once)."""
    if not tc:
        monkeypatch.setenv("KGB_NO_TC", "1")
    rng = np.random.default_rng(21)
    batch = 40
    ns = [int(x) for x in rng.integers(33, 400, batch)]
    ns[0], ns[1], ns[2] = 400, 177, 257
    ms = [int(x) for x in rng.integers(1, 7, batch)]
    As, Bs = make_vbatch(wl, ns, ms, seed=500, indefinite={5})
    Aout, Bout, info, it = run_vbatch(gpu, kb, handle, As, Bs, ns, ms, True)
    refA = [a.copy() for a in As]
    refB = [b.copy() for b in Bs]
    ldas = [a.shape[1] for a in As]
    ldbs = [b.shape[1] for b in Bs]
    info_ref = orc.posv_vbatch(ms, ns, refA, ldas, refB, ldbs)
    assert np.array_equal(info, info_ref)
    assert info_ref[5] > 0
    good = [i for i in range(batch) if info_ref[i] == 0]
    eta = orc.backward_error_r_vbatch([ms[i] for i in good], [ns[i] for i in good],
                                      [As[i] for i in good], [ldas[i] for i in good],
                                      [Bout[i] for i in good], [ldbs[i] for i in good],
                                      [Bs[i] for i in good], [ldbs[i] for i in good])
    assert (eta <= np.array([10 * ns[i] * EPS64 for i in good])).all()
    assert (it[good] >= 0).all()  # well-conditioned: refinement, no fallback
    for i in good:
        assert np.array_equal(Aout[i], As[i])
    assert np.array_equal(Bout[5], Bs[5])


def test_vbatch_needs_workspace(gpu, handle, kb):
    one = gpu.ones(4, dtype=gpu.int32, device="cuda")
    p = gpu.zeros(4, dtype=gpu.int64, device="cuda")
    st = handle.call("kblasDposv_vbatch_mixed", "R", "L", one.data_ptr(), one.data_ptr(), 1, 1,
                     p.data_ptr(), one.data_ptr(), p.data_ptr(), one.data_ptr(), 4, one.data_ptr(),
                     None)
    assert st == kb.KBLAS_InsufficientWorkspace


def test_tuning_override_roundtrip(gpu, handle, kb, wl, orc):
    """A different launch-shape table gives the same (correct) answers."""
    L = kb.lib()
    arr = lambda v: (ctypes.c_int * 8)(*v)  # KBLAS_POSV_TUNING_CLASSES
    nmax = [8, 16, 32, 64, 96, 128, 176, 1024]
    assert L.kblasSetPosvTuning(1, arr(nmax), arr([8, 16, 32, 64, 64, 256, 256, 256]),
                                arr([32, 16, 8, 4, 4, 1, 1, 1])) == 1
    try:
        n, m, batch = 40, 2, 30
        a = wl.spd_shifted(batch, n, seed=21)
        b = wl.rhs_rows(batch, m, n, seed=22)
        A, X, info, it = run_uniform_mixed(gpu, kb, handle, a, b, m, n)
        assert (info == 0).all() and (it >= 0).all()
        assert orc.backward_error_r(a, X, b, m, n).max() <= 10 * n * EPS64
    finally:
        assert L.kblasSetPosvTuning(1, None, None, None) == 1
    # invalid tables are rejected: a register-path team narrower than its
    # orders, a team size that is not a power of two
    assert L.kblasSetPosvTuning(1, arr(nmax), arr([8, 8, 32, 64, 64, 256, 256, 256]),
                                arr([32, 32, 8, 4, 4, 1, 1, 1])) == kb.KBLAS_Error_WrongInput
    assert L.kblasSetPosvTuning(1, arr(nmax), arr([3, 16, 32, 64, 64, 256, 256, 256]),
                                arr([32, 16, 8, 4, 4, 1, 1, 1])) == kb.KBLAS_Error_WrongInput
