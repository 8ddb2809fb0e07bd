"""The allocation-free mixed-precision POSV (kblasDposv_batch_mixed_strided_noalloc)
against the handle-based kblasDposv_batch_mixed_strided on the same inputs.

Its scratch is one fixed device array shared by every call, so each GPU test
calls it twice in a row and checks both calls: the work counter must be
cleared between launches and no state may leak from the previous call. The
file is named to be collected last, so the routine is also exercised after
every other test of the suite has used the device; it passes alone in a fresh
process too (the first call does the per-device set-up).

Bar: info and iter identical to the handle-based routine; X and (for systems
that fell back to FP64) A within rounding of it; the backward error of every
system <= 10 n eps64 (oracle); free device memory unchanged by a call made
after set-up.
"""
import numpy as np
import pytest

from gpu_util import to_dev

EPS64 = 2.0 ** -53
MAX_N = 256            # KBLAS_POSV_NOALLOC_MAX_N
NOT_SUPPORTED = -1     # KBLAS_NotSupported
SUCCESS = 1


def make_batch(wl, n, m, batch, seed, n_cond, indefinite):
    """Well-conditioned systems, then n_cond with cond in [1e2, 1e8] (some of
    them reach the FP64 fallback), with a few indefinite ones planted."""
    lda, ldb = n + 1, m + 2
    a = wl.spd_shifted(batch, n, seed=seed, ld=lda)
    if n_cond:
        c, _ = wl.spd_cond(n_cond, n, seed=seed + 1, ld=lda)
        a[:n_cond] = c
    for s in indefinite:
        a[s] = wl.flip_one_eigenvalue(a[s], n, seed=seed + s)
    b = wl.rhs_rows(batch, m, n, seed=seed + 2, ld=ldb)
    return a, b


def run(gpu, kb, a, b, m, n, handle=None, stream=None):
    batch, lda, ldb = a.shape[0], a.shape[2], b.shape[2]
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    it = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    gpu.cuda.synchronize()
    args = ("R", "L", m, n, da.data_ptr(), lda, a.shape[1] * lda, db.data_ptr(), ldb,
            b.shape[1] * ldb, batch, info.data_ptr(), it.data_ptr())
    if handle is not None:
        kb.lib().kblas_posv_batch_mixed_wsquery(handle.ptr, b"R", m, n, batch)
        assert handle.allocate_workspace() == 1
        st = handle.call("kblasDposv_batch_mixed_strided", *args)
    else:
        conv = [x.encode() if isinstance(x, str) else x for x in args]
        st = kb.lib().kblasDposv_batch_mixed_strided_noalloc(stream.cuda_stream, *conv)
    assert st == SUCCESS, st
    gpu.cuda.synchronize()
    return da.cpu().numpy(), db.cpu().numpy(), info.cpu().numpy(), it.cpu().numpy()


def check_same(ref, got, a, b, m, n, orc):
    A_r, X_r, info_r, it_r = ref
    A_g, X_g, info_g, it_g = got
    assert np.array_equal(info_g, info_r)
    assert np.array_equal(it_g, it_r)
    tol = 1e-8  # relative, per system; both runs are the same kernel
    for s in range(a.shape[0]):
        xs = max(np.abs(X_r[s, :n, :m]).max(), 1e-300)
        assert np.abs(X_g[s] - X_r[s]).max() <= tol * xs, s
        As = max(np.abs(A_r[s, :n, :n]).max(), 1e-300)
        assert np.abs(np.tril(A_g[s, :n, :n].T) - np.tril(A_r[s, :n, :n].T)).max() <= tol * As, s
    ok = info_g == 0
    eta = orc.backward_error_r(a[ok], X_g[ok], b[ok], m, n)
    assert eta.max() <= 10 * n * EPS64, (eta.max(), 10 * n * EPS64)
    assert np.array_equal(X_g[~ok], b[~ok]), "B must be unchanged for a failed system"


@pytest.mark.gpu
@pytest.mark.parametrize("n,m,batch,n_cond,indef", [
    (16, 3, 600, 60, (5, 77)),         # register path: no per-CTA scratch
    (64, 4, 900, 300, (1, 400, 899)),  # panel path: FP64 fallback factors in scratch
    (256, 2, 400, 40, (7, 250)),       # largest order: grid cut to the slots that fit
])
def test_noalloc_matches_handle_routine_twice(gpu, kb, wl, orc, n, m, batch, n_cond, indef):
    a, b = make_batch(wl, n, m, batch, seed=40 + n, n_cond=n_cond, indefinite=indef)
    h = kb.Handle()
    try:
        ref = run(gpu, kb, a, b, m, n, handle=h)
    finally:
        gpu.cuda.synchronize()
        h.close()
    assert (ref[2][list(indef)] > 0).all()
    stream = gpu.cuda.Stream()
    first = run(gpu, kb, a, b, m, n, stream=stream)
    free_after_first = gpu.cuda.mem_get_info()[0]
    second = run(gpu, kb, a, b, m, n, stream=stream)
    assert gpu.cuda.mem_get_info()[0] == free_after_first, "a call after set-up allocated"
    check_same(ref, first, a, b, m, n, orc)
    check_same(ref, second, a, b, m, n, orc)


@pytest.mark.gpu
def test_noalloc_alternating_orders_share_the_array(gpu, kb, wl, orc):
    """Back-to-back calls of different orders in one stream reuse the array."""
    stream = gpu.cuda.Stream()
    for n, m, batch in ((200, 1, 300), (40, 5, 700), (200, 1, 300)):
        a, b = make_batch(wl, n, m, batch, seed=7 * n + m, n_cond=batch // 4, indefinite=(3,))
        h = kb.Handle()
        try:
            ref = run(gpu, kb, a, b, m, n, handle=h)
        finally:
            gpu.cuda.synchronize()
            h.close()
        got = run(gpu, kb, a, b, m, n, stream=stream)
        check_same(ref, got, a, b, m, n, orc)


@pytest.mark.gpu
def test_noalloc_quick_returns(gpu, kb):
    stream = gpu.cuda.Stream()
    info = gpu.full((5,), -99, dtype=gpu.int32, device="cuda")
    it = gpu.full((5,), -99, dtype=gpu.int32, device="cuda")
    a = gpu.zeros(8, dtype=gpu.float64, device="cuda")
    f = kb.lib().kblasDposv_batch_mixed_strided_noalloc
    assert f(stream.cuda_stream, b"R", b"L", 1, 0, a.data_ptr(), 1, 0, a.data_ptr(), 1, 0, 5,
             info.data_ptr(), it.data_ptr()) == SUCCESS
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all() and (it.cpu().numpy() == 0).all()
    assert f(stream.cuda_stream, b"R", b"L", 1, 4, a.data_ptr(), 4, 16, a.data_ptr(), 1, 4, 0,
             info.data_ptr(), it.data_ptr()) == SUCCESS
    assert f(stream.cuda_stream, b"L", b"L", 1, 4, a.data_ptr(), 4, 16, a.data_ptr(), 1, 4, 1,
             info.data_ptr(), it.data_ptr()) == -2  # KBLAS_NotImplemented, as the handle form


def test_noalloc_rejects_orders_beyond_its_scratch(kb):
    """Checked on the host before any CUDA call, so this runs without a GPU."""
    kb.build()
    f = kb.lib().kblasDposv_batch_mixed_strided_noalloc
    for n in (MAX_N + 1, 1024, 5000):
        assert f(None, b"R", b"L", 1, n, None, n, n * n, None, 1, n, 10, None, None) == NOT_SUPPORTED
