"""The largest configuration of the path at small batch: n = 512 squared-
exponential covariance matrices with a 1e-4 nugget (ill-conditioned), 8
right-hand sides -- the plain FP64 POSV / POTRF / POTRS and the mixed-precision
POSV against the CPU oracle.

Bar: backward error <= 10 n eps64 per system, info identical to the oracle's;
the mixed form's results agree with the FP64 form's to the conditioning."""
import numpy as np
import pytest

from gpu_util import to_dev

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -53
N, M, BATCH = 512, 8, 6


@pytest.fixture(scope="module")
def cov(wl):
    a = wl.sqexp_cov(BATCH, N, seed=5)
    b = wl.rhs_rows(BATCH, M, N, seed=6)
    return a, b


def test_posv_fp64_n512(gpu, handle, orc, cov):
    a, b = cov
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((BATCH,), -99, dtype=gpu.int32, device="cuda")
    st = handle.call("kblasDposv_batch_strided", "R", "L", M, N, da.data_ptr(), N, N * N,
                     db.data_ptr(), M, M * N, BATCH, info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, N)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    ok = info_ref == 0
    X = db.cpu().numpy()
    eta = orc.backward_error_r(a[ok], X[ok], b[ok], M, N)
    assert eta.max() <= 10 * N * EPS64, eta.max()


def test_potrf_potrs_fp64_n512(gpu, handle, orc, cov):
    a, b = cov
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((BATCH,), -99, dtype=gpu.int32, device="cuda")
    assert handle.call("kblasDpotrf_batch_strided", "L", N, da.data_ptr(), N, N * N, BATCH,
                       info.data_ptr()) == 1
    assert handle.call("kblasDpotrs_batch_strided", "R", "L", M, N, da.data_ptr(), N, N * N,
                       db.data_ptr(), M, M * N, BATCH) == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    L = da.cpu().numpy()
    for s in range(BATCH):
        assert orc.factor_backward_error(a[s], L[s], N) <= 10 * N * EPS64
    eta = orc.backward_error_r(a, db.cpu().numpy(), b, M, N)
    assert eta.max() <= 10 * N * EPS64, eta.max()


def test_posv_mixed_n512(gpu, handle, kb, orc, cov):
    a, b = cov
    kb.lib().kblas_posv_batch_mixed_wsquery(handle.ptr, b"R", M, N, BATCH)
    assert handle.allocate_workspace() == 1
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((BATCH,), -99, dtype=gpu.int32, device="cuda")
    it = gpu.full((BATCH,), -99, dtype=gpu.int32, device="cuda")
    st = handle.call("kblasDposv_batch_mixed_strided", "R", "L", M, N, da.data_ptr(), N, N * N,
                     db.data_ptr(), M, M * N, BATCH, info.data_ptr(), it.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    X = db.cpu().numpy()
    eta = orc.backward_error_r(a, X, b, M, N)
    assert eta.max() <= 10 * N * EPS64, eta.max()
    iters = it.cpu().numpy()
    A_out = da.cpu().numpy()
    for s in range(BATCH):
        if iters[s] >= 0:
            assert np.array_equal(A_out[s], a[s]), "A must be unchanged after converged refinement"
    ref_a, ref_b = a.copy(), b.copy()
    orc.posv_batch(ref_a, ref_b, M, N)
    fwd = np.abs(X - ref_b).max() / np.abs(ref_b).max()
    assert fwd <= 1e-6, fwd  # cond <= ~5e6 for these matrices
