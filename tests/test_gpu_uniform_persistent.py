"""Double-precision POTRF / POTRS / POSV of orders 33..1024 with the workspace
their wsqueries request allocated: these run on the persistent panel kernel
(the tests in test_gpu_chol.py, which allocate none, cover the one-launch
blocked kernel). Same bars: backward error <= 10 n eps64 per system, info codes
identical to the oracle's (LAPACK), untouched regions unchanged, B left as is for
a failed system."""
import numpy as np
import pytest

from gpu_util import ptr_array, to_dev
from test_gpu_chol import check_untouched, make_batch

pytestmark = pytest.mark.gpu

EPS64 = 2.0 ** -53


def alloc(kb, handle, which, *args):
    getattr(kb.lib(), which)(handle.ptr, *args)
    assert handle.allocate_workspace() == 1


@pytest.mark.parametrize("n", [33, 64, 100, 129, 200, 257, 512])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_posv_persistent(gpu, handle, kb, wl, orc, n, form):
    m = 3
    batch = 48 if n <= 128 else 8
    lda, ldb = n + 1, m + 1
    a = make_batch(wl, batch, n, lda, np.float64, seed=n + 5)
    bad = [1, batch - 2]
    for s in bad:
        a[s] = wl.flip_one_eigenvalue(a[s], n, seed=s)
    b = wl.rhs_rows(batch, m, n, seed=n, ld=ldb)
    fn = "kblas_posv_batch_strided_wsquery" if form == "strided" else "kblas_posv_batch_wsquery"
    alloc(kb, handle, fn, b"R", m, n, batch)
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        st = handle.call("kblasDposv_batch_strided", "R", "L", m, n, da.data_ptr(), lda, n * lda,
                         db.data_ptr(), ldb, n * ldb, batch, info.data_ptr())
    else:
        pa, pb = ptr_array(gpu, da), ptr_array(gpu, db)
        st = handle.call("kblasDposv_batch", "R", "L", m, n, pa.data_ptr(), lda, pb.data_ptr(), ldb,
                         batch, info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, n)
    got = info.cpu().numpy()
    assert np.array_equal(got, info_ref)
    assert (info_ref[bad] > 0).all()
    X = db.cpu().numpy()
    ok = info_ref == 0
    eta = orc.backward_error_r(a[ok], X[ok], b[ok], m, n)
    assert eta.max() <= 10 * n * EPS64, eta.max()
    assert np.array_equal(X[~ok], b[~ok]), "B of a failed system must be unchanged"
    check_untouched(a, da.cpu().numpy(), n)


@pytest.mark.parametrize("n", [40, 96, 160, 256])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_potrf_potrs_persistent(gpu, handle, kb, wl, orc, n, form):
    m = 2
    batch = 32 if n <= 128 else 8
    lda, ldb = n, m + 3
    a = make_batch(wl, batch, n, lda, np.float64, seed=3 * n)
    b = wl.rhs_rows(batch, m, n, seed=n + 1, ld=ldb)
    if form == "strided":
        alloc(kb, handle, "kblas_potrf_batch_strided_wsquery", n, batch)
        alloc(kb, handle, "kblas_potrs_batch_strided_wsquery", m, n, batch)
    else:
        alloc(kb, handle, "kblas_potrf_batch_wsquery", n, batch)
        alloc(kb, handle, "kblas_potrs_batch_wsquery", m, n, batch)
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        assert handle.call("kblasDpotrf_batch_strided", "L", n, da.data_ptr(), lda, n * lda, batch,
                           info.data_ptr()) == 1
        assert handle.call("kblasDpotrs_batch_strided", "R", "L", m, n, da.data_ptr(), lda,
                           n * lda, db.data_ptr(), ldb, n * ldb, batch) == 1
    else:
        pa, pb = ptr_array(gpu, da), ptr_array(gpu, db)
        assert handle.call("kblasDpotrf_batch", "L", n, pa.data_ptr(), lda, batch,
                           info.data_ptr()) == 1
        assert handle.call("kblasDpotrs_batch", "R", "L", m, n, pa.data_ptr(), lda, pb.data_ptr(),
                           ldb, batch) == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    Lg = da.cpu().numpy()
    check_untouched(a, Lg, n)
    for s in range(batch):
        assert orc.factor_backward_error(a[s], Lg[s], n) <= 10 * n * EPS64
    X = db.cpu().numpy()
    eta = orc.backward_error_r(a, X, b, m, n)
    assert eta.max() <= 10 * n * EPS64, eta.max()
    assert np.array_equal(X[:, :, m:], b[:, :, m:]), "ldb padding written"


def test_without_workspace_blocked_kernel_still_runs(gpu, handle, wl, orc):
    """No wsquery / allocation: the same call runs on the blocked kernel."""
    n, m, batch = 96, 1, 16
    a = make_batch(wl, batch, n, n, np.float64, seed=9)
    b = wl.rhs_rows(batch, m, n, seed=10)
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    st = handle.call("kblasDposv_batch_strided", "R", "L", m, n, da.data_ptr(), n, n * n,
                     db.data_ptr(), m, n * m, batch, info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    eta = orc.backward_error_r(a, db.cpu().numpy(), b, m, n)
    assert eta.max() <= 10 * n * EPS64
