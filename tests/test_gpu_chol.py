"""GPU parity of batched POTRF / POTRS / POSV against the CPU oracle.

Every case runs the CUDA library through its C ABI on seeded inputs
(A = G G^T + n I, the benchmark recipe) and checks, per matrix:
  * info codes identical to the oracle's (LAPACK semantics), exactly;
  * the factor's backward error ||A - L L^T||_max / ||A||_max <= 10 n eps and
    its distance to the oracle's factor <= 10 n eps (relative, reference
    tests' measure);
  * the solution's normwise backward error <= 10 n eps (per right-hand side);
  * the strict upper triangle of A, the padding rows (lda > n) and the gaps
    between matrices are left untouched.
"""
import numpy as np
import pytest

from gpu_util import eps, gather_scattered, lower, ptr_array, scattered_copies, to_dev

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 5, 8, 9, 15, 16, 17, 24, 31, 32, 33, 47, 63, 64, 65, 100, 128, 129, 200, 257]
SENT = -7.25  # sentinel in the strict upper triangle / padding


def make_batch(wl, batch, n, ld, dt, seed):
    a = wl.spd_shifted(batch, n, seed=seed, ld=ld, dtype=np.float64)
    # strict upper triangle and padding rows hold a sentinel
    for b in range(batch):
        m = a[b]
        for j in range(n):
            m[j, :j] = SENT
            m[j, n:] = SENT
    return a.astype(dt)


def check_untouched(a_in, a_out, n):
    batch, _, ld = a_in.shape
    for j in range(n):
        assert np.array_equal(a_out[:, j, :j], a_in[:, j, :j]), "strict upper triangle written"
        assert np.array_equal(a_out[:, j, n:], a_in[:, j, n:]), "padding rows written"


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("n", SIZES)
def test_potrf_strided(gpu, handle, wl, orc, dt, n):
    batch = 67 if n <= 64 else 9
    ld = n + 3
    a = make_batch(wl, batch, n, ld, dt, seed=n)
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, n)
    da = to_dev(gpu, a)
    dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    pfx = "D" if dt == np.float64 else "S"
    st = handle.call(f"kblas{pfx}potrf_batch_strided", "L", n, da.data_ptr(), ld, n * ld, batch,
                     dinfo.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    out = da.cpu().numpy()
    info = dinfo.cpu().numpy()
    assert np.array_equal(info, info_ref)
    check_untouched(a, out, n)
    tol = 10 * max(n, 2) * eps(dt)
    for b in range(batch):
        L = np.tril(out[b, :n, :n].T).astype(np.float64)
        A0 = a[b, :n, :n].T.astype(np.float64)
        Asym = np.tril(A0) + np.tril(A0, -1).T
        fb = np.abs(Asym - L @ L.T).max() / np.abs(Asym).max()
        assert fb <= tol, (b, fb)
        Lr = np.tril(ref[b, :n, :n].T)
        rd = np.abs(L - Lr).max() / np.abs(Lr).max()
        assert rd <= tol, (b, rd)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("n", [4, 16, 32, 33, 96])
def test_potrf_pointer_array(gpu, handle, wl, orc, dt, n):
    batch = 45
    a = make_batch(wl, batch, n, n, dt, seed=100 + n)
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, n)
    pool, ptrs, offs = scattered_copies(gpu, a, seed=n)
    dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    pfx = "D" if dt == np.float64 else "S"
    st = handle.call(f"kblas{pfx}potrf_batch", "L", n, ptrs.data_ptr(), n, batch, dinfo.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    out = gather_scattered(pool, offs, a.shape)
    assert np.array_equal(dinfo.cpu().numpy(), info_ref)
    check_untouched(a, out, n)
    # gaps between the scattered matrices are still NaN
    p = pool.cpu().numpy()
    mask = np.ones(p.size, bool)
    for o in offs:
        mask[o:o + a.shape[1] * a.shape[2]] = False
    assert np.isnan(p[mask]).all()
    tol = 10 * n * eps(dt)
    rd = max(np.abs(np.tril(out[b, :n, :n].T) - np.tril(ref[b, :n, :n].T)).max()
             / np.abs(np.tril(ref[b, :n, :n].T)).max() for b in range(batch))
    assert rd <= tol


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("n", [1, 7, 8, 16, 20, 32, 33, 64, 100, 129])
@pytest.mark.parametrize("m", [1, 4, 11])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_posv_and_potrs(gpu, handle, wl, orc, dt, n, m, form):
    batch = 40 if n <= 64 else 6
    lda, ldb = n + 1, m + 2
    a = make_batch(wl, batch, n, lda, dt, seed=7 * n + m)
    bmat = wl.rhs_rows(batch, m, n, seed=n + m, ld=ldb, dtype=np.float64).astype(dt)
    pfx = "D" if dt == np.float64 else "S"
    # POSV
    da, db = to_dev(gpu, a), to_dev(gpu, bmat)
    dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        st = handle.call(f"kblas{pfx}posv_batch_strided", "R", "L", m, n, da.data_ptr(), lda,
                         n * lda, db.data_ptr(), ldb, n * ldb, batch, dinfo.data_ptr())
    else:
        pa, pb = ptr_array(gpu, da), ptr_array(gpu, db)
        st = handle.call(f"kblas{pfx}posv_batch", "R", "L", m, n, pa.data_ptr(), lda, pb.data_ptr(),
                         ldb, batch, dinfo.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    assert (dinfo.cpu().numpy() == 0).all()
    L = da.cpu().numpy()
    X = db.cpu().numpy()
    check_untouched(a, L, n)
    assert np.array_equal(X[:, :, m:], bmat[:, :, m:]), "ldb padding written"
    eta = orc.backward_error_r(a.astype(np.float64), X.astype(np.float64), bmat.astype(np.float64), m, n)
    assert eta.max() <= 10 * n * eps(dt), eta.max()
    # POTRS with the GPU factor reproduces the POSV solution
    db2 = to_dev(gpu, bmat)
    if form == "strided":
        st = handle.call(f"kblas{pfx}potrs_batch_strided", "R", "L", m, n, da.data_ptr(), lda,
                         n * lda, db2.data_ptr(), ldb, n * ldb, batch)
    else:
        pa, pb2 = ptr_array(gpu, da), ptr_array(gpu, db2)
        st = handle.call(f"kblas{pfx}potrs_batch", "R", "L", m, n, pa.data_ptr(), lda,
                         pb2.data_ptr(), ldb, batch)
    assert st == 1
    gpu.cuda.synchronize()
    X2 = db2.cpu().numpy()
    eta2 = orc.backward_error_r(a.astype(np.float64), X2.astype(np.float64), bmat.astype(np.float64), m, n)
    assert eta2.max() <= 10 * n * eps(dt), eta2.max()
    assert np.abs(X2 - X).max() <= 64 * n * eps(dt) * max(1.0, np.abs(X).max())


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("n", [1, 3, 7, 8, 9, 15, 16, 17, 30, 31, 32])
@pytest.mark.parametrize("pad", [0, 4])
def test_register_kernel_vector_path(gpu, handle, wl, orc, dt, n, pad):
    """n <= 32 with 16-byte aligned matrices and lda a multiple of 16 bytes:
    POTRS runs on the register kernel, which loads the factor in 128-bit
    chunks; POTRF and POSV (team kernel) leave the strict upper triangle and
    the padding rows untouched, and all three agree with the oracle."""
    batch, m = 37, 3
    lda = -(-n // 4) * 4 + pad  # 16-byte multiple for both precisions
    a = make_batch(wl, batch, n, lda, dt, seed=300 + n)
    ref = a.copy()
    info_ref = orc.potrf_batch(ref, n)
    pfx = "D" if dt == np.float64 else "S"
    da = to_dev(gpu, a)
    assert da.data_ptr() % 16 == 0
    dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert handle.call(f"kblas{pfx}potrf_batch_strided", "L", n, da.data_ptr(), lda, n * lda, batch,
                       dinfo.data_ptr()) == 1
    gpu.cuda.synchronize()
    out = da.cpu().numpy()
    assert np.array_equal(dinfo.cpu().numpy(), info_ref)
    check_untouched(a, out, n)
    tol = 10 * max(n, 2) * eps(dt)
    rd = max(np.abs(np.tril(out[b, :n, :n].T) - np.tril(ref[b, :n, :n].T)).max()
             / np.abs(np.tril(ref[b, :n, :n].T)).max() for b in range(batch))
    assert rd <= tol, rd
    # POSV and POTRS (right-hand sides as rows of B, ldb = m)
    bmat = wl.rhs_rows(batch, m, n, seed=n + 5, dtype=np.float64).astype(dt)
    da, db = to_dev(gpu, a), to_dev(gpu, bmat)
    assert handle.call(f"kblas{pfx}posv_batch_strided", "R", "L", m, n, da.data_ptr(), lda,
                       n * lda, db.data_ptr(), m, n * m, batch, dinfo.data_ptr()) == 1
    gpu.cuda.synchronize()
    X = db.cpu().numpy()
    check_untouched(a, da.cpu().numpy(), n)
    eta = orc.backward_error_r(a.astype(np.float64), X.astype(np.float64),
                               bmat.astype(np.float64), m, n)
    assert eta.max() <= 10 * n * eps(dt), eta.max()
    db2 = to_dev(gpu, bmat)
    assert handle.call(f"kblas{pfx}potrs_batch_strided", "R", "L", m, n, da.data_ptr(), lda,
                       n * lda, db2.data_ptr(), m, n * m, batch) == 1
    gpu.cuda.synchronize()
    assert np.abs(db2.cpu().numpy() - X).max() <= 64 * n * eps(dt) * max(1.0, np.abs(X).max())


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
def test_info_codes_match_lapack_golden(gpu, handle, golden, dt):
    """Non-SPD matrices with a known failing leading minor (LAPACK golden
    vectors): identical info, B untouched by POSV for the failed systems."""
    pfx = "d" if dt == np.float64 else "s"
    for n, k in ((1, 1), (5, 3), (8, 8), (16, 1), (17, 9), (32, 20), (33, 33), (64, 40), (97, 77)):
        A = golden[f"{pfx}nonspd_n{n}_A"].astype(dt)
        good = golden[f"{pfx}potrf_n{n}_A"].astype(dt) if f"{pfx}potrf_n{n}_A" in golden.files else None
        mats = [A, A] if good is None else [good, A, good]
        a = np.stack([np.ascontiguousarray(x.T) for x in mats])
        batch = len(mats)
        bm = np.ones((batch, n, 1), dtype=dt)
        da, db = to_dev(gpu, a), to_dev(gpu, bm)
        dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
        st = handle.call(f"kblas{pfx.upper()}posv_batch_strided", "R", "L", 1, n, da.data_ptr(), n,
                         n * n, db.data_ptr(), 1, n, batch, dinfo.data_ptr())
        assert st == 1
        gpu.cuda.synchronize()
        info = dinfo.cpu().numpy()
        exp = [k if x is A else 0 for x in mats]
        assert list(info) == exp, (n, info, exp)
        X = db.cpu().numpy()
        for b, x in enumerate(mats):
            if x is A:
                assert (X[b] == 1).all(), "B of a failed system was modified"
        # the columns before the failing one are the true factor
        L = da.cpu().numpy()
        for b, x in enumerate(mats):
            if x is A and k > 1:
                Lk = np.tril(L[b, : k - 1, : k - 1].T).astype(np.float64)
                A0 = x[: k - 1, : k - 1].astype(np.float64)
                assert np.abs(Lk @ Lk.T - A0).max() <= 10 * n * eps(dt) * np.abs(A0).max()


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
def test_nan_and_zero_pivot(gpu, handle, dt):
    pfx = "D" if dt == np.float64 else "S"
    n, batch = 12, 4
    a = np.stack([np.ascontiguousarray((np.eye(n) * 4).T) for _ in range(batch)]).astype(dt)
    a[1, 5, 5] = np.nan      # NaN pivot at column 6
    a[2, 0, 0] = 0.0         # zero pivot at column 1
    a[3, 11, 11] = -1.0      # negative last pivot
    da = to_dev(gpu, a)
    dinfo = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    st = handle.call(f"kblas{pfx}potrf_batch_strided", "L", n, da.data_ptr(), n, n * n, batch,
                     dinfo.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    assert list(dinfo.cpu().numpy()) == [0, 6, 1, 12]


def test_empty_and_degenerate(gpu, handle, kb):
    d = gpu.zeros(64, dtype=gpu.float64, device="cuda")
    dinfo = gpu.full((3,), -5, dtype=gpu.int32, device="cuda")
    # n == 0: success, info zeroed
    assert handle.call("kblasDpotrf_batch_strided", "L", 0, d.data_ptr(), 1, 0, 3, dinfo.data_ptr()) == 1
    gpu.cuda.synchronize()
    assert (dinfo.cpu().numpy() == 0).all()
    # batch == 0: success, nothing touched
    assert handle.call("kblasDpotrf_batch_strided", "L", 8, d.data_ptr(), 8, 64, 0, dinfo.data_ptr()) == 1
    # m == 0 POSV factors only
    assert handle.call("kblasDposv_batch_strided", "R", "L", 0, 0, d.data_ptr(), 1, 1, d.data_ptr(), 1,
                       1, 1, dinfo.data_ptr()) == 1


def test_argument_errors(gpu, handle, kb):
    d = gpu.zeros(256, dtype=gpu.float64, device="cuda")
    info = gpu.zeros(4, dtype=gpu.int32, device="cuda")
    p, ip = d.data_ptr(), info.data_ptr()
    WI = kb.KBLAS_Error_WrongInput
    # Upper / Left POTRF, POTRS, POSV and Upper SYRK are implemented here (the
    # reference returns KBLAS_NotImplemented); malformed flags are still errors
    assert handle.call("kblasDpotrs_batch_strided", "X", "U", 1, 8, p, 8, 64, p, 1, 8, 1) == WI
    assert handle.call("kblasDposv_batch_strided", "L", "Q", 1, 8, p, 8, 64, p, 1, 8, 1, ip) == WI
    # side L: A is m x m, so lda < m is an error
    assert handle.call("kblasDposv_batch_strided", "L", "L", 8, 1, p, 7, 64, p, 8, 8, 1, ip) == WI
    # malformed arguments
    assert handle.call("kblasDpotrf_batch_strided", "L", -1, p, 8, 64, 1, ip) == WI
    assert handle.call("kblasDpotrf_batch_strided", "L", 8, p, 7, 64, 1, ip) == WI
    assert handle.call("kblasDpotrf_batch_strided", "L", 8, p, 8, 63, 2, ip) == WI
    assert handle.call("kblasDpotrf_batch_strided", "X", 8, p, 8, 64, 1, ip) == WI
    assert handle.call("kblasDtrsm_batch_strided", "L", "L", "N", "N", 8, 4, 1.0, p, 7, 64, p, 8, 32, 1) == WI
    assert handle.call("kblasDtrsm_batch_strided", "Q", "L", "N", "N", 8, 4, 1.0, p, 8, 64, p, 8, 32, 1) == WI
