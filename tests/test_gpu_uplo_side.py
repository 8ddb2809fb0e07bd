"""GPU parity of the Cholesky variants the reference leaves unimplemented:
POTRF with uplo 'U', POTRS / POSV with side 'L' and / or uplo 'U' (S and D,
strided and pointer-array, with and without the persistent-path workspace),
and the upper-triangle inversion routines, against the CPU oracle (pinned to
LAPACK in test_oracle.py).

Bars as for the lower / side-R forms: factor and solve backward errors
<= 10 n eps per system, info codes identical to LAPACK's, the triangle that is
not referenced and the leading-dimension padding bit-identical afterwards, B
of a failed system unchanged."""
import numpy as np
import pytest

from gpu_util import eps, ptr_array, to_dev

pytestmark = pytest.mark.gpu


def make_sym(wl, batch, n, ld, seed):
    """Full symmetric SPD batch (both triangles hold A), padding rows -3."""
    a = wl.spd_shifted(batch, n, seed=seed, ld=ld)
    a[:, :, n:] = -3.0
    return a


def with_sentinel(a, n, uplo):
    """Fill the triangle that must not be referenced with a sentinel."""
    a = a.copy()
    for j in range(n):
        if uplo == "U":
            a[:, j, j + 1:n] = -7.25     # strict lower (rows > j of column j)
        else:
            a[:, j, :j] = -7.25          # strict upper
    return a


def other_tri_equal(got, ref, n, uplo):
    for j in range(n):
        sl = slice(j + 1, n) if uplo == "U" else slice(0, j)
        if not np.array_equal(got[:, j, sl], ref[:, j, sl]):
            return False
    return np.array_equal(got[:, :n, n:], ref[:, :n, n:])


def factor_err(orc, a, F, n, uplo):
    """Backward error of a factor of either triangle (the upper factor is
    transposed into the lower one the oracle measures)."""
    A2, F2 = a.astype(np.float64), F.astype(np.float64)
    if uplo == "U":
        A2, F2 = A2.copy(), F2.copy()
        A2[:n, :n] = A2[:n, :n].T
        F2[:n, :n] = F2[:n, :n].T
    return orc.factor_backward_error(A2, F2, n)


def solve_err(a, X, B, side, uplo, m, n):
    """max over systems of ||op residual|| / (||A|| ||X|| + ||B||) (inf norms),
    A symmetric from its referenced triangle."""
    order = m if side == "L" else n
    worst = 0.0
    for s in range(a.shape[0]):
        T = a[s, :order, :order].T.astype(np.float64)       # row-major
        tri = np.triu(T) if uplo == "U" else np.tril(T)
        A = tri + tri.T - np.diag(np.diag(tri))
        x = X[s, :n, :m].T.astype(np.float64)                # m x n
        b = B[s, :n, :m].T.astype(np.float64)
        r = A @ x - b if side == "L" else x @ A - b
        den = np.abs(A).sum(1).max() * np.abs(x).max() + np.abs(b).max()
        worst = max(worst, np.abs(r).max() / den)
    return worst


def alloc(kb, handle, fn, *args):
    getattr(kb.lib(), fn)(handle.ptr, *args)
    assert handle.allocate_workspace() == 1


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("n", [1, 5, 16, 32, 33, 64, 100, 257])
@pytest.mark.parametrize("form", ["strided", "array"])
@pytest.mark.parametrize("ws", [False, True], ids=["blocked", "persistent"])
def test_potrf_upper(gpu, handle, kb, wl, orc, dt, n, form, ws):
    batch = 24 if n <= 64 else 6
    lda = n + 3
    a = make_sym(wl, batch, n, lda, seed=5 * n + 1)
    bad = [1] if batch > 2 else []
    for s in bad:
        a[s] = wl.flip_one_eigenvalue(a[s], n, seed=s)
    a = with_sentinel(a, n, "U").astype(dt)
    if ws:
        alloc(kb, handle, "kblas_potrf_batch_strided_wsquery" if form == "strided"
              else "kblas_potrf_batch_wsquery", n, batch)
    dA = to_dev(gpu, a)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    pfx = "D" if dt == np.float64 else "S"
    if form == "strided":
        st = handle.call(f"kblas{pfx}potrf_batch_strided", "U", n, dA.data_ptr(), lda, n * lda,
                         batch, info.data_ptr())
    else:
        pa = ptr_array(gpu, dA)   # referenced until the kernel has run
        st = handle.call(f"kblas{pfx}potrf_batch", "U", n, pa.data_ptr(), lda, batch,
                         info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    out = dA.cpu().numpy()
    ref = a.astype(np.float64).copy()
    info_ref = orc.potrf_batch_uplo(ref, n, "U")
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert other_tri_equal(out, a, n, "U"), "strict lower triangle or padding written"
    for s in np.where(info_ref == 0)[0]:
        assert factor_err(orc, a[s], out[s], n, "U") <= 10 * n * eps(dt) * (8 if dt == np.float32 else 1)


COMBOS = [("R", "U"), ("L", "L"), ("L", "U"), ("R", "L")]


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("combo", COMBOS, ids=["".join(c) for c in COMBOS])
@pytest.mark.parametrize("order", [7, 32, 48, 129])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_posv_potrs_sides(gpu, handle, kb, wl, orc, dt, combo, order, form):
    side, uplo = combo
    nrhs = 3
    m, n = (order, nrhs) if side == "L" else (nrhs, order)
    batch = 16 if order <= 64 else 4
    lda, ldb = order + 2, m + 1
    a = make_sym(wl, batch, order, lda, seed=order + len(form))
    bad = [2] if batch > 3 else []
    for s in bad:
        a[s] = wl.flip_one_eigenvalue(a[s], order, seed=s + 7)
    a = with_sentinel(a, order, uplo).astype(dt)
    rng = np.random.default_rng(order)
    b = np.full((batch, n, ldb), np.nan)
    b[:, :, :m] = rng.standard_normal((batch, n, m))
    b = b.astype(dt)
    pfx = "D" if dt == np.float64 else "S"
    # POSV
    dA, dB = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        st = handle.call(f"kblas{pfx}posv_batch_strided", side, uplo, m, n, dA.data_ptr(), lda,
                         order * lda, dB.data_ptr(), ldb, n * ldb, batch, info.data_ptr())
    else:
        pa, pb = ptr_array(gpu, dA), ptr_array(gpu, dB)
        st = handle.call(f"kblas{pfx}posv_batch", side, uplo, m, n, pa.data_ptr(), lda, pb.data_ptr(),
                         ldb, batch, info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    F, X = dA.cpu().numpy(), dB.cpu().numpy()
    refA, refB = a.astype(np.float64).copy(), b.astype(np.float64).copy()
    info_ref = orc.posv_batch_side(side, uplo, m, n, refA, refB)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert (info_ref[bad] > 0).all()
    ok = info_ref == 0
    assert np.array_equal(X[~ok], b[~ok], equal_nan=True), "B of a failed system changed"
    assert np.array_equal(X[:, :, m:], b[:, :, m:], equal_nan=True), "ldb padding written"
    assert other_tri_equal(F, a, order, uplo)
    tol = 10 * order * eps(dt) * (8 if dt == np.float32 else 1)
    assert solve_err(a[ok], X[ok], b[ok], side, uplo, m, n) <= tol
    # POTRS with the factor just computed (the systems that factored)
    okk = np.where(ok)[0]
    Fk, bk = np.ascontiguousarray(F[okk]), np.ascontiguousarray(b[okk])
    dF, dB2 = to_dev(gpu, Fk), to_dev(gpu, bk)
    k = len(okk)
    if form == "strided":
        st = handle.call(f"kblas{pfx}potrs_batch_strided", side, uplo, m, n, dF.data_ptr(), lda,
                         order * lda, dB2.data_ptr(), ldb, n * ldb, k)
    else:
        pf, pb2 = ptr_array(gpu, dF), ptr_array(gpu, dB2)
        st = handle.call(f"kblas{pfx}potrs_batch", side, uplo, m, n, pf.data_ptr(), lda,
                         pb2.data_ptr(), ldb, k)
    assert st == 1
    gpu.cuda.synchronize()
    X2 = dB2.cpu().numpy()
    assert np.array_equal(dF.cpu().numpy(), Fk), "POTRS wrote its factor"
    assert solve_err(a[okk], X2, bk, side, uplo, m, n) <= tol


def test_posv_upper_persistent_path(gpu, handle, kb, wl, orc):
    """uplo 'U', side 'R' with the persistent-path workspace allocated."""
    n, m, batch = 96, 2, 12
    a = make_sym(wl, batch, n, n, seed=77)
    a[4] = wl.flip_one_eigenvalue(a[4], n, seed=3)
    a = with_sentinel(a, n, "U")
    b = wl.rhs_rows(batch, m, n, seed=78)
    alloc(kb, handle, "kblas_posv_batch_strided_wsquery", b"R", m, n, batch)
    dA, dB = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert handle.call("kblasDposv_batch_strided", "R", "U", m, n, dA.data_ptr(), n, n * n,
                       dB.data_ptr(), m, n * m, batch, info.data_ptr()) == 1
    gpu.cuda.synchronize()
    refA, refB = a.copy(), b.copy()
    info_ref = orc.posv_batch_side("R", "U", m, n, refA, refB)
    assert np.array_equal(info.cpu().numpy(), info_ref) and info_ref[4] > 0
    ok = info_ref == 0
    X = dB.cpu().numpy()
    assert solve_err(a[ok], X[ok], b[ok], "R", "U", m, n) <= 10 * n * eps(np.float64)
    assert np.array_equal(X[4], b[4])
    assert other_tri_equal(dA.cpu().numpy(), a, n, "U")


@pytest.mark.parametrize("op", ["trtri", "lauum", "potri", "poti"])
@pytest.mark.parametrize("n", [1, 9, 32, 64, 130])
def test_inverse_upper(gpu, handle, wl, orc, op, n):
    batch = 12 if n <= 64 else 4
    lda = n + 1
    a = make_sym(wl, batch, n, lda, seed=9 * n)
    if op != "poti":   # the others take the Cholesky factor, here its upper form U
        info0 = orc.potrf_batch_uplo(a, n, "U")
        assert (info0 == 0).all()
        for j in range(n):
            a[:, j, j + 1:n] = 0.0
    a = with_sentinel(a, n, "U")
    fn = {"trtri": orc.trtri_batch, "lauum": orc.lauum_batch, "potri": orc.potri_batch,
          "poti": orc.poti_batch}[op]
    ref = a.copy()
    ref[:, :n, :n] = ref[:, :n, :n].transpose(0, 2, 1).copy()    # upper data -> lower
    fn(ref, n)
    ref[:, :n, :n] = ref[:, :n, :n].transpose(0, 2, 1).copy()
    dA = to_dev(gpu, a)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    flags = ("U", "N") if op == "trtri" else ("U",)
    assert handle.call(f"kblasD{op}_batch_strided", *flags, n, dA.data_ptr(), lda, n * lda, batch,
                       info.data_ptr()) == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    out = dA.cpu().numpy()
    assert other_tri_equal(out, a, n, "U")
    g = np.triu(out[:, :n, :n].transpose(0, 2, 1))
    r = np.triu(ref[:, :n, :n].transpose(0, 2, 1))
    assert np.abs(g - r).max() / np.abs(r).max() <= 100 * n * eps(np.float64)
