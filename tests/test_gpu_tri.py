"""GPU parity of batched TRSM / TRMM (every side/uplo/trans/diag) and SYRK
against the CPU oracle, on the benchmark's triangle recipe (off-diagonal
N(0,1)/sqrt(n), diagonal U[1,2]); strided and pointer-array forms.

Tolerances: the GPU and the oracle evaluate the same sums in a different
order, so results agree to a few units of eps times the size of the terms:
TRMM/SYRK elementwise |diff| <= 10 k eps * (|op(A)| |B|) (resp. |A||A|^T);
TRSM through its residual |op(A) X - alpha B| <= 10 k eps (|op(A)| |X|)."""
import itertools

import numpy as np
import pytest

from gpu_util import dense, eps, ptr_array, to_dev

pytestmark = pytest.mark.gpu


def tri_input(wl, batch, k, uplo, seed, dt, ld=None):
    a = wl.lower_tri(batch, k, seed=seed, ld=ld, upper_fill=np.nan)
    if uplo == "U":  # transpose each matrix: upper triangle holds the data, NaN below
        for b in range(batch):
            kk = a.shape[1]
            t = a[b, :k, :k].T.copy()
            a[b, :k, :k] = t
    return a.astype(dt)


def op_dense(a, k, uplo, trans, diag):
    """op(A) as dense (batch, k, k) float64 with the unused triangle zeroed."""
    A = dense(a.astype(np.float64), k, k)
    A = np.nan_to_num(A, nan=0.0)
    A = np.tril(A) if uplo == "L" else np.triu(A)
    if diag == "U":
        idx = np.arange(k)
        A[:, idx, idx] = 1.0
    return A.transpose(0, 2, 1) if trans == "T" else A


COMBOS = list(itertools.product("LR", "LU", "NT", "NU"))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("combo", COMBOS, ids=["".join(c) for c in COMBOS])
@pytest.mark.parametrize("shape", [(5, 3), (16, 16), (33, 7), (64, 64), (3, 70), (130, 9)])
def test_trsm_trmm(gpu, handle, wl, orc, dt, combo, shape):
    side, uplo, trans, diag = combo
    m, n = shape
    k = m if side == "L" else n
    batch = 13
    lda, ldb = k + 2, m + 1
    a = tri_input(wl, batch, k, uplo, seed=m * 31 + n, dt=dt, ld=lda)
    b = wl.general(batch, m, n, seed=m + n, ld=ldb).astype(dt)
    alpha = 1.5
    pfx = "D" if dt == np.float64 else "S"
    Aop = op_dense(a, k, uplo, trans, diag)
    for op, name in (("trsm", "trsm"), ("trmm", "trmm")):
        for form in ("strided", "array"):
            da, db = to_dev(gpu, a), to_dev(gpu, b)
            if form == "strided":
                st = handle.call(f"kblas{pfx}{op}_batch_strided", side, uplo, trans, diag, m, n, alpha,
                                 da.data_ptr(), lda, k * lda, db.data_ptr(), ldb, n * ldb, batch)
            else:
                pa, pb = ptr_array(gpu, da), ptr_array(gpu, db)
                st = handle.call(f"kblas{pfx}{op}_batch", side, uplo, trans, diag, m, n, alpha,
                                 pa.data_ptr(), lda, pb.data_ptr(), ldb, batch)
            assert st == 1, (name, form, st)
            gpu.cuda.synchronize()
            out = db.cpu().numpy()
            assert np.array_equal(out[:, :, m:], b[:, :, m:]), "ldb padding written"
            X = dense(out.astype(np.float64), m, n)
            B = dense(b.astype(np.float64), m, n)
            if name == "trsm":
                # residual op(A) X - alpha B  (side L)  or  X op(A) - alpha B  (side R)
                prod = Aop @ X if side == "L" else X @ Aop
                absprod = np.abs(Aop) @ np.abs(X) if side == "L" else np.abs(X) @ np.abs(Aop)
                res = np.abs(prod - alpha * B)
                bound = 10 * k * eps(dt) * (absprod + abs(alpha) * np.abs(B)) + 1e-300
                assert (res <= bound).all(), (name, form, combo, shape, (res / bound).max())
            else:
                ref = b.copy()
                orc.trmm_batch(side, uplo, trans, diag, m, n, alpha, np.nan_to_num(a, nan=0.0), ref)
                R = dense(ref.astype(np.float64), m, n)
                absprod = np.abs(Aop) @ np.abs(B) if side == "L" else np.abs(B) @ np.abs(Aop)
                bound = 10 * k * eps(dt) * abs(alpha) * absprod + 1e-300
                assert (np.abs(X - R) <= bound).all(), (name, form, combo, shape)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
def test_trsm_alpha_zero_does_not_read_A(gpu, handle, dt):
    pfx = "D" if dt == np.float64 else "S"
    batch, m, n = 3, 9, 5
    a = np.full((batch, m, m), np.nan, dtype=dt)
    b = np.ones((batch, n, m), dtype=dt)
    da, db = to_dev(gpu, a), to_dev(gpu, b)
    st = handle.call(f"kblas{pfx}trsm_batch_strided", "L", "L", "N", "N", m, n, 0.0, da.data_ptr(), m,
                     m * m, db.data_ptr(), m, m * n, batch)
    assert st == 1
    gpu.cuda.synchronize()
    assert (db.cpu().numpy() == 0).all()


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("mk", [(1, 1), (5, 3), (16, 16), (33, 17), (64, 64), (70, 9), (100, 130)])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_syrk(gpu, handle, wl, orc, dt, uplo, trans, mk, form):
    m, k = mk
    batch = 11
    rows, cols = (m, k) if trans == "N" else (k, m)
    lda, ldc = rows + 1, m + 2
    a = wl.general(batch, rows, cols, seed=m + 3 * k, ld=lda).astype(dt)
    c = wl.spd_shifted(batch, m, seed=m, ld=ldc).astype(dt)
    # sentinel in the triangle of C that is not referenced must survive
    # (column j of the column-major batch holds rows 0..ld-1)
    other = [slice(0, j) if uplo == "L" else slice(j + 1, m) for j in range(m)]
    for j in range(m):
        c[:, j, other[j]] = -3.5
    ref = c.copy()
    orc.syrk_batch(uplo, trans, m, k, -1.0, a, 1.0, ref)
    pfx = "D" if dt == np.float64 else "S"
    da, dc = to_dev(gpu, a), to_dev(gpu, c)
    if form == "strided":
        st = handle.call(f"kblas{pfx}syrk_batch_strided", uplo, trans, m, k, -1.0, da.data_ptr(), lda,
                         cols * lda, 1.0, dc.data_ptr(), ldc, m * ldc, batch)
    else:
        pa, pc = ptr_array(gpu, da), ptr_array(gpu, dc)
        st = handle.call(f"kblas{pfx}syrk_batch", uplo, trans, m, k, -1.0, pa.data_ptr(), lda, 1.0,
                         pc.data_ptr(), ldc, batch)
    assert st == 1
    gpu.cuda.synchronize()
    out = dc.cpu().numpy()
    for j in range(m):
        assert (out[:, j, other[j]] == -3.5).all(), "unreferenced triangle of C written"
        assert np.array_equal(out[:, j, m:], c[:, j, m:]), "ldc padding written"
    A = dense(a.astype(np.float64), rows, cols)
    opA = A if trans == "N" else A.transpose(0, 2, 1)
    scale = np.abs(opA) @ np.abs(opA).transpose(0, 2, 1) + np.abs(dense(c.astype(np.float64), m, m))
    tri = np.tril if uplo == "L" else np.triu
    G = tri(dense(out.astype(np.float64), m, m))
    R = tri(dense(ref.astype(np.float64), m, m))
    assert (np.abs(G - R) <= 10 * max(k, 1) * eps(dt) * tri(scale) + 1e-300).all()
