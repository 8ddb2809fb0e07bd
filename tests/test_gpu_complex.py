"""GPU parity of the complex (C, Z) routines against the complex oracle (pinned
in test_oracle.py). These are the reference's complex-symmetric forms: POTRF
factors A = L L^T without conjugation, op = transpose, SYRK forms A A^T; the
matrices follow the reference's complex test recipe (random entries, diagonal
+= n + n i, symmetrized; testing/testing_helper.cu:405-414).

Bars: results within c * n * eps of the oracle relative to the largest entry
(c = 30 for factors and products, 300 for inverses), info codes identical,
the triangle that is not referenced and the padding unchanged."""
import numpy as np
import pytest

from gpu_util import ptr_array, to_dev

pytestmark = pytest.mark.gpu

EPS = {np.complex128: 2.0 ** -53, np.complex64: 2.0 ** -24}
PFX = {np.complex128: "Z", np.complex64: "C"}
DTS = [np.complex128, np.complex64]
IDS = ["z", "c"]


def csym(batch, n, ld, seed, dt):
    """(batch, n, ld) column-major complex-symmetric matrices; padding rows -3."""
    rng = np.random.default_rng(seed)
    out = np.full((batch, max(n, 1), max(ld, 1)), -3.0 + 0j)
    for b in range(batch):
        g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        g[np.arange(n), np.arange(n)] += n + 1j * n
        a = np.tril(g) + np.tril(g, -1).T
        out[b, :n, :n] = a.T
    return out.astype(dt)


def cgen(batch, rows, cols, ld, seed, dt):
    rng = np.random.default_rng(seed)
    out = np.full((batch, max(cols, 1), max(ld, 1)), np.nan + 0j)
    out[:, :cols, :rows] = rng.standard_normal((batch, cols, rows)) + 1j * rng.standard_normal((batch, cols, rows))
    return out.astype(dt)


def rel(got, ref):
    return np.abs(got.astype(np.complex128) - ref.astype(np.complex128)).max() / max(np.abs(ref).max(), 1e-300)


@pytest.mark.parametrize("dt", DTS, ids=IDS)
@pytest.mark.parametrize("n", [1, 5, 16, 32, 33, 64, 100])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_potrf_posv_potrs(gpu, handle, orc, dt, n, form):
    batch, m = (12 if n <= 64 else 4), 3
    lda, ldb = n + 1, m + 2
    a = csym(batch, n, lda, seed=n, dt=dt)
    a[2, 0, 0] = 0           # matrix 2: zero first pivot -> info 1
    b = cgen(batch, m, n, ldb, seed=n + 1, dt=dt)
    pfx = PFX[dt]
    refA, refB = a.copy(), b.copy()
    info_ref = orc.posv_batch(refA, refB, m, n)
    assert info_ref[2] == 1
    dA, dB = to_dev(gpu, a), to_dev(gpu, b)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    if form == "strided":
        st = handle.call(f"kblas{pfx}posv_batch_strided", "R", "L", m, n, dA.data_ptr(), lda, n * lda,
                         dB.data_ptr(), ldb, n * ldb, batch, info.data_ptr())
    else:
        pa, pb = ptr_array(gpu, dA), ptr_array(gpu, dB)
        st = handle.call(f"kblas{pfx}posv_batch", "R", "L", m, n, pa.data_ptr(), lda, pb.data_ptr(), ldb,
                         batch, info.data_ptr())
    assert st == 1
    gpu.cuda.synchronize()
    assert np.array_equal(info.cpu().numpy(), info_ref)
    F, X = dA.cpu().numpy(), dB.cpu().numpy()
    ok = info_ref == 0
    tol = 30 * n * EPS[dt]
    for s in np.where(ok)[0]:
        assert rel(np.tril(F[s, :n, :n].T), np.tril(refA[s, :n, :n].T)) <= tol, s
        assert rel(X[s, :n, :m], refB[s, :n, :m]) <= 10 * tol, s
    assert np.array_equal(X[~ok], b[~ok], equal_nan=True)
    for j in range(n):      # strict upper triangle untouched
        assert np.array_equal(F[:, j, :j], a[:, j, :j])
    # POTRS with the GPU factor of the good systems, side L (two TRSM passes)
    good = np.where(ok)[0]
    Fk = np.ascontiguousarray(F[good])
    bl = cgen(len(good), n, m, n + 2, seed=n + 2, dt=dt)       # side L: B is n x m
    dF, dBl = to_dev(gpu, Fk), to_dev(gpu, bl)
    assert handle.call(f"kblas{pfx}potrs_batch_strided", "L", "L", n, m, dF.data_ptr(), lda, n * lda,
                       dBl.data_ptr(), n + 2, m * (n + 2), len(good)) == 1
    gpu.cuda.synchronize()
    ref = bl.copy()
    orc.potrs_batch_side("L", "L", n, m, Fk.copy(), ref)
    assert rel(dBl.cpu().numpy()[:, :m, :n], ref[:, :m, :n]) <= 10 * tol


@pytest.mark.parametrize("dt", DTS, ids=IDS)
@pytest.mark.parametrize("n", [6, 40])
def test_potrf_upper(gpu, handle, orc, dt, n):
    batch = 6
    a = csym(batch, n, n, seed=3 * n, dt=dt)
    dA = to_dev(gpu, a)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert handle.call(f"kblas{PFX[dt]}potrf_batch_strided", "U", n, dA.data_ptr(), n, n * n, batch,
                       info.data_ptr()) == 1
    gpu.cuda.synchronize()
    ref = a.copy()
    info_ref = orc.potrf_batch_uplo(ref, n, "U")
    assert np.array_equal(info.cpu().numpy(), info_ref)
    out = dA.cpu().numpy()
    assert rel(np.triu(out[:, :n, :n].transpose(0, 2, 1)), np.triu(ref[:, :n, :n].transpose(0, 2, 1))) \
        <= 30 * n * EPS[dt]


COMBOS = [("L", "L", "N", "N"), ("L", "U", "T", "U"), ("R", "L", "T", "N"), ("R", "U", "N", "N")]


@pytest.mark.parametrize("dt", DTS, ids=IDS)
@pytest.mark.parametrize("combo", COMBOS, ids=["".join(c) for c in COMBOS])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_trsm_trmm(gpu, handle, orc, dt, combo, form):
    side, uplo, trans, diag = combo
    m, n, batch = 37, 20, 7
    k = m if side == "L" else n
    rng = np.random.default_rng(len(form) + COMBOS.index(combo))
    lda, ldb = k + 1, m + 2
    a = np.full((batch, k, lda), np.nan + 0j)
    for s in range(batch):
        L = np.tril(rng.standard_normal((k, k)) + 1j * rng.standard_normal((k, k))) / np.sqrt(k)
        L[np.arange(k), np.arange(k)] = rng.uniform(1, 2, k) + 0.5j
        M = L if uplo == "L" else L.T
        a[s, :, :k] = M.T
    a = a.astype(dt)
    b = cgen(batch, m, n, ldb, seed=9, dt=dt)
    alpha = 0.75 - 0.25j
    pfx = PFX[dt]
    for op, fn in (("trsm", orc.trsm_batch), ("trmm", orc.trmm_batch)):
        ref = b.copy()
        fn(side, uplo, trans, diag, m, n, alpha, np.nan_to_num(a), ref)
        dA, dB = to_dev(gpu, a), to_dev(gpu, b)
        if form == "strided":
            st = handle.call(f"kblas{pfx}{op}_batch_strided", side, uplo, trans, diag, m, n, alpha,
                             dA.data_ptr(), lda, k * lda, dB.data_ptr(), ldb, n * ldb, batch)
        else:
            pa, pb = ptr_array(gpu, dA), ptr_array(gpu, dB)
            st = handle.call(f"kblas{pfx}{op}_batch", side, uplo, trans, diag, m, n, alpha, pa.data_ptr(),
                             lda, pb.data_ptr(), ldb, batch)
        assert st == 1
        gpu.cuda.synchronize()
        out = dB.cpu().numpy()
        assert np.array_equal(out[:, :, m:], b[:, :, m:], equal_nan=True)
        assert rel(out[:, :, :m], ref[:, :, :m]) <= 300 * k * EPS[dt], op


@pytest.mark.parametrize("dt", DTS, ids=IDS)
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_syrk_gemm(gpu, handle, orc, dt, uplo, trans):
    m, k, batch = 45, 19, 6
    rows, cols = (m, k) if trans == "N" else (k, m)
    a = cgen(batch, rows, cols, rows + 1, seed=11, dt=dt)
    c = csym(batch, m, m + 2, seed=12, dt=dt)
    alpha, beta = -1.0 + 0.5j, 0.5 - 1j
    ref = c.copy()
    orc.syrk_batch(uplo, trans, m, k, alpha, np.nan_to_num(a), beta, ref)
    dA, dC = to_dev(gpu, a), to_dev(gpu, c)
    pfx = PFX[dt]
    assert handle.call(f"kblas{pfx}syrk_batch_strided", uplo, trans, m, k, alpha, dA.data_ptr(),
                       rows + 1, cols * (rows + 1), beta, dC.data_ptr(), m + 2, m * (m + 2), batch) == 1
    gpu.cuda.synchronize()
    out = dC.cpu().numpy()
    tri = np.tril if uplo == "L" else np.triu
    assert rel(tri(out[:, :m, :m].transpose(0, 2, 1)), tri(ref[:, :m, :m].transpose(0, 2, 1))) \
        <= 30 * k * EPS[dt]
    # GEMM C := alpha op(A) op(B) + beta C, op(B) = A^T's shape
    n = 23
    bm = cgen(batch, k, n, k + 3, seed=13, dt=dt)
    cg = cgen(batch, m, n, m + 1, seed=14, dt=dt)
    refg = cg.copy()
    orc.gemm_batch(trans, "N", m, n, k, alpha, np.nan_to_num(a), np.nan_to_num(bm), beta, refg)
    dB, dG = to_dev(gpu, bm), to_dev(gpu, cg)
    pa, pb, pg = ptr_array(gpu, dA), ptr_array(gpu, dB), ptr_array(gpu, dG)
    assert handle.call(f"kblas{pfx}gemm_batch", trans, "N", m, n, k, alpha, pa.data_ptr(), rows + 1,
                       pb.data_ptr(), k + 3, beta, pg.data_ptr(), m + 1, batch) == 1
    gpu.cuda.synchronize()
    outg = dG.cpu().numpy()
    assert np.array_equal(outg[:, :, m:], cg[:, :, m:], equal_nan=True)
    assert rel(outg[:, :, :m], refg[:, :, :m]) <= 30 * k * EPS[dt]


@pytest.mark.parametrize("dt", DTS, ids=IDS)
@pytest.mark.parametrize("op", ["trtri", "lauum", "potri", "poti"])
@pytest.mark.parametrize("n", [1, 9, 48, 70])
def test_inverse(gpu, handle, orc, dt, op, n):
    batch = 6
    a = csym(batch, n, n + 1, seed=5 * n, dt=dt)
    if op != "poti":
        assert (orc.potrf_batch(a, n) == 0).all()
    ref = a.copy()
    fn = {"trtri": orc.trtri_batch, "lauum": orc.lauum_batch, "potri": orc.potri_batch,
          "poti": orc.poti_batch}[op]
    info_ref = fn(ref, n)
    dA = to_dev(gpu, a)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    flags = ("L", "N") if op == "trtri" else ("L",)
    assert handle.call(f"kblas{PFX[dt]}{op}_batch_strided", *flags, n, dA.data_ptr(), n + 1,
                       n * (n + 1), batch, info.data_ptr()) == 1
    gpu.cuda.synchronize()
    if info_ref is not None:
        assert np.array_equal(info.cpu().numpy(), info_ref)
    out = dA.cpu().numpy()
    assert rel(np.tril(out[:, :n, :n].transpose(0, 2, 1)), np.tril(ref[:, :n, :n].transpose(0, 2, 1))) \
        <= 300 * n * EPS[dt]


@pytest.mark.parametrize("dt", DTS, ids=IDS)
def test_gemm_vbatch(gpu, handle, orc, dt):
    rng = np.random.default_rng(3)
    batch = 20
    ms, ns, ks = (rng.integers(1, 50, batch) for _ in range(3))
    As = [cgen(1, int(ms[i]), int(ks[i]), int(ms[i]), 100 + i, dt)[0] for i in range(batch)]
    Bs = [cgen(1, int(ks[i]), int(ns[i]), int(ks[i]), 200 + i, dt)[0] for i in range(batch)]
    Cs = [cgen(1, int(ms[i]), int(ns[i]), int(ms[i]), 300 + i, dt)[0] for i in range(batch)]
    dAs = [to_dev(gpu, x) for x in As]
    dBs = [to_dev(gpu, x) for x in Bs]
    dCs = [to_dev(gpu, x) for x in Cs]
    ptr = lambda ts: gpu.from_numpy(np.array([t.data_ptr() for t in ts], dtype=np.int64)).cuda()
    pA, pB, pC = ptr(dAs), ptr(dBs), ptr(dCs)
    iv = lambda v: gpu.from_numpy(np.asarray(v, dtype=np.int32)).cuda()
    dm, dn, dk = iv(ms), iv(ns), iv(ks)
    alpha, beta = 1 - 1j, 0.5j
    assert handle.call(f"kblas{PFX[dt]}gemm_vbatch", "N", "N", dm.data_ptr(), dn.data_ptr(),
                       dk.data_ptr(), 0, 0, 0, alpha, pA.data_ptr(), dm.data_ptr(), pB.data_ptr(),
                       dk.data_ptr(), beta, pC.data_ptr(), dm.data_ptr(), batch) == 1
    gpu.cuda.synchronize()
    for i in range(batch):
        ref = Cs[i][None].copy()
        orc.gemm_batch("N", "N", int(ms[i]), int(ns[i]), int(ks[i]), alpha, As[i][None], Bs[i][None],
                       beta, ref, nthreads=1)
        assert rel(dCs[i].cpu().numpy(), ref[0]) <= 30 * int(ks[i]) * EPS[dt], i
