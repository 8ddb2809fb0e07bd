"""The C oracle against the LAPACK/BLAS golden vectors (CPU only).

Pins the oracle before it is trusted as the checker of the GPU library: every
routine is compared with what LAPACK/BLAS returned on the same inputs
(tests/golden/lapack_golden.npz, made by tests/golden/make_golden.py), and
info codes of non-SPD matrices must match exactly.
"""
import re

import numpy as np
import pytest

from gpu_util import eps


def colmajor(a2d: np.ndarray, dtype=None):
    """One row-major numpy matrix -> (1, ncols, ld=rows) column-major batch."""
    a = np.asarray(a2d, dtype=dtype)
    return np.array(a.T, order="C", copy=True)[None]


def keys(golden, pat):
    rx = re.compile(pat)
    return sorted({m.group(1) for k in golden.files for m in [rx.match(k)] if m})


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_potrf_posv_vs_lapack(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    ns = sorted(int(x) for x in keys(golden, rf"{pfx}potrf_n(\d+)_A"))
    assert ns, "no golden cases"
    for n in ns:
        A = golden[f"{pfx}potrf_n{n}_A"]
        Lref = golden[f"{pfx}potrf_n{n}_L"]
        a = colmajor(A, dt)
        info = orc.potrf_batch(a, n, nthreads=1)
        assert info[0] == int(golden[f"{pfx}potrf_n{n}_info"]) == 0
        L = np.tril(a[0].T)
        rel = np.abs(L - Lref).max() / np.abs(Lref).max()
        assert rel <= 10 * n * eps(dt), (n, rel)
        for m in (1, 4):
            B = golden[f"{pfx}posv_n{n}_m{m}_B"]
            Xref = golden[f"{pfx}posv_n{n}_m{m}_X"]
            a2 = colmajor(A, dt)
            b2 = colmajor(B, dt)  # (1, n, m): m x n column-major, ld = m
            info2 = orc.posv_batch(a2, b2, m, n, nthreads=1)
            assert info2[0] == 0
            X = b2[0].T
            err = np.abs(X - Xref).max() / np.abs(Xref).max()
            assert err <= 100 * n * eps(dt), (n, m, err)
            if pfx == "d":
                eta = orc.backward_error_r(colmajor(A), b2.astype(np.float64), colmajor(B), m, n)
                assert eta[0] <= 10 * n * eps(dt), (n, m, eta)


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_nonspd_info_exact(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    ns = sorted(int(x) for x in keys(golden, rf"{pfx}nonspd_n(\d+)_A"))
    assert ns
    for n in ns:
        a = colmajor(golden[f"{pfx}nonspd_n{n}_A"], dt)
        info = orc.potrf_batch(a, n, nthreads=1)
        assert info[0] == int(golden[f"{pfx}nonspd_n{n}_info"]), n


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_trsm_trmm_vs_blas(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    cases = keys(golden, rf"{pfx}tr_(\w+_m\d+_n\d+)_A")
    assert len(cases) >= 16 * 5
    for c in cases:
        flags, ms, ns = c.split("_")
        side, uplo, trans, diag = flags
        m, n = int(ms[1:]), int(ns[1:])
        A = golden[f"{pfx}tr_{c}_A"]
        B = golden[f"{pfx}tr_{c}_B"]
        ka = m if side == "L" else n
        for op, key in ((orc.trsm_batch, "trsm"), (orc.trmm_batch, "trmm")):
            a = colmajor(A, dt)
            b = colmajor(B, dt)
            op(side, uplo, trans, diag, m, n, 1.5, a, b, nthreads=1)
            ref = golden[f"{pfx}tr_{c}_{key}"]
            got = b[0].T
            err = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-30)
            assert err <= 50 * ka * eps(dt), (key, c, err)


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_syrk_vs_blas(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    cases = keys(golden, rf"{pfx}syrk_(\w_m\d+_k\d+)_A")
    assert cases
    for c in cases:
        trans, ms, ks = c.split("_")
        m, k = int(ms[1:]), int(ks[1:])
        a = colmajor(golden[f"{pfx}syrk_{c}_A"], dt)
        cm = colmajor(golden[f"{pfx}syrk_{c}_C"], dt)
        orc.syrk_batch("L", trans, m, k, -1.0, a, 1.0, cm, nthreads=1)
        ref = golden[f"{pfx}syrk_{c}_R"]
        got = np.tril(cm[0].T)
        scale = np.abs(golden[f"{pfx}syrk_{c}_C"]).max() + k * np.abs(golden[f"{pfx}syrk_{c}_A"]).max() ** 2
        assert np.abs(got - ref).max() <= 10 * k * eps(dt) * scale, c


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_gemm_vs_blas(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    cases = keys(golden, rf"{pfx}gemm_(\w\w_m\d+_n\d+_k\d+)_A")
    assert len(cases) == 24
    for c in cases:
        tt, ms, ns, ks = c.split("_")
        m, n, k = int(ms[1:]), int(ns[1:]), int(ks[1:])
        g = {x: golden[f"{pfx}gemm_{c}_{x}"] for x in ("A", "B", "C", "ab", "R")}
        a, b, cm = colmajor(g["A"], dt), colmajor(g["B"], dt), colmajor(g["C"], dt)
        alpha, beta = (float(v) for v in g["ab"])
        orc.gemm_batch(tt[0], tt[1], m, n, k, alpha, a, b, beta, cm, nthreads=1)
        got = cm[0].T
        scale = (abs(beta) * np.abs(g["C"]).max() + abs(alpha) * k * np.abs(g["A"]).max(initial=0)
                 * np.abs(g["B"]).max(initial=0) + 1e-30)
        assert np.abs(got - g["R"]).max() <= 10 * max(k, 1) * eps(dt) * scale, c


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_syrk_upper_vs_blas(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    cases = keys(golden, rf"{pfx}syrku_(\w_m\d+_k\d+)_A")
    assert cases
    for c in cases:
        trans, ms, ks = c.split("_")
        m, k = int(ms[1:]), int(ks[1:])
        a = colmajor(golden[f"{pfx}syrku_{c}_A"], dt)
        cm = colmajor(golden[f"{pfx}syrku_{c}_C"], dt)
        orc.syrk_batch("U", trans, m, k, -1.0, a, 1.0, cm, nthreads=1)
        got = np.triu(cm[0].T)
        scale = np.abs(golden[f"{pfx}syrku_{c}_C"]).max() + k * np.abs(golden[f"{pfx}syrku_{c}_A"]).max() ** 2
        assert np.abs(got - golden[f"{pfx}syrku_{c}_R"]).max() <= 10 * k * eps(dt) * scale, c
        # the strict lower triangle is not touched
        c0 = golden[f"{pfx}syrku_{c}_C"].astype(dt)
        assert np.array_equal(np.tril(cm[0].T, -1), np.tril(c0, -1))


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_potrf_uplo_and_side_l_potrs_vs_lapack(golden, orc, pfx):
    """Upper POTRF through the transposed lower restatement, and POTRS with
    side 'L' (LAPACK's own xPOTRS) for both triangles, against LAPACK."""
    dt = np.float64 if pfx == "d" else np.float32
    ns = sorted(int(x) for x in keys(golden, rf"{pfx}potrfu_n(\d+)_A"))
    assert ns
    for n in ns:
        for uplo in "LU":
            g = {x: golden[f"{pfx}potrf{uplo.lower()}_n{n}_{x}"] for x in "AFBX"}
            a = colmajor(g["A"], dt)
            a_before = a.copy()
            info = orc.potrf_batch_uplo(a, n, uplo, nthreads=1)
            assert info[0] == 0
            tri = np.triu if uplo == "U" else np.tril
            F = tri(a[0].T)
            assert np.abs(F - g["F"]).max() <= 10 * n * eps(dt) * np.abs(g["F"]).max(), (n, uplo)
            other = np.tril(a[0].T, -1) if uplo == "U" else np.triu(a[0].T, 1)
            other0 = np.tril(a_before[0].T, -1) if uplo == "U" else np.triu(a_before[0].T, 1)
            assert np.array_equal(other, other0), "the other triangle was written"
            b = colmajor(g["B"], dt)           # n x 3, column-major
            orc.potrs_batch_side("L", uplo, n, 3, a, b, nthreads=1)
            X = b[0].T
            scale = np.abs(g["X"]).max()
            assert np.abs(X - g["X"]).max() <= 1e3 * n * eps(dt) * scale, (n, uplo)
    if pfx == "d":
        a = colmajor(golden["dpotrfu_bad_n40_A"])
        info = orc.potrf_batch_uplo(a, 40, "U", nthreads=1)
        assert info[0] == int(golden["dpotrfu_bad_n40_info"]) == 18


CEPS = {"z": 2.0 ** -53, "c": 2.0 ** -24}


@pytest.mark.parametrize("pfx", ["z", "c"])
def test_complex_blas_vs_blas(golden, orc, pfx):
    """Complex GEMM / SYRK / TRSM / TRMM (transpose, never conjugate) against
    BLAS zgemm / zsyrk / ztrsm / ztrmm (and the c routines)."""
    dt = np.complex128 if pfx == "z" else np.complex64
    e = CEPS[pfx]
    for c in keys(golden, rf"{pfx}gemm_(\w\w_m\d+_n\d+_k\d+)_A"):
        tt, ms, ns, ks = c.split("_")
        m, n, k = int(ms[1:]), int(ns[1:]), int(ks[1:])
        g = {x: golden[f"{pfx}gemm_{c}_{x}"] for x in "ABCR"}
        cm = colmajor(g["C"], dt)
        orc.gemm_batch(tt[0], tt[1], m, n, k, 1.5 - 0.5j, colmajor(g["A"], dt), colmajor(g["B"], dt),
                       0.25 + 1j, cm, nthreads=1)
        scale = 2 * k * np.abs(g["A"]).max() * np.abs(g["B"]).max() + 2 * np.abs(g["C"]).max()
        assert np.abs(cm[0].T - g["R"]).max() <= 20 * k * e * scale, c
    for c in keys(golden, rf"{pfx}syrk_(\w_m\d+_k\d+)_A"):
        trans, ms, ks = c.split("_")
        m, k = int(ms[1:]), int(ks[1:])
        cm = colmajor(golden[f"{pfx}syrk_{c}_C"], dt)
        orc.syrk_batch("L", trans, m, k, -1.0, colmajor(golden[f"{pfx}syrk_{c}_A"], dt), 1.0, cm,
                       nthreads=1)
        scale = 2 * k * np.abs(golden[f"{pfx}syrk_{c}_A"]).max() ** 2 + np.abs(golden[f"{pfx}syrk_{c}_C"]).max()
        assert np.abs(np.tril(cm[0].T) - golden[f"{pfx}syrk_{c}_R"]).max() <= 20 * k * e * scale, c
    for c in keys(golden, rf"{pfx}tri_(\w_m\d+_n\d+)_L"):
        trans, ms, ns = c.split("_")
        m, n = int(ms[1:]), int(ns[1:])
        L = colmajor(golden[f"{pfx}tri_{c}_L"], dt)
        for op, fn in (("trsm", orc.trsm_batch), ("trmm", orc.trmm_batch)):
            b = colmajor(golden[f"{pfx}tri_{c}_B"], dt)
            fn("L", "L", trans, "N", m, n, 0.5 + 0.5j, L, b, nthreads=1)
            ref = golden[f"{pfx}tri_{c}_{op}"]
            assert np.abs(b[0].T - ref).max() <= 100 * m * e * np.abs(ref).max(), (c, op)


@pytest.mark.parametrize("pfx", ["z", "c"])
def test_complex_symmetric_cholesky_properties(orc, pfx):
    """Complex POTRF / POTRS / POSV / inversion have no LAPACK counterpart
    (LAPACK's xPOTRF is Hermitian); the complex-symmetric forms are pinned by
    their defining identities on the reference's test recipe (random, diagonal
    += n + n i, symmetrized): L L^T = A, X A = B, A inv(A) = I, and on
    real-valued complex input they equal the real routines."""
    dt = np.complex128 if pfx == "z" else np.complex64
    e = CEPS[pfx]
    rng = np.random.default_rng(5)
    for n in (1, 7, 30, 65):
        g = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        g[np.arange(n), np.arange(n)] += n + 1j * n
        a = np.tril(g) + np.tril(g, -1).T
        A = colmajor(a, dt)
        L = A.copy()
        assert orc.potrf_batch(L, n, nthreads=1)[0] == 0
        Lr = np.tril(L[0].T).astype(np.complex128)
        assert np.abs(Lr @ Lr.T - a).max() <= 30 * n * e * np.abs(a).max(), n
        b = rng.standard_normal((3, n)) + 1j * rng.standard_normal((3, n))
        B = colmajor(b, dt)
        X = B.copy()
        orc.potrs_batch(L, X, 3, n, nthreads=1)
        x = X[0].T.astype(np.complex128)
        assert np.abs(x @ a - b).max() <= 100 * n * e * np.abs(a).max() * np.abs(x).max(), n
        Ai = A.copy()
        assert orc.poti_batch(Ai, n, nthreads=1)[0] == 0
        li = np.tril(Ai[0].T).astype(np.complex128)
        inv = li + np.tril(li, -1).T
        assert np.abs(inv @ a - np.eye(n)).max() <= 300 * n * e * np.abs(a).max() * np.abs(inv).max()
        # real-valued complex input: the same numbers as the real factorization
        ar = a.real + n * np.eye(n)
        Lc = colmajor(ar, dt)
        Lre = colmajor(ar, np.float64 if pfx == "z" else np.float32)
        orc.potrf_batch(Lc, n, nthreads=1)
        orc.potrf_batch(Lre, n, nthreads=1)
        assert np.abs(np.tril(Lc[0].T).imag).max() == 0
        assert np.abs(np.tril(Lc[0].T).real - np.tril(Lre[0].T)).max() <= 10 * n * e * np.abs(ar).max()


def test_backward_error_detects_wrong_solution(orc):
    """A planted mistake in the solution must blow the backward error up."""
    rng = np.random.default_rng(1)
    n, m = 24, 2
    g = rng.standard_normal((n, n))
    A = g @ g.T + n * np.eye(n)
    B = rng.standard_normal((m, n))
    X = np.linalg.solve(A, B.T).T
    a, x, b = colmajor(A), colmajor(X), colmajor(B)
    good = orc.backward_error_r(a, x, b, m, n)[0]
    assert good <= 10 * n * 2.0 ** -53
    X2 = X.copy()
    X2[1, 5] *= 1 + 1e-9
    bad = orc.backward_error_r(a, colmajor(X2), b, m, n)[0]
    assert bad > 100 * good and bad > 10 * n * 2.0 ** -53


def test_oracle_threads_agree(orc):
    """OpenMP batching gives the same bits as a single thread."""
    rng = np.random.default_rng(2)
    n, batch = 20, 64
    g = rng.standard_normal((batch, n, n))
    a = np.einsum("bij,bkj->bik", g, g) + n * np.eye(n)
    a1 = np.ascontiguousarray(a)
    a2 = a1.copy()
    i1 = orc.potrf_batch(a1, n, nthreads=1)
    i2 = orc.potrf_batch(a2, n, nthreads=4)
    assert (i1 == 0).all() and (i2 == 0).all()
    assert np.array_equal(a1, a2)


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_inversion_vs_lapack(golden, orc, pfx):
    """xTRTRI, xLAUUM and xPOTRI (lower) of the oracle against LAPACK, and POTI
    (POTRF + POTRI) against LAPACK's POTRI of LAPACK's factor."""
    dt = np.float64 if pfx == "d" else np.float32
    ns = sorted(int(x) for x in keys(golden, rf"{pfx}inv_n(\d+)_A"))
    assert ns, "no golden cases"
    for n in ns:
        L = golden[f"{pfx}inv_n{n}_L"]
        tol = 50 * n * eps(dt)
        for name, fn in (("trtri", orc.trtri_batch), ("lauum", orc.lauum_batch),
                         ("potri", orc.potri_batch)):
            ref = golden[f"{pfx}inv_n{n}_{name}"]
            a = colmajor(L, dt)
            info = fn(a, n, nthreads=1)
            if info is not None:
                assert info[0] == 0
            got = np.tril(a[0].T)
            rel = np.abs(got - ref).max() / np.abs(ref).max()
            assert rel <= tol * (10 if name == "potri" else 1), (name, n, rel)
        a = colmajor(golden[f"{pfx}inv_n{n}_A"], dt)
        assert orc.poti_batch(a, n, nthreads=1)[0] == 0
        ref = golden[f"{pfx}inv_n{n}_potri"]
        rel = np.abs(np.tril(a[0].T) - ref).max() / np.abs(ref).max()
        assert rel <= 500 * n * eps(dt), (n, rel)


@pytest.mark.parametrize("pfx", ["d", "s"])
def test_trtri_singular_info_and_unchanged(golden, orc, pfx):
    dt = np.float64 if pfx == "d" else np.float32
    ns = sorted(int(x) for x in keys(golden, rf"{pfx}trtri_sing_n(\d+)_L"))
    assert ns
    for n in ns:
        L = golden[f"{pfx}trtri_sing_n{n}_L"]
        a = colmajor(L, dt)
        a0 = a.copy()
        info = orc.trtri_batch(a, n, nthreads=1)
        assert info[0] == int(golden[f"{pfx}trtri_sing_n{n}_info"])
        assert np.array_equal(a, a0), "a singular matrix must be left unchanged"



def test_host_lapack_batch_loop_matches_restatement(orc):
    """The timed CPU baseline's loop over the host LAPACK (dpotrf + dpotrs
    through function pointers, OpenMP over the batch) gives the restatement's
    info codes exactly and the same solutions to rounding, on ragged orders
    with planted non-SPD systems."""
    pytest.importorskip("scipy.linalg.cython_lapack")
    if orc.host_lapack() is None:
        pytest.skip("no host LAPACK")
    rng = np.random.default_rng(7)
    ns = [int(x) for x in rng.integers(1, 140, 400)]
    As, Bs = [], []
    for k, n in enumerate(ns):
        g = rng.standard_normal((n, n))
        a = np.ascontiguousarray(g @ g.T + n * np.eye(n))
        if k % 13 == 5:
            j = k % n
            a[j, j] = -abs(a[j, j])  # leading minor j+1 not positive definite
        As.append(a)
        Bs.append(rng.standard_normal((n, 1)))
    A1, B1 = [a.copy() for a in As], [b.copy() for b in Bs]
    A2, B2 = [a.copy() for a in As], [b.copy() for b in Bs]
    info1 = orc.lapack_posv1_vbatch(ns, A1, ns, B1)
    info2 = orc.posv_vbatch([1] * len(ns), ns, A2, ns, B2, [1] * len(ns))
    assert np.array_equal(info1, info2)
    assert (info1 > 0).sum() == len(range(5, 400, 13))
    for k, n in enumerate(ns):
        if info1[k] == 0:
            assert np.abs(B1[k] - B2[k]).max() <= 1e3 * n * 2.0 ** -53 * np.abs(B2[k]).max()
        else:
            assert np.array_equal(B1[k], Bs[k])  # not solved
