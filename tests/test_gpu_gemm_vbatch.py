"""GPU parity of batched GEMM (uniform: strided and pointer-array) and of the
variable-size GEMM / SYRK / TRSM (per-matrix sizes and leading dimensions in
device arrays), against the CPU oracle (pinned to BLAS in test_oracle.py).

Bars: the GPU and the oracle form the same dot products in a different
order, so each entry agrees within 10 k eps of the size of its terms
(|alpha| |op(A)| |op(B)| + |beta| |C|); TRSM is judged by its residual
|op(A) X - alpha B| <= 10 k eps (|op(A)| |X| + |alpha| |B|). Entries outside
each matrix (leading-dimension padding, the other triangle for SYRK) must
come back bit-identical, and C is not read when beta == 0 (NaN there stays
out of the result)."""
import itertools

import numpy as np
import pytest

from gpu_util import eps, ptr_array, to_dev

pytestmark = pytest.mark.gpu


def colmajor_batch(rng, batch, rows, cols, ld, dt, fill=None):
    a = np.full((batch, max(cols, 1), max(ld, 1)), np.nan if fill is None else fill, dtype=np.float64)
    a[:, :cols, :rows] = rng.standard_normal((batch, cols, rows))
    return a.astype(dt)


def op_rows_cols(trans, rows, cols):
    return (cols, rows) if trans == "T" else (rows, cols)


def gemm_bound(dt, k, alpha, beta, A, B, C, ta, tb):
    """Elementwise bound 10 k eps (|alpha| |op(A)| |op(B)| + |beta| |C|)."""
    Ad = np.abs(np.nan_to_num(A.astype(np.float64)))
    Bd = np.abs(np.nan_to_num(B.astype(np.float64)))
    Ad = Ad.transpose(0, 2, 1) if ta == "N" else Ad       # -> op(A) row-major (m, k)
    Bd = Bd.transpose(0, 2, 1) if tb == "N" else Bd       # -> op(B) row-major (k, n)
    prod = abs(alpha) * (Ad @ Bd) if k > 0 else 0.0
    cterm = abs(beta) * np.abs(np.nan_to_num(C.astype(np.float64)).transpose(0, 2, 1)) if beta != 0 else 0.0
    return 10 * max(k, 1) * eps(dt) * (prod + cterm) + 1e-300


SHAPES = [(1, 1, 1), (5, 7, 3), (16, 16, 16), (32, 32, 32), (33, 65, 17), (64, 64, 64),
          (100, 3, 129), (7, 40, 0)]
TT = ["".join(t) for t in itertools.product("NT", "NT")]


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("tt", TT)
@pytest.mark.parametrize("shape", SHAPES, ids=[f"{m}x{n}x{k}" for m, n, k in SHAPES])
@pytest.mark.parametrize("form", ["strided", "array"])
def test_gemm_uniform(gpu, handle, orc, dt, tt, shape, form):
    m, n, k = shape
    ta, tb = tt
    batch = 9
    rng = np.random.default_rng(m * 1000 + n * 10 + k + len(form))
    ra, ca = op_rows_cols(ta, m, k)
    rb, cb = op_rows_cols(tb, k, n)
    lda, ldb, ldc = max(ra, 1) + 2, max(rb, 1) + 1, m + 3
    A = colmajor_batch(rng, batch, ra, ca, lda, dt)
    B = colmajor_batch(rng, batch, rb, cb, ldb, dt)
    C = colmajor_batch(rng, batch, m, n, ldc, dt)
    alpha, beta = (1.25, -0.75) if k % 2 else (-1.0, 0.5)
    ref = C.copy()
    orc.gemm_batch(ta, tb, m, n, k, alpha, np.nan_to_num(A), np.nan_to_num(B), beta, ref)
    dA, dB, dC = to_dev(gpu, A), to_dev(gpu, B), to_dev(gpu, C)
    pfx = "D" if dt == np.float64 else "S"
    if form == "strided":
        st = handle.call(f"kblas{pfx}gemm_batch_strided", ta, tb, m, n, k, alpha, dA.data_ptr(), lda,
                         A.shape[1] * lda, dB.data_ptr(), ldb, B.shape[1] * ldb, beta, dC.data_ptr(),
                         ldc, C.shape[1] * ldc, batch)
    else:
        pa, pb, pc = ptr_array(gpu, dA), ptr_array(gpu, dB), ptr_array(gpu, dC)
        st = handle.call(f"kblas{pfx}gemm_batch", ta, tb, m, n, k, alpha, pa.data_ptr(), lda,
                         pb.data_ptr(), ldb, beta, pc.data_ptr(), ldc, batch)
    assert st == 1
    gpu.cuda.synchronize()
    out = dC.cpu().numpy()
    assert np.array_equal(out[:, :, m:], C[:, :, m:], equal_nan=True), "ldc padding written"
    got = out[:, :n, :m].astype(np.float64).transpose(0, 2, 1)
    want = ref[:, :n, :m].astype(np.float64).transpose(0, 2, 1)
    bound = gemm_bound(dt, k, alpha, beta, A[:, :ca, :ra], B[:, :cb, :rb], C[:, :n, :m], ta, tb)
    assert (np.abs(got - want) <= bound).all(), np.abs(got - want).max()


def test_gemm_blas_corner_cases(gpu, handle, orc):
    """beta == 0: C is not read (NaN stays out); alpha == 0: A, B not read."""
    m, n, k, batch = 20, 12, 9, 4
    rng = np.random.default_rng(5)
    A = colmajor_batch(rng, batch, m, k, m, np.float64)
    B = colmajor_batch(rng, batch, k, n, k, np.float64)
    C = np.full((batch, n, m), np.nan)
    dA, dB, dC = to_dev(gpu, A), to_dev(gpu, B), to_dev(gpu, C)
    assert handle.call("kblasDgemm_batch_strided", "N", "N", m, n, k, 2.0, dA.data_ptr(), m, k * m,
                       dB.data_ptr(), k, n * k, 0.0, dC.data_ptr(), m, n * m, batch) == 1
    gpu.cuda.synchronize()
    ref = np.zeros_like(C)
    orc.gemm_batch("N", "N", m, n, k, 2.0, A, B, 0.0, ref)
    out = dC.cpu().numpy()
    assert np.isfinite(out).all()
    assert np.abs(out - ref).max() <= 10 * k * eps(np.float64) * 2 * np.abs(ref).max()
    # alpha == 0 with NaN operands: C := beta C exactly
    An = to_dev(gpu, np.full_like(A, np.nan))
    C2 = rng.standard_normal(C.shape)
    dC2 = to_dev(gpu, C2)
    assert handle.call("kblasDgemm_batch_strided", "N", "N", m, n, k, 0.0, An.data_ptr(), m, k * m,
                       An.data_ptr(), k, n * k, 3.0, dC2.data_ptr(), m, n * m, batch) == 1
    gpu.cuda.synchronize()
    assert np.array_equal(dC2.cpu().numpy(), 3.0 * C2)


def test_gemm_argument_codes(gpu, handle):
    P = 0
    # batchCount < 1 is an error for GEMM, as in the reference
    assert handle.call("kblasDgemm_batch_strided", "N", "N", 4, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0,
                       P, 4, 16, 0) == -10
    assert handle.call("kblasDgemm_batch_strided", "X", "N", 4, 4, 4, 1.0, P, 4, 16, P, 4, 16, 0.0,
                       P, 4, 16, 1) == -10
    assert handle.call("kblasDgemm_batch_strided", "N", "N", 4, 4, 4, 1.0, P, 3, 16, P, 4, 16, 0.0,
                       P, 4, 16, 1) == -10   # lda < m
    # m == 0: quick return
    assert handle.call("kblasDgemm_batch_strided", "N", "N", 0, 4, 4, 1.0, P, 1, 0, P, 4, 16, 0.0,
                       P, 1, 0, 3) == 1


# ----------------------------------------------------------------------------
# variable-size
# ----------------------------------------------------------------------------

class Ragged:
    """Matrices of different shapes, each column-major with its own leading
    dimension, packed into one device pool with NaN gaps between them."""

    def __init__(self, gpu, mats, dt):
        self.shapes = [a.shape for a in mats]     # (ncols, ld)
        sizes = [a.size for a in mats]
        self.offs = np.zeros(len(mats), dtype=np.int64)
        o = 5
        for i, s in enumerate(sizes):
            self.offs[i] = o
            o += s + 3
        pool = np.full(o + 8, np.nan, dtype=dt)
        for i, a in enumerate(mats):
            pool[self.offs[i]:self.offs[i] + a.size] = a.reshape(-1)
        self.host = pool
        self.dev = gpu.from_numpy(pool).cuda()
        itemsize = np.dtype(dt).itemsize
        self.ptrs = gpu.from_numpy(self.dev.data_ptr() + self.offs * itemsize).cuda()

    def get(self):
        pool = self.dev.cpu().numpy()
        return [pool[o:o + c * l].reshape(c, l) for o, (c, l) in zip(self.offs, self.shapes)]

    def gaps_untouched(self):
        pool = self.dev.cpu().numpy()
        mask = np.ones(pool.size, dtype=bool)
        for o, (c, l) in zip(self.offs, self.shapes):
            mask[o:o + c * l] = False
        return np.array_equal(pool[mask], self.host[mask], equal_nan=True)


def ivec(gpu, v):
    return gpu.from_numpy(np.asarray(v, dtype=np.int32)).cuda()


def rand_mat(rng, rows, cols, ld, dt):
    a = np.full((max(cols, 1), max(ld, 1)), np.nan)
    a[:cols, :rows] = rng.standard_normal((cols, rows))
    return a.astype(dt)


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("tt", TT)
@pytest.mark.parametrize("hint", ["max", "zero"])
def test_gemm_vbatch(gpu, handle, orc, dt, tt, hint):
    ta, tb = tt
    rng = np.random.default_rng(17 + len(hint) + 3 * TT.index(tt))
    batch = 60
    ms = rng.integers(0, 90, batch)
    ns = rng.integers(0, 90, batch)
    ks = rng.integers(0, 70, batch)
    ms[3], ns[7], ks[11] = 0, 0, 0
    ms[20], ns[20], ks[20] = 130, 97, 140     # several tiles in both directions
    As, Bs, Cs, lds = [], [], [], []
    for i in range(batch):
        ra, ca = op_rows_cols(ta, ms[i], ks[i])
        rb, cb = op_rows_cols(tb, ks[i], ns[i])
        lda, ldb, ldc = max(ra, 1) + rng.integers(0, 3), max(rb, 1) + rng.integers(0, 3), \
            max(ms[i], 1) + rng.integers(0, 3)
        As.append(rand_mat(rng, ra, ca, lda, dt))
        Bs.append(rand_mat(rng, rb, cb, ldb, dt))
        Cs.append(rand_mat(rng, ms[i], ns[i], ldc, dt))
        lds.append((lda, ldb, ldc))
    lds = np.array(lds)
    RA, RB, RC = Ragged(gpu, As, dt), Ragged(gpu, Bs, dt), Ragged(gpu, Cs, dt)
    alpha, beta = 0.75, -1.5
    dm, dn, dk = ivec(gpu, ms), ivec(gpu, ns), ivec(gpu, ks)
    dla, dlb, dlc = ivec(gpu, lds[:, 0]), ivec(gpu, lds[:, 1]), ivec(gpu, lds[:, 2])
    mx = (int(ms.max()), int(ns.max()), int(ks.max())) if hint == "max" else (0, 0, 0)
    pfx = "D" if dt == np.float64 else "S"
    st = handle.call(f"kblas{pfx}gemm_vbatch", ta, tb, dm.data_ptr(), dn.data_ptr(), dk.data_ptr(),
                     *mx, alpha, RA.ptrs.data_ptr(), dla.data_ptr(), RB.ptrs.data_ptr(),
                     dlb.data_ptr(), beta, RC.ptrs.data_ptr(), dlc.data_ptr(), batch)
    assert st == 1
    gpu.cuda.synchronize()
    outs = RC.get()
    assert RC.gaps_untouched()
    for i in range(batch):
        m, n, k = int(ms[i]), int(ns[i]), int(ks[i])
        ldc = int(lds[i, 2])
        got = outs[i]
        assert np.array_equal(got[:, m:], Cs[i][:, m:], equal_nan=True), ("padding", i)
        if m == 0 or n == 0:
            assert np.array_equal(got, Cs[i], equal_nan=True)
            continue
        ref = Cs[i][None].copy()
        orc.gemm_batch(ta, tb, m, n, k, alpha, np.nan_to_num(As[i])[None],
                       np.nan_to_num(Bs[i])[None], beta, ref, nthreads=1)
        ra, ca = op_rows_cols(ta, m, k)
        rb, cb = op_rows_cols(tb, k, n)
        bound = gemm_bound(dt, k, alpha, beta, As[i][None, :ca, :ra], Bs[i][None, :cb, :rb],
                           Cs[i][None, :n, :m], ta, tb)[0]
        diff = np.abs(got[:n, :m].astype(np.float64).T - ref[0, :n, :m].astype(np.float64).T)
        assert (diff <= bound).all(), (i, m, n, k, diff.max())
        del ldc


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("uplo", ["L", "U"])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_syrk_vbatch(gpu, handle, orc, dt, uplo, trans):
    rng = np.random.default_rng(31 + 2 * (uplo == "U") + (trans == "T"))
    batch = 50
    ms = rng.integers(0, 100, batch)
    ks = rng.integers(0, 60, batch)
    ms[4], ks[9] = 0, 0
    ms[10], ks[10] = 150, 77
    As, Cs, lds = [], [], []
    for i in range(batch):
        ra, ca = op_rows_cols(trans, ms[i], ks[i])
        lda, ldc = max(ra, 1) + rng.integers(0, 3), max(ms[i], 1) + rng.integers(0, 3)
        As.append(rand_mat(rng, ra, ca, lda, dt))
        Cs.append(rand_mat(rng, ms[i], ms[i], ldc, dt))
        lds.append((lda, ldc))
    lds = np.array(lds)
    RA, RC = Ragged(gpu, As, dt), Ragged(gpu, Cs, dt)
    alpha, beta = -1.0, 1.0
    pfx = "D" if dt == np.float64 else "S"
    # keep the device size arrays referenced until the kernel has run
    dm, dk, dla, dlc = ivec(gpu, ms), ivec(gpu, ks), ivec(gpu, lds[:, 0]), ivec(gpu, lds[:, 1])
    st = handle.call(f"kblas{pfx}syrk_vbatch", uplo, trans, dm.data_ptr(), dk.data_ptr(),
                     int(ms.max()), int(ks.max()), alpha, RA.ptrs.data_ptr(), dla.data_ptr(), beta,
                     RC.ptrs.data_ptr(), dlc.data_ptr(), batch)
    assert st == 1
    gpu.cuda.synchronize()
    outs = RC.get()
    assert RC.gaps_untouched()
    tri = np.tril if uplo == "L" else np.triu
    other = (lambda x: np.triu(x, 1)) if uplo == "L" else (lambda x: np.tril(x, -1))
    for i in range(batch):
        m, k = int(ms[i]), int(ks[i])
        if m == 0:
            continue
        got = outs[i][:m, :m].T.astype(np.float64)       # row-major m x m
        c0 = Cs[i][:m, :m].T.astype(np.float64)
        assert np.array_equal(other(got), other(c0), equal_nan=True), ("other triangle", i)
        assert np.array_equal(outs[i][:, m:], Cs[i][:, m:], equal_nan=True), ("padding", i)
        ref = Cs[i][None].copy()
        orc.syrk_batch(uplo, trans, m, k, alpha, np.nan_to_num(As[i])[None], beta, ref, nthreads=1)
        want = ref[0, :m, :m].T.astype(np.float64)
        ra, ca = op_rows_cols(trans, m, k)
        opA = np.abs(np.nan_to_num(As[i][:ca, :ra].T.astype(np.float64)))
        opA = opA if trans == "N" else opA.T
        bound = 10 * max(k, 1) * eps(dt) * (opA @ opA.T + np.abs(c0)) + 1e-300
        assert (tri(np.abs(got - want)) <= tri(bound)).all(), (i, m, k)


COMBOS = list(itertools.product("LR", "LU", "NT", "NU"))


def tri_mat(rng, k, uplo, ld, dt):
    """Triangle of order k in the benchmark's recipe (off-diagonal N(0,1)/sqrt(k),
    diagonal U[1,2]); the unused triangle and padding are NaN."""
    a = np.full((max(k, 1), max(ld, 1)), np.nan)
    L = np.tril(rng.standard_normal((k, k)) / np.sqrt(max(k, 1)), -1) + np.diag(rng.uniform(1, 2, k))
    M = L if uplo == "L" else L.T
    mask = np.tril(np.ones((k, k), bool)) if uplo == "L" else np.triu(np.ones((k, k), bool))
    colmaj = np.where(mask, M, np.nan).T           # column-major: a[col, row]
    a[:k, :k] = colmaj
    return a.astype(dt)


def op_dense_1(a, k, uplo, trans, diag):
    A = np.nan_to_num(a[:k, :k].T.astype(np.float64))
    A = np.tril(A) if uplo == "L" else np.triu(A)
    if diag == "U":
        A[np.arange(k), np.arange(k)] = 1.0
    return A.T if trans == "T" else A


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("combo", COMBOS, ids=["".join(c) for c in COMBOS])
def test_trsm_vbatch(gpu, handle, kb, dt, combo):
    side, uplo, trans, diag = combo
    rng = np.random.default_rng(COMBOS.index(combo) * 7 + (dt == np.float32))
    batch = 40
    ms = rng.integers(0, 80, batch)
    ns = rng.integers(0, 80, batch)
    ms[2], ns[5] = 0, 0
    ms[6], ns[6] = 140, 150
    As, Bs, lds = [], [], []
    for i in range(batch):
        k = ms[i] if side == "L" else ns[i]
        lda, ldb = max(k, 1) + rng.integers(0, 3), max(ms[i], 1) + rng.integers(0, 3)
        As.append(tri_mat(rng, k, uplo, lda, dt))
        Bs.append(rand_mat(rng, ms[i], ns[i], ldb, dt))
        lds.append((lda, ldb))
    lds = np.array(lds)
    RA, RB = Ragged(gpu, As, dt), Ragged(gpu, Bs, dt)
    alpha = 1.5
    pfx = "D" if dt == np.float64 else "S"
    # half the combos pass the bounds, half let the library recompute them
    give_max = COMBOS.index(combo) % 2 == 0
    if not give_max:
        kb.lib().kblas_trsm_batch_nonuniform_wsquery(handle.ptr)
        assert handle.allocate_workspace() == 1
    mx = (int(ms.max()), int(ns.max())) if give_max else (0, 0)
    dm, dn, dla, dlb = ivec(gpu, ms), ivec(gpu, ns), ivec(gpu, lds[:, 0]), ivec(gpu, lds[:, 1])
    st = handle.call(f"kblas{pfx}trsm_vbatch", side, uplo, trans, diag, dm.data_ptr(),
                     dn.data_ptr(), *mx, alpha, RA.ptrs.data_ptr(), dla.data_ptr(),
                     RB.ptrs.data_ptr(), dlb.data_ptr(), batch)
    assert st == 1
    gpu.cuda.synchronize()
    outs = RB.get()
    assert RB.gaps_untouched()
    for i in range(batch):
        m, n = int(ms[i]), int(ns[i])
        k = m if side == "L" else n
        assert np.array_equal(outs[i][:, m:], Bs[i][:, m:], equal_nan=True), ("padding", i)
        if m == 0 or n == 0:
            continue
        X = outs[i][:n, :m].T.astype(np.float64)
        B = Bs[i][:n, :m].T.astype(np.float64)
        Aop = op_dense_1(As[i], k, uplo, trans, diag)
        prod = Aop @ X if side == "L" else X @ Aop
        absprod = np.abs(Aop) @ np.abs(X) if side == "L" else np.abs(X) @ np.abs(Aop)
        res = np.abs(prod - alpha * B)
        bound = 10 * k * eps(dt) * (absprod + abs(alpha) * np.abs(B)) + 1e-300
        assert (res <= bound).all(), (i, m, n, (res / bound).max())


def test_trsm_vbatch_needs_workspace_only_without_bounds(gpu, handle):
    m = ivec(gpu, [4])
    # no bounds, no workspace -> KBLAS_InsufficientWorkspace, nothing launched
    assert handle.call("kblasDtrsm_vbatch", "L", "L", "N", "N", m.data_ptr(), m.data_ptr(), 0, 0,
                       1.0, m.data_ptr(), m.data_ptr(), m.data_ptr(), m.data_ptr(), 1) == -6
    # bad flag
    assert handle.call("kblasDtrsm_vbatch", "X", "L", "N", "N", m.data_ptr(), m.data_ptr(), 4, 4,
                       1.0, m.data_ptr(), m.data_ptr(), m.data_ptr(), m.data_ptr(), 1) == -10
