"""Generate the LAPACK/BLAS golden fixtures that pin the CPU oracle.

The reference's batch tests judge every routine against host LAPACK/BLAS
looped over the batch (testing/batch_triangular/test_Xpotrf_batch.cpp:317-338,
test_Xposv_batch.cpp:313-338, test_Xtrsm_batch.cpp:330-360,
test_Xtrmm_batch.cpp:346-354, test_Xsyrk_batch.cpp:405-417) and ship no golden
vectors of their own. This script records what LAPACK/BLAS (scipy's bundled
OpenBLAS: dpotrf/spotrf, dpotrs, dtrsm/strsm, dtrmm/strmm, dsyrk/ssyrk,
dgemm/sgemm, and the xTRTRI / xLAUUM / xPOTRI inversion routines)
returns on small seeded inputs, including non-SPD matrices with a known
failing leading minor, so tests/test_oracle.py can check the C oracle against
it on any machine (scipy is not needed at test time).

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
from scipy.linalg import blas, lapack

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))


def rng(seed, stream):
    return np.random.Generator(np.random.Philox(key=seed, counter=[0, 0, 0, stream]))


def spd(n, r):
    g = r.standard_normal((n, n))
    return g @ g.T + n * np.eye(n)


def lowtri(n, r):
    a = np.tril(r.standard_normal((n, n)) / np.sqrt(n), -1)
    return a + np.diag(r.uniform(1.0, 2.0, n))


def main():
    out = {}
    r = rng(2024, 0)
    sizes = [1, 2, 3, 7, 8, 9, 15, 16, 17, 31, 32, 33, 47, 63, 64, 65, 97]
    for dt, name in ((np.float64, "d"), (np.float32, "s")):
        potrf, potrs = (lapack.dpotrf, lapack.dpotrs) if name == "d" else (lapack.spotrf, lapack.spotrs)
        trsm, trmm, syrk = ((blas.dtrsm, blas.dtrmm, blas.dsyrk) if name == "d"
                            else (blas.strsm, blas.strmm, blas.ssyrk))
        for n in sizes:
            a = spd(n, r).astype(dt)
            c, info = potrf(a, lower=1, clean=1)
            out[f"{name}potrf_n{n}_A"] = a
            out[f"{name}potrf_n{n}_L"] = np.tril(c)
            out[f"{name}potrf_n{n}_info"] = np.int32(info)
            for m in (1, 4):
                b = r.standard_normal((m, n)).astype(dt)  # rows = right-hand sides
                x, info2 = potrs(c, b.T.copy(), lower=1)
                out[f"{name}posv_n{n}_m{m}_B"] = b
                out[f"{name}posv_n{n}_m{m}_X"] = x.T.copy()
        # non-SPD with a known failing leading minor k (1-based)
        for n, k in ((1, 1), (5, 3), (8, 8), (16, 1), (17, 9), (32, 20), (33, 33), (64, 40),
                     (97, 77)):
            a = spd(n, r)
            # pivot k of the untouched matrix, then push it to -1
            piv = a[k - 1, k - 1]
            if k > 1:
                l11 = np.linalg.cholesky(a[: k - 1, : k - 1])
                w = np.linalg.solve(l11, a[: k - 1, k - 1])
                piv = a[k - 1, k - 1] - w @ w
            a[k - 1, k - 1] -= piv + 1.0
            a = a.astype(dt)
            c, info = potrf(a, lower=1, clean=0)
            assert info == k, (n, k, info)
            out[f"{name}nonspd_n{n}_A"] = a
            out[f"{name}nonspd_n{n}_info"] = np.int32(info)
        # TRSM / TRMM all flag combinations on small shapes
        for (m, n) in ((5, 3), (16, 16), (33, 7), (40, 24), (3, 40)):
            for side in "LR":
                ka = m if side == "L" else n
                for uplo in "LU":
                    for trans in "NT":
                        for diag in "NU":
                            a = lowtri(ka, r)
                            if uplo == "U":
                                a = a.T.copy()
                            b = r.standard_normal((m, n))
                            alpha = 1.5
                            kw = dict(side=int(side == "R"), lower=int(uplo == "L"),
                                      trans_a=int(trans == "T"), diag=int(diag == "U"))
                            xs = trsm(alpha, a.astype(dt), b.astype(dt), **kw)
                            xm = trmm(alpha, a.astype(dt), b.astype(dt), **kw)
                            key = f"{name}tr_{side}{uplo}{trans}{diag}_m{m}_n{n}"
                            out[key + "_A"] = a.astype(dt)
                            out[key + "_B"] = b.astype(dt)
                            out[key + "_trsm"] = xs
                            out[key + "_trmm"] = xm
        # SYRK lower, both transposes
        for (m, k) in ((1, 1), (5, 3), (16, 16), (33, 17), (48, 40), (70, 9)):
            for trans in "NT":
                a = r.standard_normal((m, k) if trans == "N" else (k, m))
                c0 = spd(m, r)
                res = syrk(-1.0, a.astype(dt), beta=1.0, c=c0.astype(dt),
                           trans=int(trans == "T"), lower=1)
                key = f"{name}syrk_{trans}_m{m}_k{k}"
                out[key + "_A"] = a.astype(dt)
                out[key + "_C"] = c0.astype(dt)
                out[key + "_R"] = np.tril(res)
    # inversion routines (own stream, so the arrays above do not change):
    # xTRTRI / xLAUUM / xPOTRI on a Cholesky factor, and a singular TRTRI
    r2 = rng(2025, 1)
    for dt, name in ((np.float64, "d"), (np.float32, "s")):
        potrf = lapack.dpotrf if name == "d" else lapack.spotrf
        trtri, lauum, potri = ((lapack.dtrtri, lapack.dlauum, lapack.dpotri) if name == "d"
                               else (lapack.strtri, lapack.slauum, lapack.spotri))
        for n in (1, 2, 7, 16, 31, 33, 64, 97):
            a = spd(n, r2).astype(dt)
            c, info = potrf(a, lower=1, clean=1)
            assert info == 0
            x, info = trtri(c, lower=1, unitdiag=0)
            assert info == 0
            u, info = lauum(c, lower=1)
            assert info == 0
            pinv, info = potri(c, lower=1)
            assert info == 0
            key = f"{name}inv_n{n}"
            out[key + "_A"] = a
            out[key + "_L"] = np.tril(c)
            out[key + "_trtri"] = np.tril(x)
            out[key + "_lauum"] = np.tril(u)
            out[key + "_potri"] = np.tril(pinv)
        for n, k in ((1, 1), (9, 4), (40, 40)):
            c = np.tril(lowtri(n, r2)).astype(dt)
            c[k - 1, k - 1] = 0
            x, info = trtri(c, lower=1, unitdiag=0)
            assert info == k, (n, k, info)
            out[f"{name}trtri_sing_n{n}_L"] = c
            out[f"{name}trtri_sing_n{n}_info"] = np.int32(info)
    # GEMM (every transA / transB, alpha, beta incl. 0) and upper SYRK, on a
    # third stream so the arrays above do not change
    r3 = rng(2026, 2)
    for dt, name in ((np.float64, "d"), (np.float32, "s")):
        gemm, syrk = (blas.dgemm, blas.dsyrk) if name == "d" else (blas.sgemm, blas.ssyrk)
        for (m, n, k) in ((1, 1, 1), (5, 7, 3), (16, 16, 16), (33, 17, 40), (64, 9, 70), (3, 50, 0)):
            for ta in "NT":
                for tb in "NT":
                    a = r3.standard_normal((m, k) if ta == "N" else (k, m))
                    b = r3.standard_normal((k, n) if tb == "N" else (n, k))
                    c0 = r3.standard_normal((m, n))
                    alpha, beta = (1.5, -0.5) if (m + n) % 2 else (-1.0, 0.0)
                    res = gemm(alpha, a.astype(dt), b.astype(dt), beta=beta, c=c0.astype(dt),
                               trans_a=int(ta == "T"), trans_b=int(tb == "T"))
                    key = f"{name}gemm_{ta}{tb}_m{m}_n{n}_k{k}"
                    out[key + "_A"] = a.astype(dt)
                    out[key + "_B"] = b.astype(dt)
                    out[key + "_C"] = c0.astype(dt)
                    out[key + "_ab"] = np.array([alpha, beta])
                    out[key + "_R"] = res
        for (m, k) in ((5, 3), (33, 17), (48, 40)):
            for trans in "NT":
                a = r3.standard_normal((m, k) if trans == "N" else (k, m))
                c0 = spd(m, r3)
                res = syrk(-1.0, a.astype(dt), beta=1.0, c=c0.astype(dt),
                           trans=int(trans == "T"), lower=0)
                key = f"{name}syrku_{trans}_m{m}_k{k}"
                out[key + "_A"] = a.astype(dt)
                out[key + "_C"] = c0.astype(dt)
                out[key + "_R"] = np.triu(res)
    # Upper-triangle xPOTRF and side-L xPOTRS for both triangles (LAPACK's own
    # side), on a fourth stream
    r4 = rng(2027, 3)
    for dt, name in ((np.float64, "d"), (np.float32, "s")):
        potrf, potrs = (lapack.dpotrf, lapack.dpotrs) if name == "d" else (lapack.spotrf, lapack.spotrs)
        for n in (1, 3, 16, 33, 64, 97):
            a = spd(n, r4).astype(dt)
            b = r4.standard_normal((n, 3)).astype(dt)
            for uplo in "LU":
                c, info = potrf(a, lower=int(uplo == "L"), clean=1)
                assert info == 0
                x, info = potrs(c, b, lower=int(uplo == "L"))
                assert info == 0
                key = f"{name}potrf{uplo.lower()}_n{n}"
                out[key + "_A"] = a
                out[key + "_F"] = c
                out[key + "_B"] = b
                out[key + "_X"] = x
        a = spd(40, r4)
        a[17, 17] = -1.0
        c, info = lapack.dpotrf(a, lower=0, clean=0)
        out["dpotrfu_bad_n40_A"] = a
        out["dpotrfu_bad_n40_info"] = np.int32(info)
    # complex BLAS (no conjugation: op = transpose, SYRK = A A^T), the forms
    # the reference's C / Z batch routines compute; a fifth stream
    r5 = rng(2028, 4)
    for dt, name in ((np.complex128, "z"), (np.complex64, "c")):
        gemm, syrk, trsm, trmm = (getattr(blas, name + f) for f in ("gemm", "syrk", "trsm", "trmm"))

        def cn(*shape):
            return (r5.standard_normal(shape) + 1j * r5.standard_normal(shape)).astype(dt)
        for (m, n, k) in ((5, 7, 3), (33, 17, 40)):
            for ta in "NT":
                for tb in "NT":
                    a = cn(*((m, k) if ta == "N" else (k, m)))
                    b = cn(*((k, n) if tb == "N" else (n, k)))
                    c0 = cn(m, n)
                    res = gemm(1.5 - 0.5j, a, b, beta=0.25 + 1j, c=c0, trans_a=int(ta == "T"),
                               trans_b=int(tb == "T"))
                    key = f"{name}gemm_{ta}{tb}_m{m}_n{n}_k{k}"
                    out.update({key + "_A": a, key + "_B": b, key + "_C": c0, key + "_R": res})
        for (m, k) in ((6, 4), (40, 23)):
            for trans in "NT":
                a = cn(*((m, k) if trans == "N" else (k, m)))
                c0 = cn(m, m)
                c0 = np.tril(c0) + np.tril(c0, -1).T
                res = syrk(-1.0, a, beta=1.0, c=c0, trans=int(trans == "T"), lower=1)
                key = f"{name}syrk_{trans}_m{m}_k{k}"
                out.update({key + "_A": a, key + "_C": c0, key + "_R": np.tril(res)})
        for (m, n) in ((9, 4), (33, 12)):
            L = np.tril(cn(m, m)) / np.sqrt(m) + np.diag(r5.uniform(1, 2, m) + 0.5j)
            L = L.astype(dt)
            b = cn(m, n)
            for trans in "NT":
                key = f"{name}tri_{trans}_m{m}_n{n}"
                out[key + "_L"] = L
                out[key + "_B"] = b
                out[key + "_trsm"] = trsm(0.5 + 0.5j, L, b, lower=1, trans_a=int(trans == "T"))
                out[key + "_trmm"] = trmm(0.5 + 0.5j, L, b, lower=1, trans_a=int(trans == "T"))
    path = os.path.join(HERE, "lapack_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, len(out), "arrays", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
