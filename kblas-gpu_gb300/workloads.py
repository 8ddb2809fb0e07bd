"""Seeded synthetic inputs for the batched Cholesky / triangular workloads.

Every generator is deterministic in ``seed`` (numpy ``Philox`` bit generator,
one stream per workload) and returns batches in the layout used by the host
bindings: a numpy array of shape ``(batch, ncols, ld)`` in C order, i.e.
element (i, j) of matrix ``b`` is ``arr[b, j, i]`` -- column-major matrices
with leading dimension ``ld`` and stride ``ld * ncols``.

Workloads (matrix recipes of the benchmark configurations):
  * ``spd_shifted``   A = G G^T + n I, G i.i.d. N(0, 1)   (POTRF/POSV n = 32,
    variable-size POSV n in [8, 256])
  * ``lower_tri``     off-diagonal N(0, 1)/sqrt(n), diagonal U[1, 2]
    (TRSM/TRMM 64 x 64)
  * ``spd_cond``      Q diag(lambda) Q^T, lambda geometric, cond log-uniform
    in [1e2, 1e8] (mixed-precision POSV n = 64)
  * ``sqexp_cov``     squared-exponential covariance on points in the unit
    square, length scale U[0.05, 0.3], nugget 1e-4 (n = 512)
  * ``indefinite``    one eigenvalue of an spd_shifted matrix flipped in sign
"""
from __future__ import annotations

import numpy as np


def rng(seed: int, stream: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=seed, counter=[0, 0, 0, stream]))


def spd_shifted(batch: int, n: int, seed: int = 0, ld: int | None = None,
                dtype=np.float64) -> np.ndarray:
    """A = G G^T + n I with G ~ N(0,1), column-major (batch, n, ld)."""
    ld = ld or n
    g = rng(seed, 1).standard_normal((batch, n, n))
    a = np.einsum("bij,bkj->bik", g, g) + n * np.eye(n)[None]
    out = np.zeros((batch, n, ld), dtype=dtype)
    out[:, :, :n] = a.transpose(0, 2, 1)
    return out


def rhs_rows(batch: int, m: int, n: int, seed: int = 0, ld: int | None = None,
             dtype=np.float64, stream: int = 2) -> np.ndarray:
    """m right-hand sides as rows of an m x n matrix B (side 'R' layout)."""
    ld = ld or m
    b = rng(seed, stream).standard_normal((batch, n, m))
    out = np.zeros((batch, n, ld), dtype=dtype)
    out[:, :, :m] = b
    return out


def general(batch: int, rows: int, cols: int, seed: int = 0, ld: int | None = None,
            dtype=np.float64, stream: int = 3) -> np.ndarray:
    ld = ld or rows
    x = rng(seed, stream).standard_normal((batch, cols, rows))
    out = np.zeros((batch, cols, ld), dtype=dtype)
    out[:, :, :rows] = x
    return out


def lower_tri(batch: int, n: int, seed: int = 0, ld: int | None = None, dtype=np.float64,
              upper_fill: float = np.nan) -> np.ndarray:
    """Lower triangular: off-diagonal N(0,1)/sqrt(n), diagonal U[1,2]; the strict
    upper triangle holds ``upper_fill`` (NaN by default, so a kernel that
    reads it is caught)."""
    ld = ld or n
    r = rng(seed, 4)
    a = r.standard_normal((batch, n, n)) / np.sqrt(n)
    a = np.tril(a, -1) + np.eye(n)[None] * r.uniform(1.0, 2.0, (batch, 1, n))
    a = a + np.triu(np.full((n, n), upper_fill), 1)[None]
    out = np.zeros((batch, n, ld), dtype=dtype)
    out[:, :, :n] = a.transpose(0, 2, 1)
    return out


def spd_cond(batch: int, n: int, seed: int = 0, logc=(2.0, 8.0), dtype=np.float64,
             ld: int | None = None) -> tuple[np.ndarray, np.ndarray]:
    """A = Q diag(lambda) Q^T, Q from the QR of a Gaussian matrix, lambda
    geometrically spaced in [1, cond] with log10(cond) ~ U[logc]. Returns
    (A, cond)."""
    ld = ld or n
    r = rng(seed, 5)
    q, _ = np.linalg.qr(r.standard_normal((batch, n, n)))
    cond = 10.0 ** r.uniform(logc[0], logc[1], batch)
    t = np.linspace(0.0, 1.0, n)
    lam = cond[:, None] ** (-t[None, :])  # from 1 down to 1/cond
    a = np.einsum("bij,bj,bkj->bik", q, lam, q)
    a = 0.5 * (a + a.transpose(0, 2, 1))
    out = np.zeros((batch, n, ld), dtype=dtype)
    out[:, :, :n] = a.transpose(0, 2, 1)
    return out, cond


def sqexp_cov(batch: int, n: int, seed: int = 0, nugget: float = 1e-4, dtype=np.float64,
              ld: int | None = None) -> np.ndarray:
    ld = ld or n
    r = rng(seed, 6)
    x = r.uniform(0.0, 1.0, (batch, n, 2))
    ell = r.uniform(0.05, 0.3, batch)
    d2 = ((x[:, :, None, :] - x[:, None, :, :]) ** 2).sum(-1)
    a = np.exp(-d2 / (2.0 * ell[:, None, None] ** 2)) + nugget * np.eye(n)[None]
    out = np.zeros((batch, n, ld), dtype=dtype)
    out[:, :, :n] = a.transpose(0, 2, 1)
    return out


def flip_one_eigenvalue(a_colmajor: np.ndarray, n: int, seed: int) -> np.ndarray:
    """A <- A - 2 lambda_k v_k v_k^T for a random k (one negative eigenvalue)."""
    a = a_colmajor[:n, :n].T.copy()
    w, v = np.linalg.eigh(a)
    k = int(rng(seed, 7).integers(0, n))
    a = a - 2.0 * w[k] * np.outer(v[:, k], v[:, k])
    a = 0.5 * (a + a.T)
    out = a_colmajor.copy()
    out[:n, :n] = a.T
    return out


def vbatch_sizes(batch: int, nmin: int = 8, nmax: int = 256, seed: int = 0) -> np.ndarray:
    """n = floor(exp(U[ln nmin, ln(nmax+1)))) -- integer, log-uniform."""
    u = rng(seed, 8).uniform(np.log(nmin), np.log(nmax + 1), batch)
    return np.clip(np.floor(np.exp(u)).astype(np.int32), nmin, nmax)
