"""CPU oracle for the batched Cholesky / triangular path -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module: it is the checker and the timed CPU
baseline, never part of the product path.

It wraps ``liboracle.so`` (built from ``kblas_oracle.c`` / ``oracle_impl.h``,
a C restatement of the LAPACK/BLAS routines the reference tests check
against) with numpy-friendly helpers, plus the seeded input generators used
by tests and the benchmark.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc -O2 -fopenmp (portable flags only)."""
    srcs = [os.path.join(_HERE, "kblas_oracle.c"), os.path.join(_HERE, "oracle_impl.h")]
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= t for s in srcs):
            return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", tmp,
           os.path.join(_HERE, "kblas_oracle.c"), "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            P = C.c_void_p
            I, Lg, D, F, Ch = C.c_int, C.c_long, C.c_double, C.c_float, C.c_char
            for pfx, R in (("d", D), ("s", F), ("z", _Z), ("c", _CF)):
                getattr(L, f"oracle_{pfx}potrf").argtypes = [I, P, I]
                getattr(L, f"oracle_{pfx}potrf").restype = I
                getattr(L, f"oracle_{pfx}potrs").argtypes = [I, I, P, I, P, I]
                getattr(L, f"oracle_{pfx}posv").argtypes = [I, I, P, I, P, I]
                getattr(L, f"oracle_{pfx}posv").restype = I
                getattr(L, f"oracle_{pfx}trsm").argtypes = [Ch, Ch, Ch, Ch, I, I, R, P, I, P, I]
                getattr(L, f"oracle_{pfx}trmm").argtypes = [Ch, Ch, Ch, Ch, I, I, R, P, I, P, I]
                getattr(L, f"oracle_{pfx}syrk").argtypes = [Ch, Ch, I, I, R, P, I, R, P, I]
                getattr(L, f"oracle_{pfx}potrf_batch").argtypes = [I, P, I, Lg, I, P, I]
                getattr(L, f"oracle_{pfx}potrs_batch").argtypes = [I, I, P, I, Lg, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}posv_batch").argtypes = [I, I, P, I, Lg, P, I, Lg, I, P, I]
                getattr(L, f"oracle_{pfx}trsm_batch").argtypes = [Ch, Ch, Ch, Ch, I, I, R, P, I, Lg, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}trmm_batch").argtypes = [Ch, Ch, Ch, Ch, I, I, R, P, I, Lg, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}syrk_batch").argtypes = [Ch, Ch, I, I, R, P, I, Lg, R, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}gemm").argtypes = [Ch, Ch, I, I, I, R, P, I, P, I, R, P, I]
                getattr(L, f"oracle_{pfx}gemm_batch").argtypes = [Ch, Ch, I, I, I, R, P, I, Lg, P, I, Lg,
                                                                  R, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}posv_vbatch").argtypes = [P, P, P, P, P, P, I, P, I]
                getattr(L, f"oracle_{pfx}trtri_batch").argtypes = [I, I, P, I, Lg, I, P, I]
                getattr(L, f"oracle_{pfx}lauum_batch").argtypes = [I, P, I, Lg, I, I]
                getattr(L, f"oracle_{pfx}potri_batch").argtypes = [I, P, I, Lg, I, P, I]
                getattr(L, f"oracle_{pfx}poti_batch").argtypes = [I, P, I, Lg, I, P, I]
            L.oracle_backward_error_r.argtypes = [I, I, P, I, P, I, P, I]
            L.oracle_backward_error_r.restype = D
            L.oracle_backward_error_r_batch.argtypes = [I, I, P, I, Lg, P, I, Lg, P, I, Lg, I, P, I]
            L.oracle_backward_error_r_vbatch.argtypes = [P, P, P, P, P, P, P, P, I, P, I]
            L.oracle_factor_backward_error.argtypes = [I, P, I, P, I]
            L.oracle_factor_backward_error.restype = D
            L.oracle_lower_rel_diff.argtypes = [I, P, I, P, I]
            L.oracle_lower_rel_diff.restype = D
            L.oracle_max_threads.restype = I
            _lib = L
    return _lib


class _Z(C.Structure):
    """double _Complex passed by value (same ABI class as two doubles)."""
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class _CF(C.Structure):
    """float _Complex passed by value."""
    _fields_ = [("re", C.c_float), ("im", C.c_float)]


def _scal(a: np.ndarray, v):
    """A scalar argument (alpha / beta) in the type of the array's routines."""
    if a.dtype == np.complex128:
        v = complex(v)
        return _Z(v.real, v.imag)
    if a.dtype == np.complex64:
        v = complex(v)
        return _CF(v.real, v.imag)
    return v


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _pfx(a: np.ndarray) -> str:
    if a.dtype == np.float64:
        return "d"
    if a.dtype == np.float32:
        return "s"
    if a.dtype == np.complex128:
        return "z"
    if a.dtype == np.complex64:
        return "c"
    raise TypeError(a.dtype)


def _b(c: str) -> bytes:
    return c.encode()


def nthreads_default() -> int:
    return max(1, os.cpu_count() or 1)


# --------------------------------------------------------------------------
# Batched storage convention used throughout tests/bench: a batch of
# column-major matrices is a numpy array of shape (batch, ncols, ld) in C
# order, i.e. element (i, j) of matrix b is arr[b, j, i]; strideA = ld*ncols.
# --------------------------------------------------------------------------

def potrf_batch(A: np.ndarray, n: int, nthreads: int | None = None):
    """In-place lower Cholesky of A[b, :, :] (shape (batch, n, lda)); returns info."""
    assert A.flags.c_contiguous
    batch, ncol, lda = A.shape
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"oracle_{_pfx(A)}potrf_batch")(n, _p(A), lda, ncol * lda, batch, _p(info),
                                                   nthreads or nthreads_default())
    return info


def potrs_batch(L: np.ndarray, B: np.ndarray, m: int, n: int, nthreads: int | None = None):
    batch, ncol, lda = L.shape
    _, ncolb, ldb = B.shape
    getattr(lib(), f"oracle_{_pfx(L)}potrs_batch")(m, n, _p(L), lda, ncol * lda, _p(B), ldb,
                                                   ncolb * ldb, batch, nthreads or nthreads_default())


def posv_batch(A: np.ndarray, B: np.ndarray, m: int, n: int, nthreads: int | None = None):
    batch, ncol, lda = A.shape
    _, ncolb, ldb = B.shape
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"oracle_{_pfx(A)}posv_batch")(m, n, _p(A), lda, ncol * lda, _p(B), ldb,
                                                  ncolb * ldb, batch, _p(info),
                                                  nthreads or nthreads_default())
    return info


def trsm_batch(side, uplo, trans, diag, m, n, alpha, A, B, nthreads=None):
    batch, ncol, lda = A.shape
    _, ncolb, ldb = B.shape
    getattr(lib(), f"oracle_{_pfx(A)}trsm_batch")(_b(side), _b(uplo), _b(trans), _b(diag), m, n,
                                                  _scal(A, alpha), _p(A), lda, ncol * lda, _p(B), ldb,
                                                  ncolb * ldb, batch, nthreads or nthreads_default())


def trmm_batch(side, uplo, trans, diag, m, n, alpha, A, B, nthreads=None):
    batch, ncol, lda = A.shape
    _, ncolb, ldb = B.shape
    getattr(lib(), f"oracle_{_pfx(A)}trmm_batch")(_b(side), _b(uplo), _b(trans), _b(diag), m, n,
                                                  _scal(A, alpha), _p(A), lda, ncol * lda, _p(B), ldb,
                                                  ncolb * ldb, batch, nthreads or nthreads_default())


def syrk_batch(uplo, trans, m, k, alpha, A, beta, Cm, nthreads=None):
    batch, ncol, lda = A.shape
    _, ncolc, ldc = Cm.shape
    getattr(lib(), f"oracle_{_pfx(A)}syrk_batch")(_b(uplo), _b(trans), m, k, _scal(A, alpha), _p(A),
                                                  lda, ncol * lda, _scal(A, beta), _p(Cm), ldc,
                                                  ncolc * ldc,
                                                  batch, nthreads or nthreads_default())


def gemm_batch(transA, transB, m, n, k, alpha, A, B, beta, Cm, nthreads=None):
    """C := alpha op(A) op(B) + beta C over a (batch, ncol, ld) column-major stack."""
    batch, ncol, lda = A.shape
    _, ncolb, ldb = B.shape
    _, ncolc, ldc = Cm.shape
    getattr(lib(), f"oracle_{_pfx(A)}gemm_batch")(_b(transA), _b(transB), m, n, k, _scal(A, alpha),
                                                  _p(A), lda, ncol * lda, _p(B), ldb, ncolb * ldb,
                                                  _scal(A, beta),
                                                  _p(Cm), ldc, ncolc * ldc, batch,
                                                  nthreads or nthreads_default())


def _swap_uplo(A: np.ndarray, n: int):
    """Transpose the leading n x n block of every matrix in place."""
    A[:, :n, :n] = A[:, :n, :n].transpose(0, 2, 1).copy()


def potrf_batch_uplo(A: np.ndarray, n: int, uplo: str, nthreads=None):
    """xPOTRF for either triangle (only that triangle referenced, LAPACK): the
    upper factor U of A = U^T U is the transpose of the lower factor of A^T,
    so uplo 'U' runs the lower restatement between two transposes."""
    if uplo == "L":
        return potrf_batch(A, n, nthreads)
    _swap_uplo(A, n)
    info = potrf_batch(A, n, nthreads)
    _swap_uplo(A, n)
    return info


_POTRS_SEQ = {("R", "L"): ("T", "N"), ("R", "U"): ("N", "T"),
              ("L", "L"): ("N", "T"), ("L", "U"): ("T", "N")}


def potrs_batch_side(side: str, uplo: str, m: int, n: int, F: np.ndarray, B: np.ndarray,
                     nthreads=None):
    """xPOTRS with the factor F of either triangle, for A X = B (side 'L', A
    m x m, LAPACK xPOTRS: two triangular solves, dpotrs.f) or X A = B (side
    'R', A n x n); B is m x n. The two TRSM passes:
      R,L: B L^-T then L^-1   R,U: B U^-1 then U^-T
      L,L: L^-1 B then L^-T   L,U: U^-T B then U^-1"""
    t1, t2 = _POTRS_SEQ[(side, uplo)]
    trsm_batch(side, uplo, t1, "N", m, n, 1.0, F, B, nthreads)
    trsm_batch(side, uplo, t2, "N", m, n, 1.0, F, B, nthreads)


def posv_batch_side(side: str, uplo: str, m: int, n: int, A: np.ndarray, B: np.ndarray,
                    nthreads=None):
    """xPOSV for every side / uplo: factor, then solve the systems whose info
    is 0 (the others keep B, LAPACK)."""
    order = m if side == "L" else n
    info = potrf_batch_uplo(A, order, uplo, nthreads)
    ok = np.where(info == 0)[0]
    if len(ok):
        Fa, Bb = np.ascontiguousarray(A[ok]), np.ascontiguousarray(B[ok])
        potrs_batch_side(side, uplo, m, n, Fa, Bb, nthreads)
        B[ok] = Bb
    return info


def backward_error_r(A: np.ndarray, X: np.ndarray, B: np.ndarray, m: int, n: int,
                     nthreads: int | None = None) -> np.ndarray:
    """Per-system normwise backward error of X*A = B (A symmetric, lower)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    batch, ncol, lda = A.shape
    _, ncx, ldx = X.shape
    _, ncb, ldb = B.shape
    eta = np.zeros(batch, dtype=np.float64)
    lib().oracle_backward_error_r_batch(m, n, _p(A), lda, ncol * lda, _p(X), ldx, ncx * ldx,
                                        _p(B), ldb, ncb * ldb, batch, _p(eta),
                                        nthreads or nthreads_default())
    return eta


def factor_backward_error(A2d: np.ndarray, L2d: np.ndarray, n: int) -> float:
    """||A - L L^T||_max / ||A||_max; arguments are (n, ld) arrays in C order
    holding one column-major matrix."""
    A2d = np.ascontiguousarray(A2d, dtype=np.float64)
    L2d = np.ascontiguousarray(L2d, dtype=np.float64)
    return lib().oracle_factor_backward_error(n, _p(A2d), A2d.shape[1], _p(L2d), L2d.shape[1])


def lower_rel_diff(L1: np.ndarray, L2: np.ndarray, n: int) -> float:
    L1 = np.ascontiguousarray(L1, dtype=np.float64)
    L2 = np.ascontiguousarray(L2, dtype=np.float64)
    return lib().oracle_lower_rel_diff(n, _p(L1), L1.shape[1], _p(L2), L2.shape[1])


def trtri_batch(A: np.ndarray, n: int, unit: bool = False, nthreads=None):
    """In-place inverse of the lower triangles of A[b] (LAPACK xTRTRI, lower);
    returns info (first zero diagonal, 1-based; A[b] unchanged then)."""
    assert A.flags.c_contiguous
    batch, ncol, lda = A.shape
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"oracle_{_pfx(A)}trtri_batch")(int(unit), n, _p(A), lda, ncol * lda, batch,
                                                   _p(info), nthreads or nthreads_default())
    return info


def lauum_batch(A: np.ndarray, n: int, nthreads=None):
    """In place: lower triangle of L^T L over L (LAPACK xLAUUM, lower)."""
    assert A.flags.c_contiguous
    batch, ncol, lda = A.shape
    getattr(lib(), f"oracle_{_pfx(A)}lauum_batch")(n, _p(A), lda, ncol * lda, batch,
                                                   nthreads or nthreads_default())


def potri_batch(A: np.ndarray, n: int, nthreads=None):
    """In place: lower triangle of A^{-1} from the Cholesky factor in A; info."""
    assert A.flags.c_contiguous
    batch, ncol, lda = A.shape
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"oracle_{_pfx(A)}potri_batch")(n, _p(A), lda, ncol * lda, batch, _p(info),
                                                   nthreads or nthreads_default())
    return info


def poti_batch(A: np.ndarray, n: int, nthreads=None):
    """In place: lower triangle of A^{-1} for SPD A (POTRF + POTRI); info."""
    assert A.flags.c_contiguous
    batch, ncol, lda = A.shape
    info = np.zeros(batch, dtype=np.int32)
    getattr(lib(), f"oracle_{_pfx(A)}poti_batch")(n, _p(A), lda, ncol * lda, batch, _p(info),
                                                  nthreads or nthreads_default())
    return info


def posv_vbatch(ms, ns, As, ldas, Bs, ldbs, nthreads=None):
    """Variable-size POSV over lists of numpy arrays (each (ncol, ld) C order)."""
    batch = len(ns)
    m = np.asarray(ms, dtype=np.int32)
    n = np.asarray(ns, dtype=np.int32)
    lda = np.asarray(ldas, dtype=np.int32)
    ldb = np.asarray(ldbs, dtype=np.int32)
    pa = np.array([a.ctypes.data for a in As], dtype=np.uint64)
    pb = np.array([b.ctypes.data for b in Bs], dtype=np.uint64)
    info = np.zeros(batch, dtype=np.int32)
    lib().oracle_dposv_vbatch(_p(m), _p(n), _p(pa), _p(lda), _p(pb), _p(ldb), batch, _p(info),
                              nthreads or nthreads_default())
    return info


def backward_error_r_vbatch(ms, ns, As, ldas, Xs, ldxs, Bs, ldbs, nthreads=None):
    batch = len(ns)
    m = np.asarray(ms, dtype=np.int32)
    n = np.asarray(ns, dtype=np.int32)
    lda = np.asarray(ldas, dtype=np.int32)
    ldx = np.asarray(ldxs, dtype=np.int32)
    ldb = np.asarray(ldbs, dtype=np.int32)
    pa = np.array([a.ctypes.data for a in As], dtype=np.uint64)
    px = np.array([x.ctypes.data for x in Xs], dtype=np.uint64)
    pb = np.array([b.ctypes.data for b in Bs], dtype=np.uint64)
    eta = np.zeros(batch, dtype=np.float64)
    lib().oracle_backward_error_r_vbatch(_p(m), _p(n), _p(pa), _p(lda), _p(px), _p(ldx), _p(pb),
                                         _p(ldb), batch, _p(eta), nthreads or nthreads_default())
    return eta


# --------------------------------------------------------------------------
# the host's optimized LAPACK (for the timed CPU baseline)
# --------------------------------------------------------------------------

_lapack = None


def _single_thread_openblas():
    """Pin the OpenBLAS that scipy loaded to one thread (the batch loop is the
    parallel level, as in the reference testers). Returns what was done."""
    import re
    try:
        maps = open("/proc/self/maps").read()
    except OSError:
        return "unknown"
    for path in sorted(set(re.findall(r"/\S*scipy\S*openblas\S*\.so\S*", maps))):
        try:
            L = C.CDLL(path)
        except OSError:
            continue
        for sym in ("scipy_openblas_set_num_threads", "openblas_set_num_threads"):
            f = getattr(L, sym, None)
            if f is not None:
                f.argtypes = [C.c_int]
                f(1)
                return "OpenBLAS pinned to 1 thread (%s)" % sym
    return "OpenBLAS threads not found"


def host_lapack():
    """(dpotrf, dpotrs, description) of the host LAPACK that scipy links, as
    raw function addresses, or None when scipy's LAPACK is not importable."""
    global _lapack
    with _lock:
        if _lapack is None:
            os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")  # if scipy is not loaded yet
            try:
                import scipy
                from scipy.linalg import cython_lapack
                api = C.pythonapi
                api.PyCapsule_GetName.restype = C.c_char_p
                api.PyCapsule_GetName.argtypes = [C.py_object]
                api.PyCapsule_GetPointer.restype = C.c_void_p
                api.PyCapsule_GetPointer.argtypes = [C.py_object, C.c_char_p]
                ptrs = []
                for name in ("dpotrf", "dpotrs"):
                    cap = cython_lapack.__pyx_capi__[name]
                    ptrs.append(api.PyCapsule_GetPointer(cap, api.PyCapsule_GetName(cap)))
                if not all(ptrs):
                    raise RuntimeError("null LAPACK entry point")
                how = _single_thread_openblas()
            except Exception:
                _lapack = False
                return None
            _lapack = (ptrs[0], ptrs[1], "LAPACK dpotrf + dpotrs of scipy %s (%s)" % (scipy.__version__, how))
    return _lapack or None


def lapack_posv_batch(A: np.ndarray, B: np.ndarray, nthreads=None):
    """The host LAPACK's dpotrf + dpotrs over a uniform batch: A (batch, n, n)
    column-major matrices (array [b, j, i] = a_ij), B (batch, nrhs, n), i.e.
    each system's right-hand sides as n x nrhs column-major (LAPACK's layout).
    OpenMP over the batch. Returns info, or None without a host LAPACK."""
    lp = host_lapack()
    if lp is None:
        return None
    L = lib()
    f = L.oracle_lapack_dposv_vbatch
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                  C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int]
    f.restype = None
    assert A.flags.c_contiguous and B.flags.c_contiguous and A.dtype == np.float64
    batch, n = A.shape[0], A.shape[-1]
    nrhs = B.shape[1]
    nn = np.full(batch, n, dtype=np.int32)
    pa = (A.ctypes.data + np.arange(batch, dtype=np.uint64) * np.uint64(A[0].nbytes)).astype(np.uint64)
    pb = (B.ctypes.data + np.arange(batch, dtype=np.uint64) * np.uint64(B[0].nbytes)).astype(np.uint64)
    info = np.zeros(batch, dtype=np.int32)
    f(lp[0], lp[1], _p(nn), nrhs, _p(pa), _p(nn), _p(pb), _p(nn), batch, _p(info),
      nthreads or nthreads_default())
    return info


def lapack_posv1_vbatch(ns, As, ldas, Bs, nthreads=None):
    """The host LAPACK's dpotrf + dpotrs over a variable-size batch (one
    right-hand side per system, Bs[b] holding n contiguous values), OpenMP
    over the batch. Returns info, or None when no host LAPACK is available."""
    lp = host_lapack()
    if lp is None:
        return None
    L = lib()
    f = L.oracle_lapack_dposv1_vbatch
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                  C.c_void_p, C.c_int]
    f.restype = None
    batch = len(ns)
    n = np.asarray(ns, dtype=np.int32)
    lda = np.asarray(ldas, dtype=np.int32)
    pa = np.array([a.ctypes.data for a in As], dtype=np.uint64)
    pb = np.array([b.ctypes.data for b in Bs], dtype=np.uint64)
    info = np.zeros(batch, dtype=np.int32)
    f(lp[0], lp[1], _p(n), _p(pa), _p(lda), _p(pb), batch, _p(info), nthreads or nthreads_default())
    return info
