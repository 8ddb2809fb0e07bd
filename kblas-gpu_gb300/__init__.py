"""Python host bindings of the GB300 KBLAS batched Cholesky / triangular library.

A thin ctypes mirror of the C ABI declared in ``include/kblas*.h`` (the same
entry points a C or C++ KBLAS caller links against). Device buffers are
passed as raw device pointers, e.g. ``tensor.data_ptr()`` of a CUDA tensor;
nothing here computes -- every call goes to ``libkblas_gb300.so``. Importing
the package does not load the library; the first call does, and raises if
it has not been built (``build()``), so no path silently falls back.
"""
from __future__ import annotations

import ctypes as C
import importlib.util
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkblas_gb300.so")
PROBE_PATH = os.path.join(HERE, "libkblas_probe.so")

KBLAS_Success = 1
KBLAS_UnknownError = 0
KBLAS_NotSupported = -1
KBLAS_NotImplemented = -2
KBLAS_CUDA_Error = -5
KBLAS_InsufficientWorkspace = -6
KBLAS_Error_NotInitialized = -9
KBLAS_Error_WrongInput = -10
KBLAS_Error_Timeout = -13

_lock = threading.Lock()
_lib = None
_probe = None


def build(verbose: bool = False) -> str:
    spec = importlib.util.spec_from_file_location("_kblas_gb300_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)


class KblasError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = lib().kblasGetErrorString(code).decode()
        super().__init__(f"{where}: KBLAS error {code} ({msg})")
        self.code = code


P = C.c_void_p
I = C.c_int
L = C.c_long
D = C.c_double
F = C.c_float
CH = C.c_char

# name -> (restype, argtypes); R marks the real type (F or D) per precision
_SIG = {
    "kblasCreate": (I, [P]),
    "kblasDestroy": (I, [P]),
    "kblasTimerTic": (None, [P]),
    "kblasTimerRecordEnd": (None, [P]),
    "kblasTimerToc": (D, [P]),
    "kblasCreateStreams": (I, [P, I]),
    "kblasGetStream": (P, [P]),
    "kblasSetStream": (None, [P, P]),
    "kblasGetCublasHandle": (P, [P]),
    "kblasEnableMagma": (I, [P]),
    "kblasGetErrorString": (C.c_char_p, [I]),
    "kblasAllocateWorkspace": (I, [P]),
    "kblasFreeWorkspace": (I, [P]),
    "kblas_roundup": (I, [I, I]),
    "kblasGetDeviceStatus": (I, [P]),
    "kblas_syrk_batch_wsquery": (None, [P, I, I]),
    "kblas_trsm_batch_wsquery": (None, [P, CH, I, I, I]),
    "kblas_trsm_batch_strided_wsquery": (None, [P, CH, I, I, I]),
    "kblas_trmm_batch_wsquery": (None, [P, CH, I, I, I]),
    "kblas_trmm_batch_strided_wsquery": (None, [P, CH, I, I, I]),
    "kblas_potrf_batch_wsquery": (None, [P, I, I]),
    "kblas_potrf_batch_strided_wsquery": (None, [P, I, I]),
    "kblas_potrs_batch_wsquery": (None, [P, I, I, I]),
    "kblas_potrs_batch_strided_wsquery": (None, [P, I, I, I]),
    "kblas_posv_batch_wsquery": (None, [P, CH, I, I, I]),
    "kblas_posv_batch_strided_wsquery": (None, [P, CH, I, I, I]),
    "kblas_posv_batch_mixed_wsquery": (None, [P, CH, I, I, I]),
    "kblas_posv_vbatch_wsquery": (None, [P, I, I]),
    "kblasDposv_batch_mixed_strided": (I, [P, CH, CH, I, I, P, I, L, P, I, L, I, P, P]),
    "kblasDposv_batch_mixed_strided_noalloc": (I, [P, CH, CH, I, I, P, I, L, P, I, L, I, P, P]),
    "kblasDposv_batch_mixed": (I, [P, CH, CH, I, I, P, I, P, I, I, P, P]),
    "kblasDposv_vbatch": (I, [P, CH, CH, P, P, I, I, P, P, P, P, I, P]),
    "kblasDposv_vbatch_mixed": (I, [P, CH, CH, P, P, I, I, P, P, P, P, I, P, P]),
    "kblasSetPosvTuning": (I, [I, P, P, P]),
    "kblasSetPosvRouting": (I, [D]),
    "kblas_trtri_batch_wsquery": (None, [P, I, I]),
    "kblas_trtri_batch_strided_wsquery": (None, [P, I, I]),
    "kblas_lauum_batch_wsquery": (None, [P, I, I]),
    "kblas_lauum_batch_strided_wsquery": (None, [P, I, I]),
    "kblas_potri_batch_wsquery": (None, [P, I, I]),
    "kblas_potri_batch_strided_wsquery": (None, [P, I, I]),
    "kblas_poti_batch_wsquery": (None, [P, I, I]),
    "kblas_poti_batch_strided_wsquery": (None, [P, I, I]),
    "kblas_gemm_batch_strided_wsquery": (None, [P, I]),
    "kblas_gemm_batch_nonuniform_wsquery": (None, [P]),
    "kblas_syrk_batch_nonuniform_wsquery": (None, [P]),
    "kblas_trsm_batch_nonuniform_wsquery": (None, [P]),
}
for _x in ("S", "D", "C", "Z"):
    _SIG.update({
        f"kblas{_x}trtri_batch": (I, [P, CH, CH, I, P, I, I, P]),
        f"kblas{_x}trtri_batch_strided": (I, [P, CH, CH, I, P, I, L, I, P]),
    })
    for _op in ("lauum", "potri", "poti"):
        _SIG.update({
            f"kblas{_x}{_op}_batch": (I, [P, CH, I, P, I, I, P]),
            f"kblas{_x}{_op}_batch_strided": (I, [P, CH, I, P, I, L, I, P]),
        })
class ComplexF(C.Structure):
    """cuFloatComplex by value."""
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class ComplexD(C.Structure):
    """cuDoubleComplex by value."""
    _fields_ = [("x", C.c_double), ("y", C.c_double)]


for _x, _R in (("S", F), ("D", D), ("C", ComplexF), ("Z", ComplexD)):
    _SIG.update({
        f"kblas{_x}syrk_batch": (I, [P, CH, CH, I, I, _R, P, I, _R, P, I, I]),
        f"kblas{_x}syrk_batch_strided": (I, [P, CH, CH, I, I, _R, P, I, L, _R, P, I, L, I]),
        f"kblas{_x}trsm_batch": (I, [P, CH, CH, CH, CH, I, I, _R, P, I, P, I, I]),
        f"kblas{_x}trsm_batch_strided": (I, [P, CH, CH, CH, CH, I, I, _R, P, I, L, P, I, L, I]),
        f"kblas{_x}trmm_batch": (I, [P, CH, CH, CH, CH, I, I, _R, P, I, P, I, I]),
        f"kblas{_x}trmm_batch_strided": (I, [P, CH, CH, CH, CH, I, I, _R, P, I, L, P, I, L, I]),
        f"kblas{_x}potrf_batch": (I, [P, CH, I, P, I, I, P]),
        f"kblas{_x}potrf_batch_strided": (I, [P, CH, I, P, I, L, I, P]),
        f"kblas{_x}potrs_batch": (I, [P, CH, CH, I, I, P, I, P, I, I]),
        f"kblas{_x}potrs_batch_strided": (I, [P, CH, CH, I, I, P, I, L, P, I, L, I]),
        f"kblas{_x}posv_batch": (I, [P, CH, CH, I, I, P, I, P, I, I, P]),
        f"kblas{_x}posv_batch_strided": (I, [P, CH, CH, I, I, P, I, L, P, I, L, I, P]),
        f"kblas{_x}gemm_batch": (I, [P, CH, CH, I, I, I, _R, P, I, P, I, _R, P, I, I]),
        f"kblas{_x}gemm_batch_strided": (I, [P, CH, CH, I, I, I, _R, P, I, L, P, I, L, _R, P, I,
                                             L, I]),
        f"kblas{_x}gemm_vbatch": (I, [P, CH, CH, P, P, P, I, I, I, _R, P, P, P, P, _R, P, P, I]),
        f"kblas{_x}syrk_vbatch": (I, [P, CH, CH, P, P, I, I, _R, P, P, _R, P, P, I]),
        f"kblas{_x}trsm_vbatch": (I, [P, CH, CH, CH, CH, P, P, I, I, _R, P, P, P, P, I]),
    })

EXPORTED = sorted(_SIG)


def lib():
    """Load libkblas_gb300.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: run build() (nvcc, sm_103a) first")
            L_ = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIG.items():
                f = getattr(L_, name)
                f.restype = res
                f.argtypes = args
            _lib = L_
    return _lib


def probe_lib():
    global _probe
    with _lock:
        if _probe is None:
            if not os.path.exists(PROBE_PATH):
                raise RuntimeError(f"{PROBE_PATH} is missing: run build() first")
            _probe = C.CDLL(PROBE_PATH)
            _probe.kblas_probe_fma.restype = C.c_float
            _probe.kblas_probe_fma.argtypes = [I, I, I, I, I, P]
            _probe.kblas_probe_fma64_lanes.restype = C.c_float
            _probe.kblas_probe_fma64_lanes.argtypes = [I, I, I, I, P]
    return _probe


def check(code: int, where: str = "kblas"):
    if code != KBLAS_Success:
        raise KblasError(code, where)
    return code


def _b(c: str) -> bytes:
    return c.encode() if isinstance(c, str) else c


def prefix(dtype) -> str:
    """'D' for float64 / 'S' for float32 (numpy or torch dtype)."""
    s = str(dtype)
    if "float64" in s or s == "double":
        return "D"
    if "float32" in s or s == "float":
        return "S"
    raise TypeError(f"unsupported dtype {dtype}")


class Handle:
    """Owns a kblasHandle_t; optional stream (cudaStream_t as int)."""

    def __init__(self, stream: int | None = None):
        self.ptr = P()
        check(lib().kblasCreate(C.byref(self.ptr)), "kblasCreate")
        if stream is not None:
            lib().kblasSetStream(self.ptr, P(stream))

    def close(self):
        if self.ptr:
            lib().kblasDestroy(C.byref(self.ptr))
            self.ptr = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream: int):
        lib().kblasSetStream(self.ptr, P(stream))

    def allocate_workspace(self):
        return lib().kblasAllocateWorkspace(self.ptr)

    def device_status(self) -> int:
        return lib().kblasGetDeviceStatus(self.ptr)

    # ---- generic call by C name: self.call("kblasDposv_batch_strided", ...) ----
    def call(self, name: str, *args) -> int:
        f = getattr(lib(), name)
        types = list(f.argtypes[1:]) if f.argtypes else []
        types += [None] * (len(args) - len(types))
        conv = []
        for a, t in zip(args, types):
            if isinstance(a, str):
                a = _b(a)
            elif t in (ComplexF, ComplexD):
                z = complex(a)
                a = t(z.real, z.imag)
            conv.append(a)
        return f(self.ptr, *conv)
