"""The C-ABI library builds, loads and exports every symbol the headers
declare (CPU only: no compute call needs a GPU here)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in ("kblas.h", "kblas_batch.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
            nm = m.group(1)
            if nm.startswith("kblas") and nm not in CXX_OVERLOADS:
                names.add(nm)
    return names


CXX_OVERLOADS = {"kblas_potrf_batch", "kblas_potrs_batch", "kblas_posv_batch", "kblas_trsm_batch",
                 "kblas_trmm_batch", "kblas_syrk_batch", "kblas_gemm_batch", "kblas_trtri_batch",
                 "kblas_lauum_batch", "kblas_potri_batch", "kblas_poti_batch"}


@pytest.fixture(scope="module")
def built(kb):
    kb.build()
    return kb


def test_headers_compile_as_c(tmp_path):
    """include/kblas.h is valid C (the drop-in boundary is a C ABI)."""
    src = tmp_path / "t.c"
    src.write_text('#include "kblas.h"\nint main(void){ return KBLAS_Success == 1 ? 0 : 1; }\n')
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        "-I", cuda_inc, str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 55
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # the Python mirror covers the same set
    assert names <= set(built.EXPORTED) | {"kblasCreate"}, sorted(names - set(built.EXPORTED))


def test_cxx_overloads_exported(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built.LIB_PATH], capture_output=True,
                         text=True).stdout
    # the reference's sets: S, D, C, Z x (pointer array, strided); GEMM, SYRK and
    # TRSM add the four variable-size forms (100 overloads in all)
    counts = {b: 8 for b in CXX_OVERLOADS}
    counts.update({"kblas_trsm_batch": 12, "kblas_syrk_batch": 12, "kblas_gemm_batch": 12})
    for base, want in counts.items():
        mangled = [l for l in out.splitlines() if f"{len(base)}{base}" in l]
        assert len(mangled) == want, (base, mangled)


def test_no_oracle_or_fallback_linked(built):
    """The product library never links the oracle or a CPU LAPACK."""
    out = subprocess.run(["nm", "-D", built.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle_" not in out
    for bad in ("dpotrf_", "LAPACKE", "openblas", "mkl_"):
        assert bad not in out, bad


def test_host_side_codes_without_gpu(built):
    lib = built.lib()
    assert lib.kblasGetErrorString(-6).decode().startswith("Insufficient workspace")
    assert lib.kblas_roundup(33, 32) == 64
    # a NULL handle is rejected before any device work
    P = ctypes.c_void_p
    assert lib.kblasDpotrf_batch_strided(P(), b"L", 8, P(), 8, 64, 1, P()) == built.KBLAS_Error_NotInitialized
    assert lib.kblasDposv_batch_strided(P(), b"R", b"L", 1, 8, P(), 8, 64, P(), 1, 8, 1, P()) == \
        built.KBLAS_Error_NotInitialized
    assert lib.kblasAllocateWorkspace(P()) == built.KBLAS_Error_NotInitialized
