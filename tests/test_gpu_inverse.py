"""GPU parity of the batched inversion routines (lower; the upper forms are in
test_gpu_uplo_side.py): TRTRI, LAUUM, POTRI, POTI, S and D, strided and
pointer-array forms, against the CPU oracle (itself pinned to LAPACK in
test_oracle.py).

Bars: FP64 results within 100 n eps of the oracle relative to the largest
entry (the inverse amplifies rounding by the conditioning; the matrices here
are well conditioned), FP32 at the FP32 analogue; info codes identical to
LAPACK's; the strict upper triangle and padding never written; a singular
triangle (TRTRI / POTRI) or a non-SPD matrix (POTI) reported exactly."""
import numpy as np
import pytest

from gpu_util import eps, ptr_array, to_dev
from test_gpu_chol import check_untouched, make_batch

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 7, 16, 31, 32, 33, 64, 100, 129, 170, 257]


def factor(orc, a, n):
    L = a.astype(np.float64).copy()
    assert (orc.potrf_batch(L, n) == 0).all()
    return L.astype(a.dtype)


def call(gpu, handle, pfx, op, form, n, dev, lda, batch, info, diag="N"):
    args_d = (diag,) if op == "trtri" else ()
    if form == "strided":
        return handle.call(f"kblas{pfx}{op}_batch_strided", "L", *args_d, n, dev.data_ptr(), lda,
                           n * lda, batch, info.data_ptr())
    pa = ptr_array(gpu, dev)
    return handle.call(f"kblas{pfx}{op}_batch", "L", *args_d, n, pa.data_ptr(), lda, batch,
                       info.data_ptr())


def rel_lower(got, ref, n):
    g = np.tril(got[:, :n, :n].transpose(0, 2, 1))
    r = np.tril(ref[:, :n, :n].transpose(0, 2, 1))
    return float(np.abs(g - r).max() / max(np.abs(r).max(), 1e-300))


@pytest.mark.parametrize("dt", [np.float64, np.float32], ids=["d", "s"])
@pytest.mark.parametrize("op", ["trtri", "lauum", "potri", "poti"])
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("form", ["strided", "array"])
def test_inverse_vs_oracle(gpu, handle, wl, orc, dt, op, n, form):
    batch = 24 if n <= 64 else 4
    lda = n + 2
    a = make_batch(wl, batch, n, lda, np.float64, seed=11 * n + len(op))
    src = a if op == "poti" else factor(orc, a, n)   # POTI takes A, the others L
    src = src.astype(dt)
    ref = src.astype(np.float64).copy()
    fn = {"trtri": orc.trtri_batch, "lauum": orc.lauum_batch, "potri": orc.potri_batch,
          "poti": orc.poti_batch}[op]
    info_ref = fn(ref, n)
    dev = to_dev(gpu, src)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert call(gpu, handle, "D" if dt == np.float64 else "S", op, form, n, dev, lda, batch,
                info) == 1
    gpu.cuda.synchronize()
    out = dev.cpu().numpy()
    if info_ref is not None:
        assert np.array_equal(info.cpu().numpy(), info_ref)
    else:
        assert (info.cpu().numpy() == 0).all()
    check_untouched(src, out, n)
    tol = (100 if dt == np.float64 else 30) * n * eps(dt)
    assert rel_lower(out.astype(np.float64), ref, n) <= tol


@pytest.mark.parametrize("op", ["trtri", "potri"])
def test_singular_triangle_reported_and_untouched(gpu, handle, wl, orc, op):
    n, batch = 40, 6
    a = make_batch(wl, batch, n, n, np.float64, seed=3)
    L = factor(orc, a, n)
    L[2, 17, 17] = 0.0   # (17, 17) of matrix 2
    L[4, 0, 0] = 0.0
    dev = to_dev(gpu, L)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert call(gpu, handle, "D", op, "strided", n, dev, n, batch, info) == 1
    gpu.cuda.synchronize()
    got = info.cpu().numpy()
    assert got[2] == 18 and got[4] == 1
    out = dev.cpu().numpy()
    assert np.array_equal(out[2], L[2]) and np.array_equal(out[4], L[4])


def test_poti_non_spd_info(gpu, handle, wl, orc):
    n, batch = 48, 8
    a = make_batch(wl, batch, n, n, np.float64, seed=4)
    for s in (1, 6):
        a[s] = wl.flip_one_eigenvalue(a[s], n, seed=s)
    ref = a.copy()
    info_ref = orc.poti_batch(ref, n)
    dev = to_dev(gpu, a)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert call(gpu, handle, "D", "poti", "array", n, dev, n, batch, info) == 1
    gpu.cuda.synchronize()
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert (info_ref[[1, 6]] > 0).all()
    out = dev.cpu().numpy()
    for s in (1, 6):  # the partial factor, as LAPACK leaves it
        k = info_ref[s]
        assert np.abs(np.tril(out[s, :k - 1].T) - np.tril(ref[s, :k - 1].T)).max() <= 1e-12 * n


def test_trtri_unit_diagonal(gpu, handle, wl, orc):
    n, batch = 50, 5
    L = wl.lower_tri(batch, n, seed=8, upper_fill=0.0)
    ref = L.copy()
    orc.trtri_batch(ref, n, unit=True)
    dev = to_dev(gpu, L)
    info = gpu.full((batch,), -99, dtype=gpu.int32, device="cuda")
    assert call(gpu, handle, "D", "trtri", "strided", n, dev, n, batch, info, diag="U") == 1
    gpu.cuda.synchronize()
    assert (info.cpu().numpy() == 0).all()
    out = dev.cpu().numpy()
    assert np.array_equal(np.diagonal(out, axis1=1, axis2=2), np.diagonal(L, axis1=1, axis2=2))
    assert rel_lower(out, ref, n) <= 100 * n * eps(np.float64)
