// tri_internal.h -- the batched TRSM kernel for internal callers (the
// side-L and upper-triangle POTRS / POSV, which solve with two TRSM passes).
#pragma once

#include "device_util.cuh"
#include "kblas_internal.h"

namespace kgb {

// op(A) X = alpha B (side 'L') or X op(A) = alpha B (side 'R') over a batch;
// skip (device int[batch] or null): matrices whose entry is non-zero are left
// untouched. Instantiated for float / double with Strided or PtrArr operands.
template <typename T, class AccA, class AccB>
int trsm_batch_internal(KBlasHandle *h, char side, char uplo, char trans, char diag, int m, int n,
                        T alpha, AccA A, int lda, AccB B, int ldb, long long batch,
                        const int *skip);

}  // namespace kgb
