// posv_vbatch.cu -- variable-size batched POSV (work in progress).
#include "kblas_internal.h"

extern "C" {
int kblasDposv_vbatch(kblasHandle_t, char, char, int *, int *, int, int, double **, int *,
                      double **, int *, int, int *) {
  return KBLAS_NotImplemented;
}
int kblasDposv_vbatch_mixed(kblasHandle_t, char, char, int *, int *, int, int, double **, int *,
                            double **, int *, int, int *, int *) {
  return KBLAS_NotImplemented;
}
}
