// posv_mixed.cu -- mixed-precision batched POSV (work in progress).
#include "kblas_internal.h"

extern "C" {
int kblasDposv_batch_mixed_strided(kblasHandle_t, char, char, const int, const int, double *, int,
                                   long, double *, int, long, int, int *, int *) {
  return KBLAS_NotImplemented;
}
int kblasDposv_batch_mixed(kblasHandle_t, char, char, const int, const int, double **, int,
                           double **, int, int, int *, int *) {
  return KBLAS_NotImplemented;
}
}
