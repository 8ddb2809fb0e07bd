/*
 * kblas.h -- handle, stream, timer, workspace and error API.
 *
 * Drop-in for the reference header include/kblas.h:35-108. The handle type is
 * opaque (`struct KBlasHandle*`) exactly as in the reference, and every
 * function below keeps the reference name, argument list and return
 * convention (KBLAS_Success == 1, errors <= 0).
 *
 * Only the batched Cholesky / triangular family is provided (kblas_batch.h);
 * the reference's Level-2/3, TLR and SVD headers are not part of this library.
 */
#ifndef KBLAS_GB300_H
#define KBLAS_GB300_H

#include <cuda_runtime_api.h>
#include <cublas_v2.h>
#include "kblas_defs.h"

#ifdef __cplusplus
extern "C" {
#endif

struct KBlasHandle;
typedef struct KBlasWorkspace *kblasWorkspace_t;
typedef struct KBlasHandle *kblasHandle_t;

/* reference src/kblas_common.cu:35 -- creates a handle bound to the current
 * device and the legacy default stream. */
int kblasCreate(kblasHandle_t *handle);

/* reference src/kblas_common.cu:77 -- frees the handle, its workspace and any
 * streams/cuBLAS handle it created; sets *handle to NULL. */
int kblasDestroy(kblasHandle_t *handle);

/* reference src/kblas_common.cu:99-109 -- CUDA-event timer on the handle's
 * stream. Toc returns elapsed milliseconds since Tic (or RecordEnd). */
void   kblasTimerTic(kblasHandle_t handle);
void   kblasTimerRecordEnd(kblasHandle_t handle);
double kblasTimerToc(kblasHandle_t handle);

/* reference src/kblas_common.cu:111-125 */
int          kblasCreateStreams(kblasHandle_t handle, int nStreams);
cudaStream_t kblasGetStream(kblasHandle_t handle);
void         kblasSetStream(kblasHandle_t handle, cudaStream_t stream);

/* reference src/kblas_common.cu:127. No routine of this library calls cuBLAS;
 * the handle is created on first request and follows kblasSetStream. */
cublasHandle_t kblasGetCublasHandle(kblasHandle_t handle);

/* reference src/kblas_common.cu:53. MAGMA is not used by this library:
 * always returns KBLAS_Error_NotInitialized, as the reference does when it is
 * built without MAGMA. */
int kblasEnableMagma(kblasHandle_t handle);

/* reference src/kblas_common.cu:170 */
const char *kblasGetErrorString(int error);

/* reference src/kblas_common.cu:88-97 -- allocate (grow) the workspace to what
 * the *_wsquery calls requested since the last allocation / release it. */
int kblasAllocateWorkspace(kblasHandle_t handle);
int kblasFreeWorkspace(kblasHandle_t handle);

/* reference src/kblas_common.cu:258 */
int kblas_roundup(int x, int y);

#ifdef __cplusplus
}
#endif

#include "kblas_batch.h"

#endif /* KBLAS_GB300_H */
