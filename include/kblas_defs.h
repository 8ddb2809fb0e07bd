/*
 * kblas_defs.h -- flag characters and return codes of the KBLAS C API.
 *
 * Drop-in replacement for the reference header include/kblas_defs.h:24-49
 * (same macro names, same values), so code written against KBLAS compiles
 * unchanged against this library.
 */
#ifndef KBLAS_GB300_DEFS_H
#define KBLAS_GB300_DEFS_H

/* flag characters (reference include/kblas_defs.h:24-33) */
#define KBLAS_Lower    'L'
#define KBLAS_Upper    'U'
#define KBLAS_Left     'L'
#define KBLAS_Right    'R'
#define KBLAS_Trans    'T'
#define KBLAS_NoTrans  'N'
#define KBLAS_Unit     'U'
#define KBLAS_NonUnit  'N'
#define KBLAS_Symm     'S'
#define KBLAS_NonSymm  'N'

/* return codes (reference include/kblas_defs.h:36-49) */
#define KBLAS_Success                 1
#define KBLAS_UnknownError            0
#define KBLAS_NotSupported           -1
#define KBLAS_NotImplemented         -2
#define KBLAS_cuBLAS_Error           -3
#define KBLAS_WrongConfig            -4
#define KBLAS_CUDA_Error             -5
#define KBLAS_InsufficientWorkspace  -6
#define KBLAS_Error_Allocation       -7
#define KBLAS_Error_Deallocation     -8
#define KBLAS_Error_NotInitialized   -9
#define KBLAS_Error_WrongInput      -10
#define KBLAS_MAGMA_Error           -11
#define KBLAS_SVD_NoConvergence     -12

/* Status code added by this library: a bounded device-side wait of the
 * mixed-precision persistent kernel (for its tensor-core MMAs) ran out; the
 * kernel stopped without writing results. Reported by kblasGetDeviceStatus.
 * No reference counterpart. */
#define KBLAS_Error_Timeout         -13

#define KBLAS_NSTREAMS 10

#endif /* KBLAS_GB300_DEFS_H */
