// tuning_table.h -- per-size-class launch shapes of the persistent POSV
// kernels: class upper bound on n, team size (threads per system) and
// systems per work item. Written by kblas-gpu_gb300/autotune.py from
// measurements on NVIDIA GB300 (2026-12-04): per class, the team size with
// the shortest variable-size POSV over orders log-uniform in the class.
#pragma once

// {nmax}, {team size}, {systems per item}
#define KGB_TUNE_MIXED_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_MIXED_TS {8, 16, 32, 32, 64, 32, 128, 256}
#define KGB_TUNE_MIXED_SPI {32, 16, 8, 8, 4, 8, 2, 1}

// conditioning routing constant of the mixed path (route_fp64); measured
// on the n = 64, 4-RHS, cond 1e2..1e8 batch: c = 0 / 8 / 32 -> mixed at
// 0.72 / 0.89 / 0.92 of the FP64 form; no effect on well-conditioned batches
#define KGB_TUNE_ROUTE_C 32.0f

#define KGB_TUNE_PLAIN_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_PLAIN_TS {8, 16, 32, 32, 32, 32, 64, 64}
#define KGB_TUNE_PLAIN_SPI {32, 16, 8, 8, 8, 8, 4, 4}

// measured ms per call, class: {team size: ms}
//   mixed class 0: 8: 1.109, 16: 2.432, 32: 6.469
//   mixed class 1: 16: 2.664, 32: 6.786
//   mixed class 2: 32: 7.768
//   mixed class 3: 32: 6.516, 64: 10.113, 128: 18.904
//   mixed class 4: 32: 6.401, 64: 6.303, 128: 9.975, 256: 18.859
//   mixed class 5: 32: 6.112, 64: 6.398, 128: 6.692, 256: 11.846
//   mixed class 6: 64: 7.724, 128: 5.941, 256: 8.501
//   mixed class 7: 64: 8.615, 128: 8.101, 256: 6.414
//   plain class 0: 8: 0.620, 16: 1.064, 32: 2.425
//   plain class 1: 16: 2.391, 32: 6.629
//   plain class 2: 32: 12.191
//   plain class 3: 32: 13.101, 64: 17.302, 128: 32.088
//   plain class 4: 32: 13.128, 64: 15.527, 128: 23.195, 256: 43.106
//   plain class 5: 32: 14.885, 64: 15.962, 128: 20.609, 256: 34.544
//   plain class 6: 64: 17.927, 128: 21.214, 256: 30.100
//   plain class 7: 64: 20.508, 128: 22.974, 256: 28.593
