// tuning_table.h -- per-size-class launch shapes of the persistent POSV
// kernels: class upper bound on n, team size (threads per system) and
// systems per work item. Written by kblas-gpu_gb300/autotune.py from
// measurements on NVIDIA GB300 (2026-12-04): per class, the team size with
// the shortest variable-size POSV over orders log-uniform in the class.
#pragma once

// {nmax}, {team size}, {systems per item}
// conditioning routing constant of the mixed path (route_fp64): the
// fastest mixed POSV on n = 64, 4 RHS, cond 1e2..1e8 (ms per call: c 0: 8.370, c 4: 6.742, c 8: 6.741, c 16: 6.626, c 32: 6.501, c 64: 6.569, c 128: 6.681)
#define KGB_TUNE_ROUTE_C 32.0f

#define KGB_TUNE_MIXED_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_MIXED_TS {8, 16, 32, 32, 64, 32, 128, 256}
#define KGB_TUNE_MIXED_SPI {32, 16, 8, 8, 4, 8, 2, 1}

#define KGB_TUNE_PLAIN_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_PLAIN_TS {8, 16, 32, 32, 32, 32, 64, 64}
#define KGB_TUNE_PLAIN_SPI {32, 16, 8, 8, 8, 8, 4, 4}

// measured ms per call, class: {team size: ms}
//   mixed class 0: 8: 1.179, 16: 2.547, 32: 6.643
//   mixed class 1: 16: 2.766, 32: 6.868
//   mixed class 2: 32: 7.839
//   mixed class 3: 32: 6.664, 64: 10.222, 128: 19.111
//   mixed class 4: 32: 6.523, 64: 6.368, 128: 10.148, 256: 19.466
//   mixed class 5: 32: 6.148, 64: 6.458, 128: 6.825, 256: 12.230
//   mixed class 6: 64: 7.771, 128: 6.020, 256: 8.805
//   mixed class 7: 64: 8.633, 128: 8.100, 256: 6.600
//   plain class 0: 8: 0.637, 16: 1.086, 32: 2.462
//   plain class 1: 16: 2.444, 32: 6.725
//   plain class 2: 32: 12.273
//   plain class 3: 32: 13.197, 64: 17.274, 128: 32.045
//   plain class 4: 32: 13.121, 64: 15.425, 128: 23.138, 256: 42.936
//   plain class 5: 32: 14.882, 64: 15.877, 128: 20.607, 256: 34.454
//   plain class 6: 64: 17.888, 128: 21.046, 256: 30.013
//   plain class 7: 64: 20.475, 128: 22.847, 256: 28.391
