// tuning_table.h -- per-size-class launch shapes of the persistent POSV
// kernels: class upper bound on n, team size (threads per system) and
// systems per work item. Written by kblas-gpu_gb300/autotune.py from
// measurements on NVIDIA GB300 (2026-12-04): per class, the team size with
// the shortest variable-size POSV over orders log-uniform in the class.
#pragma once

// {nmax}, {team size}, {systems per item}
#define KGB_TUNE_MIXED_NMAX {8, 16, 32, 64, 128, 1024}
#define KGB_TUNE_MIXED_TS {8, 16, 32, 32, 32, 128}
#define KGB_TUNE_MIXED_SPI {32, 16, 8, 8, 8, 2}

#define KGB_TUNE_PLAIN_NMAX {8, 16, 32, 64, 128, 1024}
#define KGB_TUNE_PLAIN_TS {8, 16, 32, 32, 32, 64}
#define KGB_TUNE_PLAIN_SPI {32, 16, 8, 8, 8, 4}

// measured ms per call, class: {team size: ms}
//   mixed class 0: 8: 1.147, 16: 2.587, 32: 6.995
//   mixed class 1: 16: 2.957, 32: 7.920
//   mixed class 2: 32: 9.286
//   mixed class 3: 32: 10.810, 64: 17.628, 128: 31.179, 256: 59.386
//   mixed class 4: 32: 8.580, 64: 8.793, 128: 12.546, 256: 21.681
//   mixed class 5: 64: 10.188, 128: 9.452, 256: 9.677
//   plain class 0: 8: 0.631, 16: 1.077, 32: 2.434
//   plain class 1: 16: 2.411, 32: 6.637
//   plain class 2: 32: 12.180
//   plain class 3: 32: 15.690, 64: 22.408, 128: 42.523, 256: 82.215
//   plain class 4: 32: 14.817, 64: 17.791, 128: 26.115, 256: 46.281
//   plain class 5: 64: 20.022, 128: 23.965, 256: 32.993
