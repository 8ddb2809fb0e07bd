// tuning_table.h -- per-size-class launch shapes of the persistent POSV
// kernels: class upper bound on n, team size (threads per system) and
// systems per work item. Written by kblas-gpu_gb300/autotune.py from
// measurements on NVIDIA GB300 (2026-12-04): per class, the team size with
// the shortest variable-size POSV over orders log-uniform in the class.
#pragma once

// {nmax}, {team size}, {systems per item}
#define KGB_TUNE_MIXED_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_MIXED_TS {8, 16, 32, 32, 32, 64, 128, 256}
#define KGB_TUNE_MIXED_SPI {32, 16, 8, 8, 8, 4, 2, 1}

#define KGB_TUNE_PLAIN_NMAX {8, 16, 32, 64, 96, 128, 176, 1024}
#define KGB_TUNE_PLAIN_TS {8, 16, 32, 32, 32, 32, 64, 64}
#define KGB_TUNE_PLAIN_SPI {32, 16, 8, 8, 8, 8, 4, 4}

// measured ms per call, class: {team size: ms}
//   mixed class 0: 8: 1.141, 16: 2.581, 32: 6.975
//   mixed class 1: 16: 2.949, 32: 7.898
//   mixed class 2: 32: 9.223
//   mixed class 3: 32: 7.930, 64: 12.151, 128: 22.646
//   mixed class 4: 32: 7.388, 64: 7.808, 128: 12.484, 256: 22.497
//   mixed class 5: 32: 7.474, 64: 7.294, 128: 8.519, 256: 14.222
//   mixed class 6: 64: 9.018, 128: 7.132, 256: 10.372
//   mixed class 7: 64: 10.036, 128: 9.487, 256: 7.514
//   plain class 0: 8: 0.623, 16: 1.063, 32: 2.426
//   plain class 1: 16: 2.396, 32: 6.625
//   plain class 2: 32: 12.186
//   plain class 3: 32: 15.692, 64: 22.366, 128: 42.334
//   plain class 4: 32: 14.945, 64: 19.034, 128: 30.111, 256: 56.267
//   plain class 5: 32: 16.254, 64: 18.666, 128: 25.802, 256: 44.342
//   plain class 6: 64: 19.945, 128: 25.175, 256: 37.459
//   plain class 7: 64: 21.873, 128: 25.794, 256: 34.037
