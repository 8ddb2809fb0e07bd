// tuning_table.h -- per-size-class launch shapes of the persistent POSV
// kernels: class upper bound on n, team size (threads per system) and
// systems per work item. Written by kblas-gpu_gb300/autotune.py from
// measurements on GB300; these defaults are the hand-picked starting point.
#pragma once

// {nmax}, {team size}, {systems per item}
#define KGB_TUNE_MIXED_NMAX {8, 16, 32, 64, 128, 1024}
#define KGB_TUNE_MIXED_TS {8, 16, 32, 32, 128, 256}
#define KGB_TUNE_MIXED_SPI {32, 16, 8, 8, 2, 1}

#define KGB_TUNE_PLAIN_NMAX {8, 16, 32, 64, 128, 1024}
#define KGB_TUNE_PLAIN_TS {8, 16, 32, 32, 128, 256}
#define KGB_TUNE_PLAIN_SPI {32, 16, 8, 8, 2, 1}
