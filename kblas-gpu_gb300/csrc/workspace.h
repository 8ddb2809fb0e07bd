// workspace.h -- device workspace layout of the routines that need one.
#pragma once
#include <stddef.h>

namespace kgb {

static inline size_t ws_align(size_t x) { return (x + 255) / 256 * 256; }

// Mixed-precision POSV: a queue header (counters) + a list of the systems
// that take the FP64 fallback path.
static inline size_t mixed_posv_workspace_bytes(char, int, int, int batch) {
  if (batch <= 0) return 0;
  return ws_align(64 * sizeof(int)) + ws_align((size_t)batch * sizeof(int));
}

// Variable-size POSV: the size-class histogram / offsets / queue counters,
// the binned permutation of system indices, and the FP64 fallback list.
static inline size_t vbatch_workspace_bytes(int, int batch) {
  if (batch <= 0) return 0;
  return ws_align(256 * sizeof(int)) + 2 * ws_align((size_t)batch * sizeof(int));
}

}  // namespace kgb
