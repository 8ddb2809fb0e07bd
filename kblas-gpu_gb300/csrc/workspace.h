// workspace.h -- device workspace needs of the routines that have one (the
// persistent mixed-precision and variable-size POSV); defined beside them.
#pragma once
#include <stddef.h>

struct KBlasHandle;

namespace kgb {

size_t mixed_posv_ws_bytes(KBlasHandle *h, int n, long long batch);
size_t vbatch_ws_bytes(KBlasHandle *h, int max_n, long long batch, bool mixed);
size_t fp64_uniform_ws_bytes(KBlasHandle *h, int n, long long batch);

}  // namespace kgb
