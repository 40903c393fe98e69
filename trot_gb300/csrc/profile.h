// Per-kernel event timers (profile.cu).
#pragma once
#include <cuda_runtime.h>

namespace trot {
int prof_begin(cudaStream_t st);
void prof_end(int slot, const char* name, cudaStream_t st);

// Times one launcher call: TROT_TIMED("name", st, launch_x(...));
#define TROT_TIMED(name, st, expr)                 \
  do {                                             \
    int _slot = ::trot::prof_begin(st);            \
    int _rc = (expr);                              \
    ::trot::prof_end(_slot, name, st);             \
    if (_rc != TROT_OK) return _rc;                \
  } while (0)
}  // namespace trot
