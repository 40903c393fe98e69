// Mixed-precision (tensor-core) variants of the hot-path ops (mixed.cu).
#pragma once
#include "kernels.h"

namespace trot {
size_t mixed_workspace_size(const trot_system* s, int op);
int mixed_force_bias(const trot_system* s, const Spins& sp, const double2* wa, const double2* wb, double2* fb_out,
                     void* ws, size_t ws_bytes, cudaStream_t st);
int mixed_local_energy(const trot_system* s, const Spins& sp, const double2* wa, const double2* wb,
                       double2* energy, void* ws, size_t ws_bytes, cudaStream_t st);
int mixed_apply_trotter(const trot_system* s, const Spins& sp, const double2* xs, const TrotterArgs& a, void* ws,
                        size_t ws_bytes, cudaStream_t st);
int mixed_prop_step(const trot_system* s, const Spins& sp, const trot_state* state, const double* fields,
                    double2* energy_out, void* ws, size_t ws_bytes, cudaStream_t st);
}  // namespace trot
