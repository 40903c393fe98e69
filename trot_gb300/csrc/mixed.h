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

// Complex rows x (rows, K) FP64 times a real matrix B (K, ncols) on the tensor
// cores with a 3-term BF16 split of both operands (6 products, FP32
// accumulation): D (split3_mpad(rows), npad) FP32, row 2r = Re, 2r+1 = Im of
// row r of x B.  b_image is B^T as the VHS kernel's operand image
// [npad/128][kpad/64][3 slices][128][64] (trot_gb300.mixed.split3_image);
// xq is scratch of 3 * split3_mpad(rows) * kpad uint16.  *status is set to
// TROT_ERR_DEVICE_TIMEOUT if a pipeline wait runs out.
inline int split3_mpad(int rows) { return (2 * rows + 127) / 128 * 128; }
int launch_split3_gemm(int rows, int K, int kpad, int npad, const double2* x, const uint16_t* b_image,
                       uint16_t* xq, float* D, int* status, cudaStream_t st);
}  // namespace trot
