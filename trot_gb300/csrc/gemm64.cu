// FP64 complex x real GEMM on the CUDA cores.
//
//   C[m][n] (+)= alpha * sum_k A[m][k] * B(k, n)
//
// A complex row-major (lda), B real either (N, K) row-major ("nk", the force
// bias: rot_chol_flat is (G, n*N)) or (K, N) row-major ("kn", the VHS build:
// chol_flat is (G, N*N)).  Used by the FP64 force bias
// (trot/meas/rhf.py:125) and the FP64 VHS build
// (trot/prop/chol_afqmc_ops.py:83-87: Re(x) @ chol_flat + i Im(x) @ chol_flat).
// GB300's FP64 rate is ~2 FMA/clk/SM, so this kernel is FP64-pipe bound with
// any reasonable register tiling: 64x64 tiles, 4x4 complex outputs per thread.
#include "kernels.h"

namespace trot {

static constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

template <bool B_NK>
__global__ void __launch_bounds__(NT)
zgemm_cr_kernel(int M, int Nn, int K, double alpha, const double2* __restrict__ A, int lda,
                const double* __restrict__ B, int ldb, double2* __restrict__ C, int ldc, int accumulate, int kchunk,
                double2* __restrict__ part) {
  __shared__ double2 As[BK][BM + 1];
  __shared__ double Bs[BK][BN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  double2 acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cmk(0.0, 0.0);

  // split K (part != null): slice blockIdx.z covers [kb, ke) and writes its unscaled partial
  const int kb = part ? blockIdx.z * kchunk : 0;
  const int ke = part ? min(K, kb + kchunk) : K;
  for (int k0 = kb; k0 < ke; k0 += BK) {
    // A tile: BM x BK complex, 4 per thread
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int e = tid + r * NT;
      int mm = e / BK, kk = e % BK;
      int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < ke) ? A[(size_t)gm * lda + gk] : cmk(0.0, 0.0);
    }
    // B tile: BK x BN real, 4 per thread
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      int e = tid + r * NT;
      int kk, nn;
      if (B_NK) { nn = e / BK; kk = e % BK; } else { kk = e / BN; nn = e % BN; }
      int gn = n0 + nn, gk = k0 + kk;
      double v = 0.0;
      if (gn < Nn && gk < ke) v = B_NK ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      double2 a[4];
      double bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) crfma(acc[i][j], bv[j], a[i]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gn = n0 + tx + 16 * j;
      if (gn >= Nn) continue;
      if (part) {
        part[((size_t)blockIdx.z * M + gm) * Nn + gn] = acc[i][j];
        continue;
      }
      double2 v = cscale(acc[i][j], alpha);
      double2* c = C + (size_t)gm * ldc + gn;
      *c = accumulate ? cadd(*c, v) : v;
    }
  }
}

// C[m][n] (+)= alpha sum_z part[z][m][n] in slice order (deterministic)
__global__ void zgemm_splitk_reduce_kernel(int M, int Nn, int S, double alpha, const double2* __restrict__ part,
                                           double2* __restrict__ C, int ldc, int accumulate) {
  const size_t total = (size_t)M * Nn;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    double2 v = cmk(0.0, 0.0);
    for (int z = 0; z < S; ++z) v = cadd(v, part[(size_t)z * total + e]);
    const size_t m = e / Nn, n = e % Nn;
    double2* c = C + m * ldc + n;
    v = cscale(v, alpha);
    *c = accumulate ? cadd(*c, v) : v;
  }
}

int launch_zgemm_cr(int M, int Nn, int K, double alpha, const double2* A, int lda, const double* B,
                    int ldb, bool b_is_nk, double2* C, int ldc, bool accumulate, cudaStream_t st) {
  return launch_zgemm_cr_splitk(M, Nn, K, alpha, A, lda, B, ldb, b_is_nk, C, ldc, accumulate, nullptr, 1, st);
}

int launch_zgemm_cr_splitk(int M, int Nn, int K, double alpha, const double2* A, int lda, const double* B, int ldb,
                           bool b_is_nk, double2* C, int ldc, bool accumulate, double2* part, int S,
                           cudaStream_t st) {
  if (M <= 0 || Nn <= 0) return TROT_OK;
  if (!part) S = 1;
  const int kchunk = ((K + S - 1) / S + BK - 1) / BK * BK;
  if (part) S = (K + kchunk - 1) / kchunk;
  dim3 grid((Nn + BN - 1) / BN, (M + BM - 1) / BM, part ? S : 1);
  if (grid.y > 65535 || grid.z > 65535) {
    set_error("zgemm_cr: M=%d too large", M);
    return TROT_ERR_UNSUPPORTED;
  }
  if (b_is_nk)
    zgemm_cr_kernel<true><<<grid, NT, 0, st>>>(M, Nn, K, alpha, A, lda, B, ldb, C, ldc, accumulate, kchunk, part);
  else
    zgemm_cr_kernel<false><<<grid, NT, 0, st>>>(M, Nn, K, alpha, A, lda, B, ldb, C, ldc, accumulate, kchunk, part);
  TROT_CHECK_LAUNCH("zgemm_cr_kernel");
  if (part) {
    const size_t total = (size_t)M * Nn;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    zgemm_splitk_reduce_kernel<<<blocks, 256, 0, st>>>(M, Nn, S, alpha, part, C, ldc, accumulate ? 1 : 0);
    TROT_CHECK_LAUNCH("zgemm_splitk_reduce_kernel");
  }
  return TROT_OK;
}


// ------------------------------------------------------------------ packed symmetric VHS
// With every L_g symmetric, V_b = sum_g xs[b][g] L_g is symmetric: its upper triangle
// (row-major packed columns k(p, q) = p N - p (p - 1) / 2 + q - p, q >= p) is one product over
// the N (N + 1) / 2 packed columns of the Cholesky vectors, mirrored into the full matrix:
// half the FP64 products, and every element is the same dot product over g as in the full
// product, so the values are identical.
__global__ void vhs_unpack_kernel(int W, int N, const double2* __restrict__ vp, double2* __restrict__ vhs) {
  const size_t P = (size_t)N * (N + 1) / 2, total = (size_t)W * N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / ((size_t)N * N);
    const int r = (int)(e % ((size_t)N * N)), i = r / N, j = r % N;
    const int p = i < j ? i : j, q = i < j ? j : i;
    vhs[e] = vp[b * P + (size_t)p * N - (size_t)p * (p - 1) / 2 + (q - p)];
  }
}

// Mp[b][k(i, j)] = M[b][i][j] + M[b][j][i] off the diagonal, M[b][i][i] on it: with a
// symmetric L, sum_ij L[i][j] M[i][j] = sum_{i <= j} L[i][j] Mp[k(i, j)].
__global__ void pack_sym_kernel(int N, int W, const double2* __restrict__ m, double2* __restrict__ mp) {
  const size_t P = (size_t)N * (N + 1) / 2, total = (size_t)W * N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / ((size_t)N * N);
    const int r = (int)(e % ((size_t)N * N)), i = r / N, j = r % N;
    if (j < i) continue;
    double2 v = m[e];
    if (j > i) v = cadd(v, m[b * N * N + (size_t)j * N + i]);
    mp[b * P + (size_t)i * N - (size_t)i * (i - 1) / 2 + (j - i)] = v;
  }
}

static int grid_1d(size_t total) {
  const size_t b = (total + 255) / 256;
  return (int)(b < 152 * 32 ? (b > 0 ? b : 1) : 152 * 32);
}

int launch_vhs64(int W, int N, int G, const double2* xs, const double* chol_flat, const double* chol_packed,
                 double2* vp, double2* vhs, cudaStream_t st) {
  if (!chol_packed || !vp)
    return launch_zgemm_cr(W, N * N, G, 1.0, xs, G, chol_flat, N * N, false, vhs, N * N, false, st);
  const int P = N * (N + 1) / 2;
  TROT_TRY(launch_zgemm_cr(W, P, G, 1.0, xs, G, chol_packed, P, false, vp, P, false, st));
  vhs_unpack_kernel<<<grid_1d((size_t)W * N * N), 256, 0, st>>>(W, N, vp, vhs);
  TROT_CHECK_LAUNCH("vhs_unpack_kernel");
  return TROT_OK;
}

int launch_pack_sym(int N, int W, const double2* m, double2* mp, cudaStream_t st) {
  pack_sym_kernel<<<grid_1d((size_t)W * N * N), 256, 0, st>>>(N, W, m, mp);
  TROT_CHECK_LAUNCH("pack_sym_kernel");
  return TROT_OK;
}

}  // namespace trot
