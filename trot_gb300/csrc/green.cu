// Half Green's functions, trial overlaps and one-body energy per walker (FP64).
//
// For each walker b and spin s (trot/meas/rhf.py:21-25, trot/trial/rhf.py:45-54):
//   M_s   = C_s^T w_s                     (n_s x n_s)
//   G_s   = (w_s M_s^{-1})^T              (n_s x N)   half Green's function
//   ovlp  = prod_s det(M_s)^mult_s
//   e1    = sum_s mult_s sum_{i,p} G_s[i][p] rot_h1_s[i][p]
// One CTA per walker; the walker tile, M and M^{-1} live in shared memory.
#include "kernels.h"

namespace trot {

static constexpr int kGreenThreads = 256;
static constexpr int kMaxOcc = 64;

__global__ void __launch_bounds__(kGreenThreads)
green_kernel(Spins sp, int N, const double2* __restrict__ wa, const double2* __restrict__ wb,
             double2* __restrict__ green, double2* __restrict__ ovlp_out, double2* __restrict__ e1_out) {
  extern __shared__ double2 smem[];
  __shared__ double2 red[32];
  __shared__ int piv;
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const bool want_green = green != nullptr || e1_out != nullptr;
  double2 det_all = cmk(1.0, 0.0);
  double2 e1_all = cmk(0.0, 0.0);
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    const double2* w = (s == 0 ? wa : wb) + (size_t)b * N * n;
    const double* C = sp.mo[s];
    double2* Ws = smem;                 // N x n
    double2* Ms = Ws + N * n;           // n x n
    double2* Mi = Ms + n * n;           // n x n
    for (int e = tid; e < N * n; e += nt) Ws[e] = w[e];
    __syncthreads();
    // M = C^T w
    for (int e = tid; e < n * n; e += nt) {
      const int i = e / n, j = e % n;
      double2 acc = cmk(0.0, 0.0);
      for (int p = 0; p < N; ++p) crfma(acc, C[p * n + i], Ws[p * n + j]);
      Ms[e] = acc;
    }
    __syncthreads();
    double2 det = block_gauss_jordan(Ms, n, n, want_green ? Mi : nullptr, &piv, red);
    det_all = cmul(det_all, sp.mult[s] == 2 ? cmul(det, det) : det);
    if (want_green) {
      // G[i][p] = sum_j w[p][j] Minv[j][i]
      double2 e1 = cmk(0.0, 0.0);
      const double* H = sp.rot_h1[s];
      double2* gout = green ? green + (size_t)b * sp.ntot * N + (size_t)sp.off[s] * N : nullptr;
      for (int e = tid; e < n * N; e += nt) {
        const int i = e / N, p = e % N;
        double2 acc = cmk(0.0, 0.0);
        for (int j = 0; j < n; ++j) cfma(acc, Ws[p * n + j], Mi[j * n + i]);
        if (gout) gout[e] = acc;
        if (H) crfma(e1, H[e], acc);
      }
      e1 = block_sum2(e1, red);
      e1_all = cadd(e1_all, cscale(e1, (double)sp.mult[s]));
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (ovlp_out) ovlp_out[b] = det_all;
    if (e1_out) e1_out[b] = e1_all;
  }
}

int launch_green(const Spins& sp, int W, int N, const double2* wa, const double2* wb, double2* green,
                 double2* ovlp_out, double2* e1_out, cudaStream_t st) {
  int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  if (nmax > kMaxOcc) {
    set_error("green: nocc %d > %d unsupported", nmax, kMaxOcc);
    return TROT_ERR_UNSUPPORTED;
  }
  size_t smem = (size_t)(N * nmax + 2 * nmax * nmax) * sizeof(double2);
  if (smem > 200 * 1024) {
    set_error("green: walker tile of %zu bytes exceeds shared memory", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 40 * 1024)
    cudaFuncSetAttribute(green_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  green_kernel<<<W, kGreenThreads, smem, st>>>(sp, N, wa, wb, green, ovlp_out, e1_out);
  TROT_CHECK_LAUNCH("green_kernel");
  return TROT_OK;
}

}  // namespace trot
