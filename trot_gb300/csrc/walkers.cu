// Walker QR orthonormalisation and stochastic reconfiguration (FP64).
#include "kernels.h"

namespace trot {

// ------------------------------------------------------------------ QR
// Reduced QR of one walker spin block (N x n) with diag(R) real non-negative
// (trot/walkers.py:137-148).  Classical Gram-Schmidt with one
// re-orthogonalisation pass (CGS2): column j is projected against Q[:, :j]
// twice, then normalised; the normalisation makes diag(R) = ||v|| >= 0, which is
// the reference's phase convention, so Q is the same matrix the phase-fixed
// Householder QR returns.  One CTA per (walker, spin).
static constexpr int kQrThreads = 256;

__global__ void __launch_bounds__(kQrThreads)
qr_kernel(int N, int n, double2* __restrict__ w, double2* __restrict__ norm, int norm_mode, int write_q) {
  extern __shared__ double2 smem[];
  __shared__ double2 red[32];
  __shared__ double2 coef[64];
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  double2* Q = smem;  // N x n
  double2* gw = w + (size_t)b * N * n;
  for (int e = tid; e < N * n; e += nt) Q[e] = gw[e];
  __syncthreads();
  double prod = 1.0;
  for (int j = 0; j < n; ++j) {
    for (int pass = 0; pass < 2; ++pass) {
      // coef[i] = <Q_i, v> for i < j  (one warp per i)
      for (int i = wid; i < j; i += nw) {
        double2 acc = cmk(0.0, 0.0);
        for (int p = lane; p < N; p += 32) {
          const double2 q = Q[p * n + i], v = Q[p * n + j];
          acc.x += q.x * v.x + q.y * v.y;
          acc.y += q.x * v.y - q.y * v.x;
        }
        acc = warp_sum2(acc);
        if (lane == 0) coef[i] = acc;
      }
      __syncthreads();
      for (int p = tid; p < N; p += nt) {
        double2 v = Q[p * n + j];
        for (int i = 0; i < j; ++i) v = csub(v, cmul(Q[p * n + i], coef[i]));
        Q[p * n + j] = v;
      }
      __syncthreads();
    }
    double2 nn = cmk(0.0, 0.0);
    for (int p = tid; p < N; p += nt) nn.x += cabs2(Q[p * n + j]);
    nn = block_sum2(nn, red);
    const double nrm = sqrt(nn.x);
    prod *= nrm;
    const double inv = 1.0 / nrm;
    for (int p = tid; p < N; p += nt) Q[p * n + j] = cscale(Q[p * n + j], inv);
    __syncthreads();
  }
  if (write_q)
    for (int e = tid; e < N * n; e += nt) gw[e] = Q[e];
  // norm_mode: 0 set det_r, 1 set det_r^2 (restricted), 2 multiply into the
  // alpha launch's value (unrestricted: det_a det_b; stream order keeps it safe)
  if (tid == 0 && norm) {
    if (norm_mode == 0) norm[b] = cmk(prod, 0.0);
    else if (norm_mode == 1) norm[b] = cmk(prod * prod, 0.0);
    else norm[b] = cmk(norm[b].x * prod, 0.0);
  }
}

int launch_qr(const Spins& sp, int W, int N, double2* wa, double2* wb, double2* norm_out, cudaStream_t st,
              bool write_q) {
  int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  if (nmax > 64) {
    set_error("qr: nocc %d > 64 unsupported", nmax);
    return TROT_ERR_UNSUPPORTED;
  }
  size_t smem = (size_t)N * nmax * sizeof(double2);
  if (smem > 200 * 1024) {
    set_error("qr: walker tile of %zu bytes exceeds shared memory", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 40 * 1024) cudaFuncSetAttribute(qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  qr_kernel<<<W, kQrThreads, smem, st>>>(N, sp.n[0], wa, norm_out, sp.mult[0] == 2 ? 1 : 0, write_q ? 1 : 0);
  TROT_CHECK_LAUNCH("qr_kernel");
  if (sp.nspin == 2) {
    qr_kernel<<<W, kQrThreads, smem, st>>>(N, sp.n[1], wb, norm_out, 2, write_q ? 1 : 0);
    TROT_CHECK_LAUNCH("qr_kernel");
  }
  return TROT_OK;
}

// ------------------------------------------------------------------ SR
// Comb resampling (trot/walkers.py:249-293): cw = cumsum|w| (sequential, same
// order as numpy), z_k = cw[-1] (k + zeta) / W, idx_k = first i with cw[i] >= z_k.
__global__ void __launch_bounds__(1024)
sr_index_kernel(int W, const double* __restrict__ weights, const double* __restrict__ zeta_dev, double zeta,
                double* __restrict__ cw, long long* __restrict__ idx, double* __restrict__ weights_out) {
  __shared__ double tot_s;
  if (zeta_dev) zeta = zeta_dev[0];
  if (threadIdx.x == 0) {
    double c = 0.0;
    for (int i = 0; i < W; ++i) {
      c += fabs(weights[i]);
      cw[i] = c;
    }
    tot_s = c;
  }
  __syncthreads();
  const double tot = tot_s;
  for (int k = threadIdx.x; k < W; k += blockDim.x) {
    const double z = tot * ((double)k + zeta) / (double)W;
    int lo = 0, hi = W;  // first i in [0, W) with cw[i] >= z; W if none
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (cw[mid] < z) lo = mid + 1; else hi = mid;
    }
    idx[k] = lo < W ? lo : W - 1;
    weights_out[k] = tot / (double)W;
  }
}

__global__ void gather_kernel(int W, size_t per, const double2* __restrict__ in, double2* __restrict__ out,
                              const long long* __restrict__ idx) {
  const int k = blockIdx.y;
  const double2* src = in + (size_t)idx[k] * per;
  double2* dst = out + (size_t)k * per;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per; e += (size_t)gridDim.x * blockDim.x)
    dst[e] = src[e];
}

int launch_sr(const Spins& sp, int W, int N, const double* weights, const double* zeta_dev, double zeta,
              const double2* ina,
              const double2* inb, double2* outa, double2* outb, double* weights_out, long long* idx,
              double* cw, cudaStream_t st) {
  sr_index_kernel<<<1, 1024, 0, st>>>(W, weights, zeta_dev, zeta, cw, idx, weights_out);
  TROT_CHECK_LAUNCH("sr_index_kernel");
  for (int s = 0; s < sp.nspin; ++s) {
    size_t per = (size_t)N * sp.n[s];
    int gx = (int)((per + 255) / 256);
    if (gx > 8) gx = 8;
    dim3 grid(gx, W);
    gather_kernel<<<grid, 256, 0, st>>>(W, per, s == 0 ? ina : inb, s == 0 ? outa : outb, idx);
    TROT_CHECK_LAUNCH("gather_kernel");
  }
  return TROT_OK;
}

// ------------------------------------------------------------------ block energy
// Block tail of trot/prop/blocks.py:236-257 on the device: E = Re(E_L); walkers
// with non-finite E get weight 0; E is clamped to e_ref when |E - e_ref| >
// sqrt(2/dt); e_block = sum w E / sum w (e_ref if sum w == 0);
// e_estimate <- (1 - ema) e_estimate + ema e_block.  obs = [e_block, sum w].
__global__ void __launch_bounds__(1024)
block_energy_kernel(int W, const double2* __restrict__ energy, double* __restrict__ weights,
                    double* __restrict__ scalars, double dt, double ema, double* __restrict__ obs) {
  __shared__ double2 red[32];
  const double e_ref = scalars[1];
  const double thresh = sqrt(2.0 / dt);
  double2 acc = cmk(0.0, 0.0);  // (sum w E, sum w)
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    double e = energy[i].x;
    const bool bad = !isfinite(e);
    if (bad || fabs(e - e_ref) > thresh) e = e_ref;
    double w = weights[i];
    if (bad) { w = 0.0; weights[i] = 0.0; }
    acc.x += w * e;
    acc.y += w;
  }
  acc = block_sum2(acc, red);
  if (threadIdx.x == 0) {
    const double wsum = acc.y;
    const double eb = wsum == 0.0 ? e_ref : acc.x / wsum;
    scalars[1] = (1.0 - ema) * scalars[1] + ema * eb;
    obs[0] = eb;
    obs[1] = wsum;
  }
}

}  // namespace trot

extern "C" int trot_block_energy(int n_walkers, const double* energy, double* weights, double* scalars,
                                 double dt, double shift_ema, double* obs_out, void* stream) {
  using namespace trot;
  if (!energy || !weights || !scalars || !obs_out) { set_error("null block-energy buffer"); return TROT_ERR_NULL_PTR; }
  if (n_walkers <= 0 || !(dt > 0.0)) { set_error("bad block-energy arguments"); return TROT_ERR_BAD_SHAPE; }
  block_energy_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(n_walkers, (const double2*)energy, weights, scalars,
                                                            dt, shift_ema, obs_out);
  TROT_CHECK_LAUNCH("block_energy_kernel");
  return TROT_OK;
}
