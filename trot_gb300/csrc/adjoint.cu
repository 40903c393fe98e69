// Hand-written adjoint (reverse mode) of the phaseless step, the local energy,
// the trial overlap and the QR orthonormalisation, for an RHF trial with
// restricted walkers in FP64.  The reference has no adjoint; the forward
// formulas differentiated here are trot/prop/afqmc.py:91-144 (step),
// trot/meas/rhf.py:21-60,128-138 (local energy), trot/trial/rhf.py:45-47
// (overlap) and trot/walkers.py:137-179 (QR).
//
// Cotangents follow the convention g_z = dJ/dRe z + i dJ/dIm z for a real
// objective J (so dJ = Re sum conj(g_z) dz): for a holomorphic map y = f(z),
// g_z += conj(f'(z)) g_y; for y = A z, g_z = A^H g_y.
//
// Per walker w (N x n), trial C (N x n, real), O = C^T w, P = O^-1, Gt = w P,
// G = Gt^T (n x N), overlap det(O)^2:
//   G:        g_w += (g_Gt - C (Gt^H g_Gt)) P^H
//   overlap:  g_w += 2 conj(ov) g_ov C conj(P)^T
//   QR:       Q = w R^-1 with every later quantity invariant under Q -> Q M, so
//             g_w = g_Q R^-H = g_Q (w^H Q)^-1
//   Taylor:   y = sum_k c_k V^k x, c_k = (i sqrt(dt))^k / k!:
//             g_x = sum_k conj(c_k) (V^H)^k g_y,
//             g_V = sum_l s_l (V^l x)^H,  s_l = sum_{j <= K-1-l} conj(c_{j+l+1}) (V^H)^j g_y
//   weights:  imp_ph = exp(Re q) Re(rho e^{ic}), rho = ov'/ov,
//             q = -sqrt(dt) st + ft + dt (E_shift + h0_prop), c = -sqrt(dt) Re(sum xs m)
#include <algorithm>

#include "kernels.h"

namespace trot {

// ---------------------------------------------------------------- batched complex GEMM
// C[b] = alpha op(A[b]) op(B[b]) + beta C[b]; op: 0 = X, 1 = X^T, 2 = X^H, 3 = conj(X).
struct ZBatch {
  int M, Nc, K;
  double2 alpha, beta;
  const double2* A; long long sA; int lda, opA;
  const double2* B; long long sB; int ldb, opB;
  double2* C; long long sC; int ldc;
};

__device__ __forceinline__ double2 ld_op(const double2* X, int ld, int op, int r, int c) {
  if (op == 0) return X[(size_t)r * ld + c];
  if (op == 1) return X[(size_t)c * ld + r];
  const double2 v = op == 2 ? X[(size_t)c * ld + r] : X[(size_t)r * ld + c];
  return cmk(v.x, -v.y);
}

// Tile 32 x BN, K chunks of 16, 8 * BN threads; thread (ty, tx) owns rows ty + 8 r (r < 4) of column tx.
// BN = 16 for the skinny per-walker products (n columns), 32 otherwise.
template <int BN>
__global__ void __launch_bounds__(8 * BN) zgemm_batched_kernel(ZBatch z) {
  constexpr int NT = 8 * BN;
  __shared__ double2 As[32][17], Bs[16][BN + 1];
  const int b = blockIdx.z;
  const int m0 = blockIdx.y * 32, n0 = blockIdx.x * BN;
  const int tx = threadIdx.x % BN, ty = threadIdx.x / BN;
  const double2* A = z.A + (size_t)b * z.sA;
  const double2* B = z.B + (size_t)b * z.sB;
  double2 acc[4] = {cmk(0.0, 0.0), cmk(0.0, 0.0), cmk(0.0, 0.0), cmk(0.0, 0.0)};
  for (int k0 = 0; k0 < z.K; k0 += 16) {
    for (int e = threadIdx.x; e < 32 * 16; e += NT) {
      const int r = e >> 4, c = e & 15, m = m0 + r, k = k0 + c;
      As[r][c] = (m < z.M && k < z.K) ? ld_op(A, z.lda, z.opA, m, k) : cmk(0.0, 0.0);
    }
    for (int e = threadIdx.x; e < 16 * BN; e += NT) {
      const int r = e / BN, c = e % BN, k = k0 + r, n = n0 + c;
      Bs[r][c] = (k < z.K && n < z.Nc) ? ld_op(B, z.ldb, z.opB, k, n) : cmk(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < 16; ++k) {
      const double2 bv = Bs[k][tx];
#pragma unroll
      for (int r = 0; r < 4; ++r) cfma(acc[r], As[ty + 8 * r][k], bv);
    }
    __syncthreads();
  }
  double2* C = z.C + (size_t)b * z.sC;
  const bool use_beta = z.beta.x != 0.0 || z.beta.y != 0.0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int m = m0 + ty + 8 * r, n = n0 + tx;
    if (m < z.M && n < z.Nc) {
      double2 v = cmul(z.alpha, acc[r]);
      if (use_beta) v = cadd(v, cmul(z.beta, C[(size_t)m * z.ldc + n]));
      C[(size_t)m * z.ldc + n] = v;
    }
  }
}

static int zgemm_batched(int batch, int M, int Nc, int K, double2 alpha, const double2* A, long long sA, int lda,
                         int opA, const double2* B, long long sB, int ldb, int opB, double2 beta, double2* C,
                         long long sC, int ldc, cudaStream_t st) {
  ZBatch z{M, Nc, K, alpha, beta, A, sA, lda, opA, B, sB, ldb, opB, C, sC, ldc};
  if (Nc <= 16) {
    zgemm_batched_kernel<16><<<dim3(1, (M + 31) / 32, batch), 128, 0, st>>>(z);
  } else {
    zgemm_batched_kernel<32><<<dim3((Nc + 31) / 32, (M + 31) / 32, batch), 256, 0, st>>>(z);
  }
  TROT_CHECK_LAUNCH("zgemm_batched_kernel");
  return TROT_OK;
}

static int grid_of_(size_t len) { return (int)((len + 255) / 256 < 4096 ? (len + 255) / 256 : 4096); }

// ---------------------------------------------------------------- per-walker small kernels
// O = C^T w, P = O^-1, G = (w P)^T (n x N), det(O); one block per walker (n <= 32).
__global__ void adj_green_kernel(int N, int n, const double* __restrict__ C, const double2* __restrict__ w,
                                 double2* __restrict__ green, double2* __restrict__ Pout, double2* __restrict__ det) {
  __shared__ double2 O[32 * 32], P[32 * 32];
  __shared__ int piv;
  __shared__ double2 red[32];
  const int b = blockIdx.x, tid = threadIdx.x;
  const double2* wb = w + (size_t)b * N * n;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int p = 0; p < N; ++p) crfma(acc, C[(size_t)p * n + i], wb[(size_t)p * n + j]);
    O[i * n + j] = acc;
  }
  __syncthreads();
  const double2 d = block_gauss_jordan(O, n, n, P, &piv, red);
  __syncthreads();
  for (int e = tid; e < n * N; e += blockDim.x) {
    const int j = e / N, p = e % N;  // G[j][p] = sum_k w[p][k] P[k][j]
    double2 acc = cmk(0.0, 0.0);
    for (int k = 0; k < n; ++k) cfma(acc, wb[(size_t)p * n + k], P[k * n + j]);
    green[(size_t)b * n * N + e] = acc;
  }
  for (int e = tid; e < n * n; e += blockDim.x) Pout[(size_t)b * n * n + e] = P[e];
  if (tid == 0) det[b] = d;
}

// g_w[p][j] += mult kappa_b sum_i C[p][i] conj(P[j][i]) for ov = prod_s det(O_s)^mult_s,
// kappa = conj(ov) g_ov (d ov / d w_s = mult_s ov (C_s P_s^T))
__global__ void adj_overlap_kernel(int N, int n, double mult, const double* __restrict__ C,
                                   const double2* __restrict__ P, const double2* __restrict__ kappa,
                                   double2* __restrict__ gw) {
  const int b = blockIdx.x;
  const double2 kb = cscale(kappa[b], mult);
  const double2* Pb = P + (size_t)b * n * n;
  for (int e = threadIdx.x; e < N * n; e += blockDim.x) {
    const int p = e / n, j = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int i = 0; i < n; ++i) {
      const double2 pj = Pb[j * n + i];
      crfma(acc, C[(size_t)p * n + i], cmk(pj.x, -pj.y));
    }
    double2& o = gw[(size_t)b * N * n + e];
    o = cadd(o, cmul(kb, acc));
  }
}

// kappa_b = conj(ov_b) g_ov_b (zero for a zero cotangent)
__global__ void adj_kappa_kernel(int W, const double2* __restrict__ ov, const double2* __restrict__ gov,
                                 double2* __restrict__ kappa) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W) return;
  const double2 o = ov[b], g = gov[b];
  kappa[b] = (g.x == 0.0 && g.y == 0.0) ? cmk(0.0, 0.0) : cmul(cmk(o.x, -o.y), g);
}

// ov = prod_s det_s^mult_s (up to two spins; det1 may be null)
__global__ void adj_ov_kernel(int W, const double2* __restrict__ det0, int m0, const double2* __restrict__ det1, int m1,
                              double2* __restrict__ ov) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W) return;
  double2 o = det0[b];
  if (m0 == 2) o = cmul(o, o);
  if (det1) o = cmul(o, m1 == 2 ? cmul(det1[b], det1[b]) : det1[b]);
  ov[b] = o;
}

// g_w += (g_Gt - C X) P^H with X = Gt^H g_Gt (n x n); Gt = G^T, g_Gt = g_G^T.
// Dynamic shared memory: X and P (2 n^2 complex).
__global__ void adj_green_vjp_kernel(int N, int n, const double* __restrict__ C, const double2* __restrict__ green,
                                     const double2* __restrict__ ggreen, const double2* __restrict__ P,
                                     double2* __restrict__ gw) {
  extern __shared__ double2 sm[];
  double2* X = sm;
  double2* Ps = sm + n * n;
  const int b = blockIdx.x, tid = threadIdx.x;
  const double2* Gb = green + (size_t)b * n * N;
  const double2* gG = ggreen + (size_t)b * n * N;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int p = 0; p < N; ++p) {
      const double2 g = Gb[(size_t)i * N + p];
      cfma(acc, cmk(g.x, -g.y), gG[(size_t)j * N + p]);
    }
    X[e] = acc;
    Ps[e] = P[(size_t)b * n * n + e];
  }
  __syncthreads();
  double2* out = gw + (size_t)b * N * n;
  for (int e = tid; e < N * n; e += blockDim.x) {
    const int p = e / n, k = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int j = 0; j < n; ++j) {
      double2 y = gG[(size_t)j * N + p];
      for (int i = 0; i < n; ++i) crfma(y, -C[(size_t)p * n + i], X[i * n + j]);
      const double2 pk = Ps[k * n + j];
      cfma(acc, y, cmk(pk.x, -pk.y));
    }
    out[e] = cadd(out[e], acc);
  }
}

// QR: g_w = g_Q (w^H Q)^-1 per walker (n <= 32)
__global__ void adj_qr_kernel(int N, int n, const double2* __restrict__ w, const double2* __restrict__ q,
                              const double2* __restrict__ gq, double2* __restrict__ gw) {
  __shared__ double2 M[32 * 32], Mi[32 * 32];
  __shared__ int piv;
  __shared__ double2 red[32];
  const int b = blockIdx.x, tid = threadIdx.x;
  const double2* wb = w + (size_t)b * N * n;
  const double2* qb = q + (size_t)b * N * n;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int p = 0; p < N; ++p) {
      const double2 x = wb[(size_t)p * n + i];
      cfma(acc, cmk(x.x, -x.y), qb[(size_t)p * n + j]);
    }
    M[e] = acc;
  }
  __syncthreads();
  block_gauss_jordan(M, n, n, Mi, &piv, red);
  __syncthreads();
  const double2* g = gq + (size_t)b * N * n;
  // a walker with a zero cotangent (no influence on the objective) gets exactly zero
  int nz = 0;
  for (int e = tid; e < N * n; e += blockDim.x) nz |= (g[e].x != 0.0 || g[e].y != 0.0);
  if (!__syncthreads_or(nz)) {
    for (int e = tid; e < N * n; e += blockDim.x) gw[(size_t)b * N * n + e] = cmk(0.0, 0.0);
    return;
  }
  for (int e = tid; e < N * n; e += blockDim.x) {
    const int p = e / n, k = e % n;
    double2 acc = cmk(0.0, 0.0);
    for (int j = 0; j < n; ++j) cfma(acc, g[(size_t)p * n + j], Mi[j * n + k]);
    gw[(size_t)b * N * n + e] = acc;
  }
}

// part[z][p][q] = Re sum_{b in chunk z} sum_j a[b][p][j] conj(c[b][q][j]); grid (q tiles, p tiles, chunks
// of wchunk walkers), 256 threads.  The chunk partials are summed in order by adj_outer_reduce_kernel.
__global__ void __launch_bounds__(256) adj_outer_part_kernel(int W, int N, int n, int wchunk,
                                                             const double2* __restrict__ a,
                                                             const double2* __restrict__ c, double* __restrict__ part) {
  __shared__ double2 As[32][33], Cs[32][33];
  const int q0 = blockIdx.x * 32, p0 = blockIdx.y * 32, z = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const int b0 = z * wchunk, b1 = min(W, b0 + wchunk);
  for (int b = b0; b < b1; ++b) {
    for (int j0 = 0; j0 < n; j0 += 32) {
      for (int e = threadIdx.x; e < 32 * 32; e += 256) {
        const int r = e >> 5, j = e & 31;
        const bool ok = j0 + j < n;
        As[r][j] = (ok && p0 + r < N) ? a[((size_t)b * N + p0 + r) * n + j0 + j] : cmk(0.0, 0.0);
        Cs[r][j] = (ok && q0 + r < N) ? c[((size_t)b * N + q0 + r) * n + j0 + j] : cmk(0.0, 0.0);
      }
      __syncthreads();
      const int jn = min(32, n - j0);
      for (int j = 0; j < jn; ++j) {
        const double2 cv = Cs[tx][j];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const double2 av = As[ty + 8 * r][j];
          acc[r] = fma(av.x, cv.x, fma(av.y, cv.y, acc[r]));  // Re(a conj(c))
        }
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int p = p0 + ty + 8 * r, q = q0 + tx;
    if (p < N && q < N) part[((size_t)z * N + p) * N + q] = acc[r];
  }
}

__global__ void adj_outer_reduce_kernel(int NN, int Z, const double* __restrict__ part, double* __restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < NN; e += gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int z = 0; z < Z; ++z) v += part[(size_t)z * NN + e];
    out[e] += v;
  }
}

static constexpr int kOuterChunks = 64;

// out (N x N) += Re sum_b a_b c_b^H over walkers, a_b, c_b (N x n)
static int outer_sum(int W, int N, int n, const double2* a, const double2* c, double* part, double* out,
                     cudaStream_t st) {
  const int wchunk = (W + kOuterChunks - 1) / kOuterChunks;
  const int Z = (W + wchunk - 1) / wchunk;
  adj_outer_part_kernel<<<dim3((N + 31) / 32, (N + 31) / 32, Z), 256, 0, st>>>(W, N, n, wchunk, a, c, part);
  TROT_CHECK_LAUNCH("adj_outer_part_kernel");
  const int NN = N * N;
  adj_outer_reduce_kernel<<<(NN + 255) / 256, 256, 0, st>>>(NN, Z, part, out);
  TROT_CHECK_LAUNCH("adj_outer_reduce_kernel");
  return TROT_OK;
}

// out = sum_t coef[t] x[t] over nx vectors of length len (complex coefficients)
struct Comb {
  int nx;
  double2 coef[8];
  const double2* x[8];
};
__global__ void adj_combine_kernel(size_t len, Comb cb, double2* __restrict__ out, int accumulate) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x) {
    double2 v = accumulate ? out[e] : cmk(0.0, 0.0);
    for (int t = 0; t < cb.nx; ++t) cfma(v, cb.coef[t], cb.x[t][e]);
    out[e] = v;
  }
}

static int combine(size_t len, const Comb& cb, double2* out, bool accumulate, cudaStream_t st) {
  const int blocks = (int)((len + 255) / 256 < 4096 ? (len + 255) / 256 : 4096);
  adj_combine_kernel<<<blocks, 256, 0, st>>>(len, cb, out, accumulate ? 1 : 0);
  TROT_CHECK_LAUNCH("adj_combine_kernel");
  return TROT_OK;
}

// Walkers that cannot influence the objective (zero weight before the step, or
// a weight the step's guards set to zero; zero energy / overlap cotangent) get
// exactly zero cotangents: their recomputed data, which may be non-finite, is
// replaced by zeros so that no 0 * inf enters a sum over walkers.
__global__ void adj_zero_inactive_kernel(int W, size_t per, const int* __restrict__ act, double2* __restrict__ x) {
  const size_t total = (size_t)W * per;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    if (!act[e / per]) x[e] = cmk(0.0, 0.0);
}

// act[b] = (g[b] != 0) for a real or complex per-walker cotangent
__global__ void adj_act_from_cotangent_kernel(int W, const double* __restrict__ g, int complex_g, int* __restrict__ act) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W) return;
  act[b] = complex_g ? (g[2 * b] != 0.0 || g[2 * b + 1] != 0.0) : (g[b] != 0.0);
}

static int zero_inactive(int W, size_t per, const int* act, double2* x, cudaStream_t st) {
  adj_zero_inactive_kernel<<<grid_of_(W * per), 256, 0, st>>>(W, per, act, x);
  TROT_CHECK_LAUNCH("adj_zero_inactive_kernel");
  return TROT_OK;
}

// ---------------------------------------------------------------- step: scalar forward + backward per walker
struct StepScalars {
  double2 ov_old, ov_new, st, ft;
  double wt_old, e_shift, dt, sqrt_dt, h0_prop, w_floor, w_cap;
};

// imp_ph and its mask exactly as the forward (phaseless_update)
__device__ __forceinline__ double imp_forward(const StepScalars& s, double* E_out, double2* rot_out, bool* live) {
  const double2 ratio = cdiv(s.ov_new, s.ov_old);
  const double2 expo = cadd(cadd(cscale(s.st, -s.sqrt_dt), s.ft), cmk(s.dt * (s.e_shift + s.h0_prop), 0.0));
  const double2 imp = cmul(cexp(expo), ratio);
  const double2 ph = cmul(cexp(cscale(s.st, -s.sqrt_dt)), ratio);
  const double theta = atan2(ph.y, ph.x);
  double imp_ph = hypot(imp.x, imp.y) * cos(theta);
  bool ok = true;
  if (!isfinite(imp_ph) || imp_ph < s.w_floor) { imp_ph = 0.0; ok = false; }
  if (imp_ph > s.w_cap) { imp_ph = 0.0; ok = false; }
  double wn = s.wt_old * imp_ph;
  if (wn > s.w_cap) { wn = 0.0; ok = false; }
  *E_out = exp(expo.x);
  // rho e^{ic}, c = Im(-sqrt(dt) st)
  const double c = -s.sqrt_dt * s.st.y;
  *rot_out = cmul(ratio, cmk(cos(c), sin(c)));
  *live = ok;
  return imp_ph;
}

// weights after the step (for the population-control mean)
__global__ void adj_step_fwd_kernel(int W, const double2* __restrict__ ov_old, const double2* __restrict__ ov_new,
                                    const double2* __restrict__ st, const double2* __restrict__ ft,
                                    const double* __restrict__ wt, const double* __restrict__ scal, double dt,
                                    double sqrt_dt, double h0_prop, double w_floor, double w_cap,
                                    double* __restrict__ wt_new, int* __restrict__ act) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W) return;
  StepScalars s{ov_old[b], ov_new[b], st[b], ft[b], wt[b], scal[0], dt, sqrt_dt, h0_prop, w_floor, w_cap};
  double E;
  double2 r;
  bool live;
  const double ip = imp_forward(s, &E, &r, &live);
  wt_new[b] = live ? wt[b] * ip : 0.0;
  act[b] = (live && wt[b] != 0.0) ? 1 : 0;
}

// fixed-order sum of x[0..n) into out[0] (one block)
__global__ void adj_sum_kernel(int n, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double2 red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += x[i];
  const double2 t = block_sum2(cmk(acc, 0.0), red);
  if (threadIdx.x == 0) out[0] = t.x;
}

__global__ void adj_scalar_tail_kernel(const double* __restrict__ g_out, double* __restrict__ g_in) {
  g_in[1] = g_out[1] + g_out[0];
}

// Per-walker backward of the weight update.  In: g_wt', g_ov', g_scalars' = [g_Es', g_ee'], sum of wt'.
// Out: g_wt, g_ov (old), kappa' = 2 conj(ov') g_ov'_total, per-walker g_st (real), g_c, g_Req, dt g_Req (for g_Es).
__global__ void adj_step_bwd_kernel(int W, const double2* __restrict__ ov_old, const double2* __restrict__ ov_new,
                                    const double2* __restrict__ st, const double2* __restrict__ ft,
                                    const double* __restrict__ wt, const double* __restrict__ scal, double dt,
                                    double sqrt_dt, double h0_prop, double w_floor, double w_cap, double damping,
                                    const double* __restrict__ wsum, const double* __restrict__ g_wt_new,
                                    const double2* __restrict__ g_ov_new, const double* __restrict__ g_scal_new,
                                    double* __restrict__ g_wt, double2* __restrict__ g_ov, double2* __restrict__ kappa,
                                    double* __restrict__ g_req, double* __restrict__ g_c, double* __restrict__ g_es) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= W) return;
  const double2 ovn = ov_new[b];
  StepScalars s{ov_old[b], ovn, st[b], ft[b], wt[b], scal[0], dt, sqrt_dt, h0_prop, w_floor, w_cap};
  double E;
  double2 r;
  bool live;
  const double ip = imp_forward(s, &E, &r, &live);
  // E_shift' = e_est - damping log(max(mean wt', 1e-300)) / dt
  const double mean = wsum[0] / W;
  double gw_new = g_wt_new ? g_wt_new[b] : 0.0;
  if (mean > 1e-300) gw_new += g_scal_new[0] * (-damping / dt) / (mean * W);
  const double g_imp = live ? gw_new * wt[b] : 0.0;
  g_wt[b] = live ? gw_new * ip : 0.0;
  const double greq = g_imp * ip;  // d imp_ph / d Re q = imp_ph
  // imp_ph = E Re(rho e^{ic}): g_rho = g_imp E e^{-ic}, g_c = -g_imp E Im(rho e^{ic})
  const double c = -sqrt_dt * s.st.y;
  const double2 emic = cmk(cos(c), -sin(c));
  const double2 grho = cscale(emic, g_imp * E);
  const double gc = -g_imp * E * r.y;
  const double2 rho = cdiv(ovn, s.ov_old);
  double2 gov_new = g_ov_new ? g_ov_new[b] : cmk(0.0, 0.0);
  const double2 inv_old = cdiv(cmk(1.0, 0.0), s.ov_old);
  gov_new = cadd(gov_new, cmul(cmk(inv_old.x, -inv_old.y), grho));
  const double2 rq = cmul(rho, inv_old);
  const bool active = live && wt[b] != 0.0;
  g_ov[b] = active ? cscale(cmul(cmk(rq.x, -rq.y), grho), -1.0) : cmk(0.0, 0.0);
  kappa[b] = active ? cmul(cmk(ovn.x, -ovn.y), gov_new) : cmk(0.0, 0.0);  // times mult_s per spin
  g_req[b] = active ? greq : 0.0;
  g_c[b] = active ? gc : 0.0;
  g_es[b] = active ? dt * greq : 0.0;
}

// g_fb[b][g] from g_xs^V and the per-walker scalars (see header): xs = x - fs, fs = -i sqrt(dt) (fb - m),
// st = i sum xs m, ft = sum (x fs - fs^2 / 2), c = -sqrt(dt) Re(sum xs m).
__global__ void adj_fields_kernel(int W, int G, double sqrt_dt, const double* __restrict__ mf_im,
                                  const double2* __restrict__ xs, const double2* __restrict__ gxsv,
                                  const double* __restrict__ g_req, const double* __restrict__ g_c,
                                  double2* __restrict__ gfb) {
  const size_t total = (size_t)W * G;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(e / G), g = (int)(e % G);
    const double m = mf_im[g];
    const double greq = g_req[b];
    const double gst = -sqrt_dt * greq;  // g_st (real): Re q = -sqrt(dt) Re st + ...
    const double2 gv = gxsv[e];
    const double2 gxs = cmk(gv.x - sqrt_dt * m * g_c[b], gv.y - m * gst);
    const double2 x = xs[e];
    const double2 gfs = csub(cscale(cmk(x.x, -x.y), greq), gxs);
    gfb[e] = cscale(cmk(-gfs.y, gfs.x), sqrt_dt);  // i sqrt(dt) g_fs
  }
}

// ---------------------------------------------------------------- local energy pieces
// c[b][g] = sum_i F[b n + i][g n + i]
__global__ void adj_trace_kernel(int W, int G, int n, const double2* __restrict__ F, double2* __restrict__ c) {
  const size_t total = (size_t)W * G;
  const size_t ld = (size_t)G * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / G, g = e % G;
    double2 acc = cmk(0.0, 0.0);
    for (int i = 0; i < n; ++i) acc = cadd(acc, F[(b * n + i) * ld + g * n + i]);
    c[e] = acc;
  }
}

// Ft[b n + i][g n + j] = F[b n + j][g n + i]
__global__ void adj_block_transpose_kernel(int W, int G, int n, const double2* __restrict__ F,
                                           double2* __restrict__ Ft) {
  const size_t ld = (size_t)G * n;
  const size_t total = (size_t)W * n * ld;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t row = e / ld, col = e % ld;
    const size_t b = row / n, i = row % n, g = col / n, j = col % n;
    Ft[e] = F[(b * n + j) * ld + g * n + i];
  }
}

// g_G[b][i][p] = g_E[b] conj(mult rot_h1[i][p] + D[b][i][p])
__global__ void adj_energy_green_kernel(int W, int n, int N, double mult, const double* __restrict__ rot_h1,
                                        const double2* __restrict__ D, const double* __restrict__ gE,
                                        double2* __restrict__ gG) {
  const size_t per = (size_t)n * N, total = (size_t)W * per;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / per, k = e % per;
    const double2 d = D[e];
    gG[e] = cscale(cmk(mult * rot_h1[k] + d.x, -d.y), gE[b]);
  }
}

// H[i][p] = sum_b gE[b] G[b][i][p]  (fixed order over b)
__global__ void adj_weighted_green_kernel(int W, int n, int N, const double2* __restrict__ G,
                                          const double* __restrict__ gE, double2* __restrict__ H) {
  const size_t per = (size_t)n * N;
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < per; k += (size_t)gridDim.x * blockDim.x) {
    double2 acc = cmk(0.0, 0.0);
    for (int b = 0; b < W; ++b) acc = cadd(acc, cscale(G[(size_t)b * per + k], gE[b]));
    H[k] = acc;
  }
}

// g_h1[q][p] += mult Re sum_i C[q][i] H[i][p]
__global__ void adj_h1_direct_kernel(int N, int n, double mult, const double* __restrict__ C,
                                     const double2* __restrict__ H, double* __restrict__ gh1) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)N * N; e += (size_t)gridDim.x * blockDim.x) {
    const int q = (int)(e / N), p = (int)(e % N);
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += C[(size_t)q * n + i] * H[(size_t)i * N + p].x;
    gh1[e] += mult * acc;
  }
}

// complex copy of a real matrix
__global__ void adj_to_complex_kernel(size_t len, const double* __restrict__ x, double2* __restrict__ y) {
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < len; e += (size_t)gridDim.x * blockDim.x)
    y[e] = cmk(x[e], 0.0);
}

static int grid_of(size_t len) { return (int)((len + 255) / 256 < 4096 ? (len + 255) / 256 : 4096); }

// ---------------------------------------------------------------- workspace layouts
// Spins: TROT_RHF_R has one spin with multiplicity 2; TROT_RHF_U and TROT_UHF_U two spins
// with multiplicity 1 (RHF_U uses the alpha trial and rotated integrals for both).
struct AdjCommon {
  int W, N, G, K, nspin;
  int n[2], mult[2];
  size_t wn[2], nN[2];
  const double* mo[2];
  const double* rot_h1[2];
  const double* rot_chol[2];
  const double* chol_packed;  // packed upper triangle of the Cholesky vectors, or null
};

static int check_adj(const trot_system* s) {
  if (!s) { set_error("null system"); return TROT_ERR_NULL_PTR; }
  if (s->kind != TROT_RHF_R && s->kind != TROT_RHF_U && s->kind != TROT_UHF_U) {
    set_error("bad kind %d", s->kind);
    return TROT_ERR_BAD_SHAPE;
  }
  if (s->precision != TROT_FP64) { set_error("the adjoint runs in FP64"); return TROT_ERR_UNSUPPORTED; }
  const int nb = s->kind == TROT_RHF_R ? s->nocc_a : s->nocc_b;
  if (s->n_walkers < 1 || s->n_walkers > 65535 || s->norb < 1 || s->nchol < 1 || s->nocc_a < 1 || s->nocc_a > 32 ||
      s->nocc_a > s->norb || nb < 1 || nb > 32 || nb > s->norb) {
    set_error("bad shape: W %d (<= 65535), N %d, G %d, n %d / %d (<= 32)", s->n_walkers, s->norb, s->nchol, s->nocc_a,
              nb);
    return TROT_ERR_BAD_SHAPE;
  }
  if (s->n_exp_terms < 1 || s->n_exp_terms > 7) { set_error("n_exp_terms %d outside 1..7", s->n_exp_terms); return TROT_ERR_BAD_SHAPE; }
  if (!s->mo_a || (s->kind == TROT_UHF_U && !s->mo_b)) { set_error("null trial"); return TROT_ERR_NULL_PTR; }
  return TROT_OK;
}

static AdjCommon common_of(const trot_system* s) {
  AdjCommon a{};
  a.W = s->n_walkers; a.N = s->norb; a.G = s->nchol; a.K = s->n_exp_terms;
  const bool uhf = s->kind == TROT_UHF_U;
  a.nspin = s->kind == TROT_RHF_R ? 1 : 2;
  for (int q = 0; q < a.nspin; ++q) {
    a.n[q] = q == 0 ? s->nocc_a : s->nocc_b;
    a.mult[q] = a.nspin == 1 ? 2 : 1;
    a.wn[q] = (size_t)a.W * a.N * a.n[q];
    a.nN[q] = (size_t)a.n[q] * a.N;
    a.mo[q] = (q == 1 && uhf) ? s->mo_b : s->mo_a;
    a.rot_h1[q] = (q == 1 && uhf) ? s->rot_h1_b : s->rot_h1_a;
    a.rot_chol[q] = (q == 1 && uhf) ? s->rot_chol_b : s->rot_chol_a;
  }
  a.chol_packed = s->chol_packed;
  return a;
}

struct SpinWs {  // per-spin buffers of the step adjoint
  double2 *green, *P, *det, *U, *w2, *wnew, *greenn, *Pn, *detn, *gwn, *gw2, *Vv, *S, *gG, *gw1, *wz;
};
struct StepWs {
  SpinWs sp[2];
  double2 *fb, *xs, *st, *ft, *V, *Bc, *gV, *gxsv, *gfb, *kappa, *ov_new;
  double2* vp;  // packed VHS, then the packed cotangent g_V + g_V^T (W, N(N+1)/2), with chol_packed
  double *wt_new, *wsum, *g_req, *g_c, *g_es, *opart;
  double2* kpart;  // split-K partials of the long-K products
  int* act;
};

static int splitk_slices(int M, int Nn) {  // enough CTAs for two per SM
  const int base = ((Nn + 63) / 64) * ((M + 63) / 64);
  int S = (2 * 152 + base - 1) / base;
  return S < 1 ? 1 : (S > 16 ? 16 : S);
}

static void carve_step(const AdjCommon& a, Carver& c, StepWs& b) {
  const size_t W = a.W, G = a.G, NN = (size_t)a.N * a.N;
  b = StepWs{};
  for (int q = 0; q < a.nspin; ++q) {
    SpinWs& x = b.sp[q];
    const size_t wn = a.wn[q], n = a.n[q];
    x.green = c.take<double2>(W * a.nN[q]);
    x.P = c.take<double2>(W * n * n);
    x.det = c.take<double2>(W);
    x.U = c.take<double2>((size_t)(a.K + 1) * wn);
    x.w2 = c.take<double2>(wn);
    x.wnew = c.take<double2>(wn);
    x.greenn = c.take<double2>(W * a.nN[q]);
    x.Pn = c.take<double2>(W * n * n);
    x.detn = c.take<double2>(W);
    x.gwn = c.take<double2>(wn);
    x.gw2 = c.take<double2>(wn);
    x.Vv = c.take<double2>((size_t)(a.K + 1) * wn);
    x.S = c.take<double2>((size_t)a.K * wn);
    x.gG = c.take<double2>(W * a.nN[q]);
    x.gw1 = c.take<double2>(wn);
    x.wz = c.take<double2>(wn);
  }
  b.fb = c.take<double2>(W * G);
  b.xs = c.take<double2>(W * G);
  b.st = c.take<double2>(W);
  b.ft = c.take<double2>(W);
  b.V = c.take<double2>(W * NN);
  b.Bc = c.take<double2>(NN);
  b.gV = c.take<double2>(W * NN);
  if (a.chol_packed) b.vp = c.take<double2>(W * ((size_t)a.N * (a.N + 1) / 2));
  b.gxsv = c.take<double2>(W * G);
  b.gfb = c.take<double2>(W * G);
  b.kappa = c.take<double2>(W);
  b.ov_new = c.take<double2>(W);
  b.wt_new = c.take<double>(W);
  b.wsum = c.take<double>(1);
  b.g_req = c.take<double>(W);
  b.g_c = c.take<double>(W);
  b.g_es = c.take<double>(W);
  b.opart = c.take<double>((size_t)kOuterChunks * NN);
  size_t kp = (size_t)splitk_slices(a.W, a.G) * W * G;
  for (int q = 0; q < a.nspin; ++q) kp = std::max(kp, (size_t)splitk_slices(a.W, a.G) * W * G);
  b.kpart = c.take<double2>(kp);
  b.act = c.take<int>(W);
}

struct EnergyWs {
  double2 *green[2], *P[2], *det, *F, *Ft, *c[2], *ctot, *D, *gG, *H;
  int* act;
};

static void carve_energy(const AdjCommon& a, Carver& c, EnergyWs& b) {
  const size_t W = a.W, G = a.G;
  b = EnergyWs{};
  size_t nmax = 0, nNmax = 0;
  for (int q = 0; q < a.nspin; ++q) {
    b.green[q] = c.take<double2>(W * a.nN[q]);
    b.P[q] = c.take<double2>(W * a.n[q] * a.n[q]);
    b.c[q] = c.take<double2>(W * G);
    nmax = std::max(nmax, (size_t)a.n[q]);
    nNmax = std::max(nNmax, a.nN[q]);
  }
  b.det = c.take<double2>(W);
  b.F = c.take<double2>(W * nmax * G * nmax);
  b.Ft = c.take<double2>(W * nmax * G * nmax);
  b.ctot = c.take<double2>(W * G);
  b.D = c.take<double2>(W * nNmax);
  b.gG = c.take<double2>(W * nNmax);
  b.H = c.take<double2>(nNmax);
  b.act = c.take<int>(W);
}

static int green_launch(const AdjCommon& a, int q, const double2* w, double2* green, double2* P, double2* det,
                        cudaStream_t st) {
  adj_green_kernel<<<a.W, 256, 0, st>>>(a.N, a.n[q], a.mo[q], w, green, P, det);
  TROT_CHECK_LAUNCH("adj_green_kernel");
  return TROT_OK;
}

static int green_vjp_launch(const AdjCommon& a, int q, const double2* green, const double2* ggreen, const double2* P,
                            double2* gw, cudaStream_t st) {
  const size_t smem = (size_t)2 * a.n[q] * a.n[q] * sizeof(double2);
  adj_green_vjp_kernel<<<a.W, 256, smem, st>>>(a.N, a.n[q], a.mo[q], green, ggreen, P, gw);
  TROT_CHECK_LAUNCH("adj_green_vjp_kernel");
  return TROT_OK;
}

static int ov_launch(const AdjCommon& a, const double2* d0, const double2* d1, double2* ov, cudaStream_t st) {
  adj_ov_kernel<<<(a.W + 127) / 128, 128, 0, st>>>(a.W, d0, a.mult[0], a.nspin == 2 ? d1 : nullptr,
                                                    a.nspin == 2 ? a.mult[1] : 0, ov);
  TROT_CHECK_LAUNCH("adj_ov_kernel");
  return TROT_OK;
}

static int dcopy(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
  return e == cudaSuccess ? TROT_OK : cuda_status(e, "adjoint copy");
}

}  // namespace trot

using namespace trot;

extern "C" {

size_t trot_vjp_workspace_size(const trot_system* s, int op) {
  if (check_adj(s) != TROT_OK) return 0;
  const AdjCommon a = common_of(s);
  Carver c(nullptr, 0);
  if (op == TROT_OP_PROP_STEP) {
    StepWs b;
    carve_step(a, c, b);
  } else if (op == TROT_OP_LOCAL_ENERGY) {
    EnergyWs b;
    carve_energy(a, c, b);
  } else if (op == TROT_OP_OVERLAP) {
    for (int q = 0; q < a.nspin; ++q) {
      c.take<double2>(a.W * a.nN[q]);
      c.take<double2>((size_t)a.W * a.n[q] * a.n[q]);
      c.take<double2>(a.W);
    }
    c.take<double2>((size_t)3 * a.W);  // ov, kappa, walker flags
  } else if (op == TROT_OP_QR) {
    return 256;
  } else {
    set_error("no adjoint for op %d", op);
    return 0;
  }
  return c.used + 256;
}

int trot_prop_step_vjp(const trot_system* s, const trot_state* in, const double* fields, const double* g_walkers_out_a,
                       const double* g_walkers_out_b, const double* g_weights_out, const double* g_overlaps_out,
                       const double* g_scalars_out, double* g_walkers_in_a, double* g_walkers_in_b,
                       double* g_weights_in, double* g_overlaps_in, double* g_scalars_in, double* g_exp_h1_half,
                       void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_adj(s));
  const AdjCommon a = common_of(s);
  const bool two = a.nspin == 2;
  if (!in || !in->walkers_a || (two && !in->walkers_b) || !in->weights || !in->overlaps || !in->scalars || !fields ||
      !g_walkers_out_a || (two && !g_walkers_out_b) || !g_scalars_out || !g_walkers_in_a ||
      (two && !g_walkers_in_b) || !g_weights_in || !g_overlaps_in || !g_scalars_in || !g_exp_h1_half || !ws) {
    set_error("null state, fields, cotangent or workspace");
    return TROT_ERR_NULL_PTR;
  }
  if (!a.rot_chol[0] || (two && !a.rot_chol[1]) || !s->exp_h1_half || !s->chol_flat || !s->mf_shifts_im) {
    set_error("null measurement or propagation context");
    return TROT_ERR_NULL_PTR;
  }
  Carver c(ws, ws_bytes);
  StepWs b;
  carve_step(a, c, b);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  const int W = a.W, N = a.N, G = a.G, K = a.K;
  const size_t NN = (size_t)N * N;
  const double2 one = cmk(1.0, 0.0), zero = cmk(0.0, 0.0);
  const double2* w[2] = {(const double2*)in->walkers_a, (const double2*)in->walkers_b};
  const double2* gout[2] = {(const double2*)g_walkers_out_a, (const double2*)g_walkers_out_b};
  double2* gin[2] = {(double2*)g_walkers_in_a, (double2*)g_walkers_in_b};
  // ---------------- forward recompute
  for (int q = 0; q < a.nspin; ++q) {
    TROT_TRY(green_launch(a, q, w[q], b.sp[q].green, b.sp[q].P, b.sp[q].det, st));
    // fb = sum_s mult_s R_s . G_s
    TROT_TRY(launch_zgemm_cr_splitk(W, G, (int)a.nN[q], (double)a.mult[q], b.sp[q].green, (int)a.nN[q],
                                    a.rot_chol[q], (int)a.nN[q], true, b.fb, G, q > 0, b.kpart,
                                    splitk_slices(W, G), st));
  }
  TROT_TRY(launch_fields(W, G, s->sqrt_dt, b.fb, s->mf_shifts_im, fields, b.xs, b.st, b.ft, st));
  TROT_TRY(launch_vhs64(W, N, G, b.xs, s->chol_flat, a.chol_packed, b.vp, b.V, st));
  adj_to_complex_kernel<<<grid_of(NN), 256, 0, st>>>(NN, s->exp_h1_half, b.Bc);
  TROT_CHECK_LAUNCH("adj_to_complex_kernel");
  double2 ck[8];
  {  // c_k = (i sqrt(dt))^k / k!
    double2 t = one;
    ck[0] = one;
    for (int k = 1; k <= K; ++k) {
      t = cscale(cmul(t, cmk(0.0, s->sqrt_dt)), 1.0 / k);
      ck[k] = t;
    }
  }
  for (int q = 0; q < a.nspin; ++q) {
    SpinWs& x = b.sp[q];
    const int n = a.n[q];
    const long long sw = (long long)N * n;
    // u_0 = B w, u_{l+1} = V u_l, w2 = sum_k c_k u_k, w' = B w2
    TROT_TRY(zgemm_batched(W, N, n, N, one, b.Bc, 0, N, 0, w[q], sw, n, 0, zero, x.U, sw, n, st));
    for (int l = 0; l < K; ++l)
      TROT_TRY(zgemm_batched(W, N, n, N, one, b.V, (long long)NN, N, 0, x.U + (size_t)l * a.wn[q], sw, n, 0, zero,
                             x.U + (size_t)(l + 1) * a.wn[q], sw, n, st));
    Comb cb{};
    cb.nx = K + 1;
    for (int k = 0; k <= K; ++k) { cb.coef[k] = ck[k]; cb.x[k] = x.U + (size_t)k * a.wn[q]; }
    TROT_TRY(combine(a.wn[q], cb, x.w2, false, st));
    TROT_TRY(zgemm_batched(W, N, n, N, one, b.Bc, 0, N, 0, x.w2, sw, n, 0, zero, x.wnew, sw, n, st));
    TROT_TRY(green_launch(a, q, x.wnew, x.greenn, x.Pn, x.detn, st));
  }
  TROT_TRY(ov_launch(a, b.sp[0].detn, b.sp[1].detn, b.ov_new, st));
  const int wb = (W + 127) / 128;
  adj_step_fwd_kernel<<<wb, 128, 0, st>>>(W, (const double2*)in->overlaps, b.ov_new, b.st, b.ft, in->weights,
                                           in->scalars, s->dt, s->sqrt_dt, s->h0_prop, s->weight_floor, s->weight_cap,
                                           b.wt_new, b.act);
  TROT_CHECK_LAUNCH("adj_step_fwd_kernel");
  adj_sum_kernel<<<1, 256, 0, st>>>(W, b.wt_new, b.wsum);
  TROT_CHECK_LAUNCH("adj_sum_kernel");
  // inactive walkers: zero their recomputed data (see adj_zero_inactive_kernel)
  for (int q = 0; q < a.nspin; ++q) {
    SpinWs& x = b.sp[q];
    const size_t per = (size_t)N * a.n[q], nn = (size_t)a.n[q] * a.n[q];
    TROT_TRY(dcopy(x.wz, w[q], a.wn[q] * sizeof(double2), st));
    TROT_TRY(zero_inactive(W, per, b.act, x.wz, st));
    for (int l = 0; l <= K; ++l) TROT_TRY(zero_inactive(W, per, b.act, x.U + (size_t)l * a.wn[q], st));
    TROT_TRY(zero_inactive(W, per, b.act, x.w2, st));
    TROT_TRY(zero_inactive(W, a.nN[q], b.act, x.green, st));
    TROT_TRY(zero_inactive(W, nn, b.act, x.P, st));
    TROT_TRY(zero_inactive(W, nn, b.act, x.Pn, st));
  }
  TROT_TRY(zero_inactive(W, NN, b.act, b.V, st));
  TROT_TRY(zero_inactive(W, G, b.act, b.xs, st));
  // ---------------- backward
  adj_step_bwd_kernel<<<wb, 128, 0, st>>>(W, (const double2*)in->overlaps, b.ov_new, b.st, b.ft, in->weights,
                                           in->scalars, s->dt, s->sqrt_dt, s->h0_prop, s->weight_floor, s->weight_cap,
                                           s->pop_control_damping, b.wsum, g_weights_out,
                                           (const double2*)g_overlaps_out, g_scalars_out, g_weights_in,
                                           (double2*)g_overlaps_in, b.kappa, b.g_req, b.g_c, b.g_es);
  TROT_CHECK_LAUNCH("adj_step_bwd_kernel");
  // g_scalars_in = [sum_b dt g_req_b, g_ee' + g_Es'] (e_estimate passes through; E_shift' = e_est - ...)
  adj_scalar_tail_kernel<<<1, 1, 0, st>>>(g_scalars_out, g_scalars_in);
  TROT_CHECK_LAUNCH("adj_scalar_tail_kernel");
  adj_sum_kernel<<<1, 256, 0, st>>>(W, b.g_es, g_scalars_in);
  TROT_CHECK_LAUNCH("adj_sum_kernel");
  for (int q = 0; q < a.nspin; ++q) {
    SpinWs& x = b.sp[q];
    const int n = a.n[q];
    const long long sw = (long long)N * n;
    const size_t per = (size_t)N * n;
    // g_w' (incoming) + overlap term
    TROT_TRY(dcopy(x.gwn, gout[q], a.wn[q] * sizeof(double2), st));
    TROT_TRY(zero_inactive(W, per, b.act, x.gwn, st));
    adj_overlap_kernel<<<W, 256, 0, st>>>(N, n, (double)a.mult[q], a.mo[q], x.Pn, b.kappa, x.gwn);
    TROT_CHECK_LAUNCH("adj_overlap_kernel");
    // w' = B w2: g_B += Re sum g_w' w2^H; g_w2 = B^T g_w'
    TROT_TRY(outer_sum(W, N, n, x.gwn, x.w2, b.opart, g_exp_h1_half, st));
    TROT_TRY(zgemm_batched(W, N, n, N, one, b.Bc, 0, N, 1, x.gwn, sw, n, 0, zero, x.gw2, sw, n, st));
    // v_0 = g_w2, v_{j+1} = V^H v_j
    TROT_TRY(dcopy(x.Vv, x.gw2, a.wn[q] * sizeof(double2), st));
    for (int j = 0; j < K; ++j)
      TROT_TRY(zgemm_batched(W, N, n, N, one, b.V, (long long)NN, N, 2, x.Vv + (size_t)j * a.wn[q], sw, n, 0, zero,
                             x.Vv + (size_t)(j + 1) * a.wn[q], sw, n, st));
    // g_w1 = sum_k conj(c_k) v_k
    Comb cb{};
    cb.nx = K + 1;
    for (int k = 0; k <= K; ++k) { cb.coef[k] = cmk(ck[k].x, -ck[k].y); cb.x[k] = x.Vv + (size_t)k * a.wn[q]; }
    TROT_TRY(combine(a.wn[q], cb, x.gw1, false, st));
    // s_l = sum_{j <= K-1-l} conj(c_{j+l+1}) v_j;  g_V += sum_l s_l u_l^H (both spins share V)
    for (int l = 0; l < K; ++l) {
      Comb cs{};
      cs.nx = K - l;
      for (int j = 0; j < K - l; ++j) { cs.coef[j] = cmk(ck[j + l + 1].x, -ck[j + l + 1].y); cs.x[j] = x.Vv + (size_t)j * a.wn[q]; }
      TROT_TRY(combine(a.wn[q], cs, x.S + (size_t)l * a.wn[q], false, st));
      TROT_TRY(zgemm_batched(W, N, N, n, one, x.S + (size_t)l * a.wn[q], sw, n, 0, x.U + (size_t)l * a.wn[q], sw, n,
                             2, (q == 0 && l == 0) ? zero : one, b.gV, (long long)NN, N, st));
    }
    // w1 = B w: g_B += Re sum g_w1 w^H; g_w = B^T g_w1 (the Green's-function term is added below)
    TROT_TRY(outer_sum(W, N, n, x.gw1, x.wz, b.opart, g_exp_h1_half, st));
    TROT_TRY(zgemm_batched(W, N, n, N, one, b.Bc, 0, N, 1, x.gw1, sw, n, 0, zero, gin[q], sw, n, st));
  }
  // V = sum_g xs_g L_g: g_xs^V[b][g] = sum_pq L_g[pq] g_V[b][pq] (with symmetric L_g: over the packed
  // upper triangle of g_V + g_V^T, half the FP64 products)
  if (a.chol_packed) {
    const int P = N * (N + 1) / 2;
    TROT_TRY(launch_pack_sym(N, W, b.gV, b.vp, st));
    TROT_TRY(launch_zgemm_cr_splitk(W, G, P, 1.0, b.vp, P, a.chol_packed, P, true, b.gxsv, G, false, b.kpart,
                                    splitk_slices(W, G), st));
  } else {
    TROT_TRY(launch_zgemm_cr_splitk(W, G, (int)NN, 1.0, b.gV, (int)NN, s->chol_flat, (int)NN, true, b.gxsv, G,
                                    false, b.kpart, splitk_slices(W, G), st));
  }
  adj_fields_kernel<<<grid_of((size_t)W * G), 256, 0, st>>>(W, G, s->sqrt_dt, s->mf_shifts_im, b.xs, b.gxsv, b.g_req,
                                                             b.g_c, b.gfb);
  TROT_CHECK_LAUNCH("adj_fields_kernel");
  for (int q = 0; q < a.nspin; ++q) {
    SpinWs& x = b.sp[q];
    // fb = sum_s mult_s G_s R_s^T: g_G_s = mult_s g_fb R_s
    TROT_TRY(launch_zgemm_cr(W, (int)a.nN[q], G, (double)a.mult[q], b.gfb, G, a.rot_chol[q], (int)a.nN[q], false,
                             x.gG, (int)a.nN[q], false, st));
    TROT_TRY(green_vjp_launch(a, q, x.green, x.gG, x.P, gin[q], st));
  }
  return TROT_OK;
}

int trot_local_energy_vjp(const trot_system* s, const double* walkers_a, const double* walkers_b,
                          const double* g_energy, double* g_walkers_a, double* g_walkers_b, double* g_h1, void* ws,
                          size_t ws_bytes, void* stream) {
  TROT_TRY(check_adj(s));
  const AdjCommon a = common_of(s);
  if (!walkers_a || !g_energy || !g_walkers_a || !g_h1 || !ws ||
      (a.nspin == 2 && (!walkers_b || !g_walkers_b))) {
    set_error("null walkers, cotangent or workspace");
    return TROT_ERR_NULL_PTR;
  }
  for (int q = 0; q < a.nspin; ++q)
    if (!a.rot_chol[q] || !a.rot_h1[q]) { set_error("null measurement context"); return TROT_ERR_NULL_PTR; }
  Carver c(ws, ws_bytes);
  EnergyWs b;
  carve_energy(a, c, b);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  const int W = a.W, N = a.N, G = a.G;
  const double2* w[2] = {(const double2*)walkers_a, (const double2*)walkers_b};
  double2* gw[2] = {(double2*)g_walkers_a, (double2*)g_walkers_b};
  adj_act_from_cotangent_kernel<<<(W + 127) / 128, 128, 0, st>>>(W, g_energy, 0, b.act);
  TROT_CHECK_LAUNCH("adj_act_from_cotangent_kernel");
  // traces c_s[b][g] = tr f_{s,g}, f_{s,g} = R_{s,g} G_s^T; c_tot = sum_s mult_s c_s
  for (int q = 0; q < a.nspin; ++q) {
    const int n = a.n[q];
    TROT_TRY(green_launch(a, q, w[q], b.green[q], b.P[q], b.det, st));
    TROT_TRY(zero_inactive(W, a.nN[q], b.act, b.green[q], st));
    TROT_TRY(zero_inactive(W, (size_t)n * n, b.act, b.P[q], st));
    TROT_TRY(launch_zgemm_cr(W * n, G * n, N, 1.0, b.green[q], N, a.rot_chol[q], N, true, b.F, G * n, false, st));
    adj_trace_kernel<<<grid_of((size_t)W * G), 256, 0, st>>>(W, G, n, b.F, b.c[q]);
    TROT_CHECK_LAUNCH("adj_trace_kernel");
  }
  {
    Comb cb{};
    cb.nx = a.nspin;
    for (int q = 0; q < a.nspin; ++q) { cb.coef[q] = cmk((double)a.mult[q], 0.0); cb.x[q] = b.c[q]; }
    TROT_TRY(combine((size_t)W * G, cb, b.ctot, false, st));
  }
  // dE/dG_s = mult_s (rot_h1_s + sum_g c_tot,g R_{s,g} - sum_g f_{s,g} R_{s,g})
  for (int q = 0; q < a.nspin; ++q) {
    const int n = a.n[q];
    const double m = (double)a.mult[q];
    TROT_TRY(launch_zgemm_cr(W * n, G * n, N, 1.0, b.green[q], N, a.rot_chol[q], N, true, b.F, G * n, false, st));
    adj_block_transpose_kernel<<<grid_of((size_t)W * n * G * n), 256, 0, st>>>(W, G, n, b.F, b.Ft);
    TROT_CHECK_LAUNCH("adj_block_transpose_kernel");
    TROT_TRY(launch_zgemm_cr(W * n, N, G * n, -m, b.Ft, G * n, a.rot_chol[q], N, false, b.D, N, false, st));
    TROT_TRY(launch_zgemm_cr(W, (int)a.nN[q], G, m, b.ctot, G, a.rot_chol[q], (int)a.nN[q], false, b.D, (int)a.nN[q],
                             true, st));
    adj_energy_green_kernel<<<grid_of((size_t)W * a.nN[q]), 256, 0, st>>>(W, n, N, m, a.rot_h1[q], b.D, g_energy,
                                                                           b.gG);
    TROT_CHECK_LAUNCH("adj_energy_green_kernel");
    TROT_TRY(green_vjp_launch(a, q, b.green[q], b.gG, b.P[q], gw[q], st));
    adj_weighted_green_kernel<<<grid_of(a.nN[q]), 256, 0, st>>>(W, n, N, b.green[q], g_energy, b.H);
    TROT_CHECK_LAUNCH("adj_weighted_green_kernel");
    adj_h1_direct_kernel<<<grid_of((size_t)N * N), 256, 0, st>>>(N, n, m, a.mo[q], b.H, g_h1);
    TROT_CHECK_LAUNCH("adj_h1_direct_kernel");
  }
  return TROT_OK;
}

int trot_overlap_vjp(const trot_system* s, const double* walkers_a, const double* walkers_b, const double* g_overlaps,
                     double* g_walkers_a, double* g_walkers_b, void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_adj(s));
  const AdjCommon a = common_of(s);
  if (!walkers_a || !g_overlaps || !g_walkers_a || !ws || (a.nspin == 2 && (!walkers_b || !g_walkers_b))) {
    set_error("null walkers, cotangent or workspace");
    return TROT_ERR_NULL_PTR;
  }
  Carver c(ws, ws_bytes);
  double2 *green[2] = {nullptr, nullptr}, *P[2] = {nullptr, nullptr}, *det[2] = {nullptr, nullptr};
  for (int q = 0; q < a.nspin; ++q) {
    green[q] = c.take<double2>(a.W * a.nN[q]);
    P[q] = c.take<double2>((size_t)a.W * a.n[q] * a.n[q]);
    det[q] = c.take<double2>(a.W);
  }
  double2* ov = c.take<double2>((size_t)3 * a.W);  // ov, kappa, then W ints of walker flags
  double2* kappa = ov + a.W;
  int* act = reinterpret_cast<int*>(ov + 2 * a.W);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  const double2* w[2] = {(const double2*)walkers_a, (const double2*)walkers_b};
  double2* gw[2] = {(double2*)g_walkers_a, (double2*)g_walkers_b};
  adj_act_from_cotangent_kernel<<<(a.W + 127) / 128, 128, 0, st>>>(a.W, g_overlaps, 1, act);
  TROT_CHECK_LAUNCH("adj_act_from_cotangent_kernel");
  for (int q = 0; q < a.nspin; ++q) TROT_TRY(green_launch(a, q, w[q], green[q], P[q], det[q], st));
  TROT_TRY(ov_launch(a, det[0], det[1], ov, st));
  adj_kappa_kernel<<<(a.W + 127) / 128, 128, 0, st>>>(a.W, ov, (const double2*)g_overlaps, kappa);
  TROT_CHECK_LAUNCH("adj_kappa_kernel");
  for (int q = 0; q < a.nspin; ++q) {
    TROT_TRY(zero_inactive(a.W, (size_t)a.n[q] * a.n[q], act, P[q], st));
    adj_overlap_kernel<<<a.W, 256, 0, st>>>(a.N, a.n[q], (double)a.mult[q], a.mo[q], P[q], kappa, gw[q]);
    TROT_CHECK_LAUNCH("adj_overlap_kernel");
  }
  return TROT_OK;
}

int trot_orthonormalize_vjp(const trot_system* s, const double* walkers_a, const double* walkers_b,
                            const double* q_a, const double* q_b, const double* g_q_a, const double* g_q_b,
                            double* g_walkers_a, double* g_walkers_b, void* stream) {
  TROT_TRY(check_adj(s));
  const AdjCommon a = common_of(s);
  if (!walkers_a || !q_a || !g_q_a || !g_walkers_a || (a.nspin == 2 && (!walkers_b || !q_b || !g_q_b || !g_walkers_b))) {
    set_error("null walkers or cotangent");
    return TROT_ERR_NULL_PTR;
  }
  const double* w[2] = {walkers_a, walkers_b};
  const double* qq[2] = {q_a, q_b};
  const double* gq[2] = {g_q_a, g_q_b};
  double* gw[2] = {g_walkers_a, g_walkers_b};
  for (int q = 0; q < a.nspin; ++q) {
    adj_qr_kernel<<<a.W, 256, 0, (cudaStream_t)stream>>>(a.N, a.n[q], (const double2*)w[q], (const double2*)qq[q],
                                                         (const double2*)gq[q], (double2*)gw[q]);
    TROT_CHECK_LAUNCH("adj_qr_kernel");
  }
  return TROT_OK;
}

}  // extern "C"
