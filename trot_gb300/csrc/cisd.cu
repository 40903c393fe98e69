// CISD-trial overlap, force bias and local energy (FP64), restricted walkers
// in the trial's MO basis (reference determinant = orbitals [0, n)).
//
// Restated from trot/trial/cisd.py:148-186 and trot/meas/cisd.py:548-769
// ("high" memory mode, float64 contractions).  With x = G[:, n:] (n x v) and
// ci2m[(p,t),(q,u)] = 2 ci2[p,t,q,u] - ci2[p,u,q,t] (the reference's
// 2 ci2g_c - ci2g_e, 2 l2ci2_1 - l2ci2_2 and direct - exchange combinations):
//   ci2g = x . ci2m,  gci2g = sum ci2g o x,  ci1g = sum ci1 o x,
//   ov = 1 + 2 ci1g + gci2g        (overlap = ov det(w_occ)^2)
//   ci1_green = (gp ci1^T) G,  ci2_green = (gp ci2g^T) G   (N x N; gp rows < n: x, rows >= n: -I)
//   force bias = (2 lg + 4 ci1g lg + 2 gci2g lg - 2 lcs) / ov
//     with lg = rot_chol . G, lcs = lci1g + lci2g = chol . (ci1_green + ci2_green)
//     (the energy uses lci1g and lci2g only as -4 (lci1g + lci2g) . lg as well)
//   local energy: the terms of energy_kernel_rw_rh, see cisd_energy_combine.
// The l2ci2 quadratic forms 2 sum_g X_g^T ci2 X_g - X_g^T ci2_perm X_g (ci2_perm[(p,u),(q,t)] = ci2[p,t,q,u])
// = sum_g X_g^T ci2m X_g (X_g = vec(glgp_g)) are one GEMM over all (walker, g) rows.
#include <cuda_bf16.h>

#include <algorithm>

#include "ff.cuh"
#include "kernels.h"
#include "mixed.h"
#include "profile.h"
#include "step_tail.cuh"
#include "tc.cuh"

namespace trot {

// ------------------------------------------------------------------ workspace
struct CisdBuffers {
  int* status;                  // device status word (offset 0 of the workspace)
  double2 *green, *det2, *hg2;  // G (W, n, N); det(w_occ)^2 (W); 2 hg (W)
  double2* x;                   // (W, n v) contiguous x
  double2* cg;                  // ci2g = x ci2m (W, n v)
  double2* ci1g1;               // (W, n, n)
  double2 *ms, *m2;             // ci1_green + ci2_green, ci2_green (W, N, N)
  double2* msp;                 // ms packed: upper triangle, ms[i][j] + ms[j][i] off the diagonal (W, P)
  double* lp;                   // chol packed: upper triangle of chol[g] (G, P), P = N (N + 1) / 2
  double2* p2;                  // P2 = gp ci2g^T (W, N, n): ci2_green = P2 G
  double2* wsc;                 // per-walker scalars (W, 8): ci1g, gci2g, e1_1_2, e1_2_2, ...
  double2 *lg, *lcs;            // (W, G): rot_chol . G, chol . (ci1_green + ci2_green)
  double2* kpart;               // split-K partials of the FP64 products
  ff *rd, *lc;                  // chol rows < n transposed, lci1: float-float (G, N, n)   (FP32 gl)
  uint16_t *glimg, *glq;        // split3 images of chol (rows (g, j), K = i) and of G     (FP32 gl)
  float* gld;                   // gl = G L_g for all (walker, p) x (g, j), FP32           (FP32 gl)
  double2* xg;                  // glgp rows (W G, n v)
  double2* y;                   // xg ci2m (W G, n v)    (FP64 l2ci2)
  uint16_t* xq;                 // split3 image of xg    (mixed l2ci2)
  float* yd;                    // xg ci2m, FP32         (mixed l2ci2)
  double2* gpart;               // per (walker, gamma chunk) partial sums (W, nchunk, 4)
  double2* l2part;              // l2ci2 partial sums (W, kL2Parts)
  // propagation step
  double2 *fb, *xs, *shift_term, *fb_term, *vhs, *ov_new;
  int* node_flag;
};

static constexpr int kCisdGChunk = 8;
static constexpr int kL2Parts = 8;  // CTAs per walker of the l2ci2 reductions
static int cisd_chunks(int G) { return (G + kCisdGChunk - 1) / kCisdGChunk; }
// gl = G L_g as one split-BF16 tensor-core product: K = N padded to 64, columns (g, j) to 128
static size_t cisd_gl_kpad(int N) { return (size_t)(N + 63) / 64 * 64; }
static size_t cisd_gl_npad(int N, int G) { return ((size_t)G * N + 127) / 128 * 128; }

// K slices for an FP64 product (M x Nn, long K) so that its 64 x 64 tiles fill
// every SM twice; at least 64 of K per slice.
static int cisd_splitk(int M, int Nn, int K) {
  const int base = ((Nn + 63) / 64) * ((M + 63) / 64);
  int S = (2 * 152 + base - 1) / base;
  S = std::min(S, std::max(1, K / 64));
  return std::max(1, std::min(S, 16));
}

static size_t carve_cisd(const trot_cisd* c, int W, int op, Carver& cv, CisdBuffers& b) {
  const size_t N = c->norb, n = c->nocc, v = c->nvir, G = c->nchol, nv = n * v;
  b = CisdBuffers{};
  b.status = cv.status();
  b.green = cv.take<double2>(W * n * N);
  b.det2 = cv.take<double2>(W);
  b.hg2 = cv.take<double2>(W);
  b.x = cv.take<double2>(W * nv);
  b.cg = cv.take<double2>(W * nv);
  b.wsc = cv.take<double2>(W * 8);
  {
    size_t kp = (size_t)cisd_splitk(W, (int)nv, (int)nv) * W * nv;  // ci2g
    if (op != TROT_OP_OVERLAP) {
      kp = std::max(kp, (size_t)cisd_splitk(W, (int)G, (int)(n * N)) * W * G);  // lg
      kp = std::max(kp, (size_t)cisd_splitk(W, (int)G, (int)(N * N)) * W * G);  // lcs (the packed K is shorter)
    }
    b.kpart = cv.take<double2>(kp);
  }
  if (op == TROT_OP_OVERLAP) return cv.used;
  b.ci1g1 = cv.take<double2>(W * n * n);
  b.ms = cv.take<double2>(W * N * N);
  b.m2 = cv.take<double2>(W * N * N);
  if (c->chol_symmetric) {
    b.msp = cv.take<double2>(W * N * (N + 1) / 2);
    b.lp = cv.take<double>(G * N * (N + 1) / 2);
  }
  b.p2 = cv.take<double2>(W * N * n);
  b.lg = cv.take<double2>(W * G);
  b.lcs = cv.take<double2>(W * G);
  if (op == TROT_OP_FORCE_BIAS) return cv.used;
  b.xg = cv.take<double2>((size_t)W * G * nv);
  if (c->l2ci2_precision == TROT_MIXED) {
    const size_t mpad = split3_mpad((int)(W * G));
    b.xq = cv.take<uint16_t>(3 * mpad * (size_t)c->nvpad);
    b.yd = cv.take<float>(mpad * (size_t)c->ncpad);
  } else {
    b.y = cv.take<double2>((size_t)W * G * nv);
  }
  b.gpart = cv.take<double2>((size_t)W * cisd_chunks((int)G) * 4);
  b.l2part = cv.take<double2>((size_t)W * kL2Parts);
  if (c->gl_precision == TROT_MIXED) {
    const size_t kp = cisd_gl_kpad((int)N), np = cisd_gl_npad((int)N, (int)G), mp = split3_mpad((int)(W * n));
    b.glimg = cv.take<uint16_t>(3 * np * kp);
    b.glq = cv.take<uint16_t>(3 * mp * kp);
    b.gld = cv.take<float>(mp * np);
    b.rd = cv.take<ff>(G * N * n);
    b.lc = cv.take<ff>(G * N * n);
  }
  if (op != TROT_OP_PROP_STEP) return cv.used;
  b.fb = cv.take<double2>((size_t)W * G);
  b.xs = cv.take<double2>((size_t)W * G);
  b.shift_term = cv.take<double2>(W);
  b.fb_term = cv.take<double2>(W);
  b.vhs = cv.take<double2>((size_t)W * N * N);
  b.ov_new = cv.take<double2>(W);
  b.node_flag = cv.take<int>(W);
  return cv.used;
}

// ------------------------------------------------------------------ packed symmetric contraction
// With every L_g symmetric, sum_ij L_g[i][j] M[i][j] = sum_{i <= j} L_g[i][j] Mp[i][j] over the
// upper triangle (of (L_g + L_g^T) / 2: symmetric to rounding after a basis rotation) (row-major, k(i, j) = i N - i (i - 1) / 2 + j - i), Mp[i][j] = M[i][j] + M[j][i]
// off the diagonal and M[i][i] on it: half the FP64 products of chol . (ci1_green + ci2_green).
__global__ void cisd_pack_chol_kernel(int N, int G, const double* __restrict__ chol, double* __restrict__ lp) {
  const size_t P = (size_t)N * (N + 1) / 2, total = (size_t)G * N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t g = e / ((size_t)N * N);
    const int r = (int)(e % ((size_t)N * N)), i = r / N, j = r % N;
    if (j >= i)
      lp[g * P + (size_t)i * N - (size_t)i * (i - 1) / 2 + (j - i)] =
          0.5 * (chol[e] + chol[g * N * N + (size_t)j * N + i]);
  }
}

__global__ void cisd_pack_ms_kernel(int N, int W, const double2* __restrict__ ms, double2* __restrict__ msp) {
  const size_t P = (size_t)N * (N + 1) / 2, total = (size_t)W * N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t b = e / ((size_t)N * N);
    const int r = (int)(e % ((size_t)N * N)), i = r / N, j = r % N;
    if (j < i) continue;
    double2 v = ms[e];
    if (j > i) v = cadd(v, ms[b * N * N + (size_t)j * N + i]);
    msp[b * P + (size_t)i * N - (size_t)i * (i - 1) / 2 + (j - i)] = v;
  }
}

// ------------------------------------------------------------------ x, ci1g, ci1g1
// x[b][p][t] = G[b][p][n + t];  ci1g = sum ci1 o x;  ci1g1[a][q] = sum_t ci1[a][t] G[q][n + t]
__global__ void cisd_x_kernel(int N, int n, int v, const double2* __restrict__ green, const double* __restrict__ ci1,
                              double2* __restrict__ x, double2* __restrict__ ci1g1, double2* __restrict__ wsc) {
  __shared__ double2 red[32];
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const double2* g = green + (size_t)b * n * N;
  double2 acc = cmk(0.0, 0.0);
  for (int e = tid; e < n * v; e += nt) {
    const int p = e / v, t = e % v;
    const double2 val = g[p * N + n + t];
    x[(size_t)b * n * v + e] = val;
    crfma(acc, ci1[e], val);
  }
  if (ci1g1) {
    for (int e = tid; e < n * n; e += nt) {
      const int a = e / n, q = e % n;
      double2 s = cmk(0.0, 0.0);
      for (int t = 0; t < v; ++t) crfma(s, ci1[a * v + t], g[q * N + n + t]);
      ci1g1[(size_t)b * n * n + e] = s;
    }
  }
  acc = block_sum2(acc, red);
  if (tid == 0) wsc[(size_t)b * 8 + 0] = acc;  // ci1g
}

// ------------------------------------------------------------------ per-walker N x N matrices
// gci2g = sum ci2g o x; P_Y = gp Y^T (N x n); M = P_Y G (N x N) for Y = ci1, ci2g;
// e1_1_2 = -2 sum h1 o M1, e1_2_2 = -2 sum h1 o M2.  Stores M1 + M2 (the force bias,
// the energy and the 1-RDM use chol . ci1_green and chol . ci2_green only in that sum)
// and M2 (lci2_green).
__global__ void __launch_bounds__(256)
cisd_mats_kernel(int N, int n, int v, const double2* __restrict__ green, const double* __restrict__ ci1,
                 const double2* __restrict__ cg, const double2* __restrict__ x,
                 const double* __restrict__ h1, double2* __restrict__ ms, double2* __restrict__ m2,
                 double2* __restrict__ p2o, double2* __restrict__ wsc) {
  extern __shared__ double2 sm[];
  __shared__ double2 red[32];
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  double2* Gs = sm;              // n x N
  double2* Y2 = Gs + n * N;      // n x v  (ci2g)
  double2* P1 = Y2 + n * v;      // N x n
  double2* P2 = P1 + N * n;      // N x n
  const double2* g = green + (size_t)b * n * N;
  for (int e = tid; e < n * N; e += nt) Gs[e] = g[e];
  double2 gs = cmk(0.0, 0.0);
  for (int e = tid; e < n * v; e += nt) {
    const double2 y = cg[(size_t)b * n * v + e];
    Y2[e] = y;
    cfma(gs, y, x[(size_t)b * n * v + e]);
  }
  __syncthreads();
  // P[i][p] = sum_t gp[i][t] Y[p][t]: i < n -> sum_t x[i][t] Y[p][t]; i >= n -> -Y[p][i - n]
  for (int e = tid; e < N * n; e += nt) {
    const int i = e / n, p = e % n;
    double2 a1 = cmk(0.0, 0.0), a2 = cmk(0.0, 0.0);
    if (i < n) {
      for (int t = 0; t < v; ++t) {
        const double2 xv = Gs[i * N + n + t];
        crfma(a1, ci1[p * v + t], xv);
        cfma(a2, Y2[p * v + t], xv);
      }
    } else if (i - n < v) {
      a1 = cmk(-ci1[p * v + (i - n)], 0.0);
      const double2 y = Y2[p * v + (i - n)];
      a2 = cmk(-y.x, -y.y);
    }
    P1[e] = a1;
    P2[e] = a2;
    p2o[(size_t)b * N * n + e] = a2;
  }
  __syncthreads();
  double2 h1s = cmk(0.0, 0.0), h2s = cmk(0.0, 0.0);
  for (int e = tid; e < N * N; e += nt) {
    const int i = e / N, j = e % N;
    double2 s1 = cmk(0.0, 0.0), s2 = cmk(0.0, 0.0);
    for (int p = 0; p < n; ++p) {
      const double2 gv = Gs[p * N + j];
      cfma(s1, P1[i * n + p], gv);
      cfma(s2, P2[i * n + p], gv);
    }
    ms[(size_t)b * N * N + e] = cadd(s1, s2);
    m2[(size_t)b * N * N + e] = s2;
    const double hv = h1[e];
    crfma(h1s, hv, s1);
    crfma(h2s, hv, s2);
  }
  gs = block_sum2(gs, red);
  h1s = block_sum2(h1s, red);
  h2s = block_sum2(h2s, red);
  if (tid == 0) {
    wsc[(size_t)b * 8 + 1] = gs;                           // gci2g
    wsc[(size_t)b * 8 + 2] = cmk(-2.0 * h1s.x, -2.0 * h1s.y);  // e1_1_2
    wsc[(size_t)b * 8 + 3] = cmk(-2.0 * h2s.x, -2.0 * h2s.y);  // e1_2_2
  }
}

// ------------------------------------------------------------------ per (walker, Cholesky chunk) terms
// For each g in the chunk (L = chol_g, R = L[:n, :]):
//   lg1 = R G^T (n x n), lci1g_mat B[q][a] = sum_i G[q][i] lci1_g[i][a]
//   gl = G L (n x N), lci2_green[p][j] = sum_i R[p][i] M2[j][i], glgp = gl gp (n x v) -> xg
//   partial sums: [0] sum lg1 o lg1^T, [1] tr(lg1 lg1 ci1g1), [2] sum B o lg1, [3] sum gl o lci2_green
__global__ void __launch_bounds__(256)
cisd_gamma_kernel(int N, int n, int v, int G, const double2* __restrict__ green, const double* __restrict__ chol,
                  const double* __restrict__ lci1, const double2* __restrict__ m2, const double2* __restrict__ ci1g1,
                  double2* __restrict__ xg, double2* __restrict__ gpart) {
  extern __shared__ double2 sm[];
  __shared__ double2 red[32];
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int nchunk = gridDim.x;
  double2* Gs = sm;                 // n x N
  double2* M2 = Gs + n * N;         // N x N
  double2* C1 = M2 + N * N;         // n x n  (ci1g1)
  double2* A = C1 + n * n;          // n x n  (lg1)
  double2* GL = A + n * n;          // n x N  (gl)
  double* Ls = reinterpret_cast<double*>(GL + n * N);  // N x N
  for (int e = tid; e < n * N; e += nt) Gs[e] = green[(size_t)b * n * N + e];
  for (int e = tid; e < N * N; e += nt) M2[e] = m2[(size_t)b * N * N + e];
  for (int e = tid; e < n * n; e += nt) C1[e] = ci1g1[(size_t)b * n * n + e];
  double2 s0 = cmk(0.0, 0.0), s1 = cmk(0.0, 0.0), s2 = cmk(0.0, 0.0), s3 = cmk(0.0, 0.0);
  const int g0 = chunk * kCisdGChunk, g1 = min(G, g0 + kCisdGChunk);
  for (int gg = g0; gg < g1; ++gg) {
    __syncthreads();
    const double* Lg = chol + (size_t)gg * N * N;
    for (int e = tid; e < N * N; e += nt) Ls[e] = Lg[e];
    __syncthreads();
    // lg1[p][q] = sum_j L[p][j] G[q][j]
    for (int e = tid; e < n * n; e += nt) {
      const int p = e / n, q = e % n;
      double2 a = cmk(0.0, 0.0);
      for (int j = 0; j < N; ++j) crfma(a, Ls[p * N + j], Gs[q * N + j]);
      A[e] = a;
    }
    // gl[p][i] = sum_j G[p][j] L[j][i]
    for (int e = tid; e < n * N; e += nt) {
      const int p = e / N, i = e % N;
      double2 a = cmk(0.0, 0.0);
      for (int j = 0; j < N; ++j) crfma(a, Ls[j * N + i], Gs[p * N + j]);
      GL[e] = a;
    }
    __syncthreads();
    const double* lc = lci1 + (size_t)gg * N * n;
    for (int e = tid; e < n * n; e += nt) {
      const int p = e / n, q = e % n;
      // sum lg1 o lg1^T
      cfma(s0, A[p * n + q], A[q * n + p]);
      // tr(lg1 lg1 ci1g1): [lg1 lg1][p][a] ci1g1[a][p] -> sum over (p, q, a): A[p][q] A[q][a] C1[a][p]
      double2 t = cmk(0.0, 0.0);
      for (int a2 = 0; a2 < n; ++a2) cfma(t, A[q * n + a2], C1[a2 * n + p]);
      cfma(s1, A[p * n + q], t);
      // B[q][a] = sum_i G[q][i] lci1_g[i][a]  (here (p, q) -> (q_idx = p, a = q))
      double2 bq = cmk(0.0, 0.0);
      for (int i = 0; i < N; ++i) crfma(bq, lc[i * n + q], Gs[p * N + i]);
      cfma(s2, bq, A[p * n + q]);
    }
    // sum gl o lci2_green, lci2_green[p][j] = sum_i R[p][i] M2[j][i]
    for (int e = tid; e < n * N; e += nt) {
      const int p = e / N, j = e % N;
      double2 a = cmk(0.0, 0.0);
      for (int i = 0; i < N; ++i) crfma(a, Ls[p * N + i], M2[j * N + i]);
      cfma(s3, GL[e], a);
    }
    // glgp[p][t] = sum_{i<n} gl[p][i] x[i][t] - gl[p][n + t]
    double2* xo = xg + ((size_t)b * G + gg) * n * v;
    for (int e = tid; e < n * v; e += nt) {
      const int p = e / v, t = e % v;
      double2 a = cmk(-GL[p * N + n + t].x, -GL[p * N + n + t].y);
      for (int i = 0; i < n; ++i) cfma(a, GL[p * N + i], Gs[i * N + n + t]);
      xo[e] = a;
    }
  }
  s0 = block_sum2(s0, red);
  s1 = block_sum2(s1, red);
  s2 = block_sum2(s2, red);
  s3 = block_sum2(s3, red);
  if (tid == 0) {
    double2* o = gpart + ((size_t)b * nchunk + chunk) * 4;
    o[0] = s0; o[1] = s1; o[2] = s2; o[3] = s3;
  }
}

// Same sums as cisd_gamma_kernel with gl = G L in FP32 (the reference's float32 mixed
// dtype; sums accumulated in float-float), and lg1 = R G^T, lci1g = lci1^T G^T and
// their products in float-float (FP32 pairs, ~2^-44 relative: FP64-level results on
// the FP32 pipe; GB300's FP64 pipe runs a few operations per clock per SM).  With
// ci2_green = P2 G (rank n), lci2_green = R ci2_green^T = lg1 P2^T, so the fourth sum
// sum_pj gl[p][j] lci2_green[p][j] = sum_pk lg1[p][k] (gl P2)[p][k]: an n x N x n
// product (FP32) instead of the n x N x N one.  Double -> float / float-float
// conversions by integer operations (ff.cuh) for the same reason.
TROT_D void ffc_mad(ffc& acc, const ffc& a, const ffc& b) {  // acc += a b (complex)
  ff_mad(acc.re, a.re, b.re);
  ff_mad(acc.re, ff{-a.im.hi, -a.im.lo}, b.im);
  ff_mad(acc.im, a.re, b.im);
  ff_mad(acc.im, a.im, b.re);
}
TROT_D ffc ffc_norm(ffc a) { return ffc{ff_fast(a.re.hi, a.re.lo), ff_fast(a.im.hi, a.im.lo)}; }
TROT_D double2 ffc_d(ffc a) { return make_double2(ff_d(a.re), ff_d(a.im)); }

// chol and lci1 in the operand forms of cisd_gamma_f32_kernel, once per call:
// rd[g][j][p] = chol[g][p][j] (p < n) and lc[g][i][q] = lci1[g][i][q] in float-float.
__global__ void cisd_chol_forms_kernel(int N, int n, int G, const double* __restrict__ chol,
                                       const double* __restrict__ lci1, ff* __restrict__ rd, ff* __restrict__ lc) {
  const size_t Nn = (size_t)N * n, total = (size_t)G * Nn;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t g = e / Nn;
    const int r = (int)(e % Nn), p = r / N, j = r % N;  // r < n N: rows p < n of chol_g
    rd[g * Nn + (size_t)j * n + p] = ff_from_d(chol[g * N * N + r]);
    lc[g * Nn + r] = ff_from_d(lci1[g * Nn + r]);
  }
}

// The B operand of gl = G L_g for every Cholesky vector: B(i, (g, j)) = chol[g][i][j],
// stored as B^T (rows (g, j), K = i) in the split-BF16 tensor-core image
// [npad/128][kpad/64][3 slices][128][64] (core-matrix order), once per call.
__global__ void cisd_gl_image_kernel(int N, int G, int kpad, int npad, const double* __restrict__ chol,
                                     uint16_t* __restrict__ img) {
  const int nkc = kpad / 64;
  const size_t total = (size_t)npad * kpad;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(e / kpad), k = (int)(e % kpad);
    float x = 0.f;
    if (row < G * N && k < N) {
      const int g = row / N, j = row % N;
      x = d2f_bits(chol[((size_t)g * N + k) * N + j]);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
    const size_t base = ((size_t)(row >> 7) * nkc + (k >> 6)) * 3 * 8192 + tc::tile_off(row & 127, k & 63) / 2;
    img[base] = *reinterpret_cast<const uint16_t*>(&h);
    img[base + 8192] = *reinterpret_cast<const uint16_t*>(&m);
    img[base + 16384] = *reinterpret_cast<const uint16_t*>(&l);
  }
}

// Four lanes hold partial sums of one item: add them (all lanes of the warp take part)
TROT_D ffc ffc_quad_sum(ffc a) {
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
    a.re = ff_add(a.re, ff_shfl_xor(a.re, o));
    a.im = ff_add(a.im, ff_shfl_xor(a.im, o));
  }
  return a;
}

__global__ void __launch_bounds__(256, 4)
cisd_gamma_f32_kernel(int N, int n, int v, int G, const double2* __restrict__ green, const float* __restrict__ gld,
                      int ldd, const ff* __restrict__ rd, const ff* __restrict__ lc, const double2* __restrict__ p2,
                      const double2* __restrict__ ci1g1, double2* __restrict__ xg, double2* __restrict__ gpart) {
  extern __shared__ double2 sm[];
  __shared__ double2 red[32];
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int nchunk = gridDim.x;
  // j-major copies (GsT[j][q] = G[q][j], RdT[j][p] = L_g[p][j], AT[q][p] = lg1[p][q]) keep the
  // per-thread index q (or p) fastest across a warp; their rows are padded to ns = n + 1
  // entries so that the four lanes of a quad (rows part + 4k) fall on different banks
  const int ns = n + 1;
  ffc* GsT = reinterpret_cast<ffc*>(sm);                  // N x ns
  ffc* C1 = GsT + ns * N;                                 // n x ns
  ffc* A = C1 + ns * n;                                   // n x n  (lg1)
  ff* RdT = reinterpret_cast<ff*>(A + n * n);             // N x ns (rows < n of L_g, transposed)
  float2* Gf = reinterpret_cast<float2*>(RdT + ns * N);   // n x N
  float2* P2f = Gf + n * N;                               // N x n
  float2* GLf = P2f + N * n;                              // n x N: gl_g of this walker
  ff* Lc = reinterpret_cast<ff*>(GLf + n * N);            // N x n: lci1_g
  ffc* AT = reinterpret_cast<ffc*>(Lc + N * n);           // n x ns: lg1 transposed
  for (int e = tid; e < n * N; e += nt) {
    const double2 g = green[(size_t)b * n * N + e];
    GsT[(e % N) * ns + e / N] = ffc{ff_from_d(g.x), ff_from_d(g.y)};
    Gf[e] = make_float2(d2f_bits(g.x), d2f_bits(g.y));
  }
  for (int e = tid; e < N * n; e += nt) {
    const double2 m = p2[(size_t)b * N * n + e];
    P2f[e] = make_float2(d2f_bits(m.x), d2f_bits(m.y));
  }
  for (int e = tid; e < n * n; e += nt) {
    const double2 c = ci1g1[(size_t)b * n * n + e];
    C1[(e / n) * ns + e % n] = ffc{ff_from_d(c.x), ff_from_d(c.y)};
  }
  const ffc z{{0.f, 0.f}, {0.f, 0.f}};
  ffc s0 = z, s1 = z, s2 = z, s3 = z;
  const int g0 = chunk * kCisdGChunk, g1 = min(G, g0 + kCisdGChunk);
  // the float-float n x n phases run four lanes per (p, q), each over every fourth term
  const int quad = tid >> 2, part = tid & 3, nq = nt >> 2;
  for (int gg = g0; gg < g1; ++gg) {
    __syncthreads();
    // gl_g rows p of this walker: rows 2 (b n + p) (Re) and 2 (b n + p) + 1 (Im), columns g N + j
    for (int e = tid; e < n * N; e += nt) {
      const int p = e / N, j = e % N;
      const float* r0 = gld + 2 * ((size_t)b * n + p) * ldd + (size_t)gg * N + j;
      GLf[e] = make_float2(r0[0], r0[ldd]);
    }
    const ff* rg = rd + (size_t)gg * N * n;
    const ff* cg = lc + (size_t)gg * N * n;
    for (int e = tid; e < N * n; e += nt) {
      RdT[(e / n) * ns + e % n] = rg[e];
      Lc[e] = cg[e];
    }
    __syncthreads();
    for (int e0 = 0; e0 < n * n; e0 += nq) {  // lg1[p][q] = sum_j R[p][j] G[q][j]
      const int e = e0 + quad;
      ffc a = z;
      if (e < n * n) {
        const int p = e / n, q = e % n;
        for (int j = part; j < N; j += 4) {
          const ff r = RdT[j * ns + p];
          const ffc g = GsT[j * ns + q];
          ff_mad(a.re, r, g.re);
          ff_mad(a.im, r, g.im);
        }
        a = ffc_norm(a);
      }
      a = ffc_quad_sum(a);
      if (e < n * n && part == 0) {
        A[e] = a;
        AT[(e % n) * ns + e / n] = a;
      }
    }
    __syncthreads();
    for (int e0 = 0; e0 < n * n; e0 += nq) {
      const int e = e0 + quad;
      ffc t = z, bq = z;
      float zr = 0.f, zi = 0.f;
      if (e < n * n) {
        const int p = e / n, q = e % n;
        for (int a2 = part; a2 < n; a2 += 4) ffc_mad(t, AT[a2 * ns + q], C1[a2 * ns + p]);
        for (int i = part; i < N; i += 4) {  // lci1g[q][p] = sum_i lci1[i][q] G[p][i]
          const ff l = Lc[i * n + q];
          const ffc g = GsT[i * ns + p];
          ff_mad(bq.re, l, g.re);
          ff_mad(bq.im, l, g.im);
        }
        for (int j = part; j < N; j += 4) {  // (gl P2)[p][q]
          const float2 a = GLf[p * N + j], m = P2f[j * n + q];
          zr = fmaf(a.x, m.x, fmaf(-a.y, m.y, zr));
          zi = fmaf(a.x, m.y, fmaf(a.y, m.x, zi));
        }
        t = ffc_norm(t);
        bq = ffc_norm(bq);
      }
      t = ffc_quad_sum(t);
      bq = ffc_quad_sum(bq);
#pragma unroll
      for (int o = 1; o < 4; o <<= 1) {
        zr += __shfl_xor_sync(0xffffffffu, zr, o);
        zi += __shfl_xor_sync(0xffffffffu, zi, o);
      }
      if (e < n * n && part == 0) {
        const ffc apq = A[e];
        ffc_mad(s0, apq, AT[(e / n) * ns + e % n]);
        ffc_mad(s1, apq, t);
        ffc_mad(s2, bq, apq);
        ffc_mad(s3, apq, ffc{ff{zr, 0.f}, ff{zi, 0.f}});
      }
    }
    s0 = ffc_norm(s0);
    s1 = ffc_norm(s1);
    s2 = ffc_norm(s2);
    s3 = ffc_norm(s3);
    double2* xo = xg + ((size_t)b * G + gg) * n * v;
    for (int e = tid; e < n * v; e += nt) {
      const int p = e / v, t = e % v;
      const float2 gl = GLf[p * N + n + t];
      float ar = -gl.x, ai = -gl.y;
      for (int i = 0; i < n; ++i) {
        const float2 a = GLf[p * N + i], x = Gf[i * N + n + t];
        ar = fmaf(a.x, x.x, fmaf(-a.y, x.y, ar));
        ai = fmaf(a.x, x.y, fmaf(a.y, x.x, ai));
      }
      xo[e] = make_double2(f2d_bits(ar), f2d_bits(ai));
    }
  }
  double2 d0 = block_sum2(ffc_d(s0), red);
  double2 d1 = block_sum2(ffc_d(s1), red);
  double2 d2 = block_sum2(ffc_d(s2), red);
  double2 d3 = block_sum2(ffc_d(s3), red);
  if (tid == 0) {
    double2* o = gpart + ((size_t)b * nchunk + chunk) * 4;
    o[0] = d0; o[1] = d1; o[2] = d2; o[3] = d3;
  }
}

// l2ci2 from the tensor-core product: Y = xg ci2m in FP32, rows 2r (Re) / 2r+1 (Im) of yd
// (row stride ldy); per walker sum over g of X_g . Y_g, FP64 accumulation.
// l2ci2 partial sums: CTA (c, b) takes Cholesky rows [c G/P, (c+1) G/P) of walker b
// (a warp per row, lanes along nv) and writes part[b][c] (P = kL2Parts); the energy
// kernel adds the P partials in order.

// Y is FP32 and X is rounded to FP32 (by integer operations): FP32 complex products,
// summed per thread in float-float and across the block in FP64 (no FP64-pipe work
// per element)
__global__ void __launch_bounds__(256)
cisd_l2_reduce_tc_kernel(int G, int nv, int ldy, const double2* __restrict__ xg, const float* __restrict__ yd,
                         double2* __restrict__ part) {
  __shared__ double2 red[32];
  const int c = blockIdx.x, b = blockIdx.y, nparts = gridDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int gpp = (G + nparts - 1) / nparts, g0 = c * gpp, g1 = min(G, g0 + gpp);
  ff ar{0.f, 0.f}, ai{0.f, 0.f};
  for (int g = g0 + warp; g < g1; g += nw) {
    const size_t r = (size_t)b * G + g;
    const double2* xr = xg + r * nv;
    const float* y0 = yd + 2 * r * (size_t)ldy;
    const float* y1 = y0 + ldy;
    for (int k = lane; k < nv; k += 32) {
      const double2 xv = xr[k];
      const float xre = d2f_bits(xv.x), xim = d2f_bits(xv.y);
      const float yr = y0[k], yi = y1[k];
      const float pr = fmaf(xre, yr, __fmul_rn(-xim, yi)), pi = fmaf(xre, yi, __fmul_rn(xim, yr));
      const ff tr = ff_two_sum(ar.hi, pr), ti = ff_two_sum(ai.hi, pi);
      ar = ff{tr.hi, __fadd_rn(ar.lo, tr.lo)};
      ai = ff{ti.hi, __fadd_rn(ai.lo, ti.lo)};
    }
  }
  const double2 acc = block_sum2(make_double2(ff_d(ar), ff_d(ai)), red);
  if (threadIdx.x == 0) part[(size_t)b * nparts + c] = acc;
}

// l2ci2 (FP64): per walker sum over g of X_g . Y_g, Y = xg ci2m, partials as above
__global__ void __launch_bounds__(256)
cisd_l2_reduce_kernel(int G, int nv, const double2* __restrict__ xg, const double2* __restrict__ y,
                      double2* __restrict__ part) {
  __shared__ double2 red[32];
  const int c = blockIdx.x, b = blockIdx.y, nparts = gridDim.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int gpp = (G + nparts - 1) / nparts, g0 = c * gpp, g1 = min(G, g0 + gpp);
  double2 acc = cmk(0.0, 0.0);
  for (int g = g0 + warp; g < g1; g += nw) {
    const size_t base = ((size_t)b * G + g) * nv;
    for (int k = lane; k < nv; k += 32) cfma(acc, xg[base + k], y[base + k]);
  }
  acc = block_sum2(acc, red);
  if (threadIdx.x == 0) part[(size_t)b * nparts + c] = acc;
}

// ------------------------------------------------------------------ combines
__device__ __forceinline__ double2 cdot_row(const double2* a, const double2* b, int n) {
  double2 s = cmk(0.0, 0.0);
  for (int k = 0; k < n; ++k) cfma(s, a[k], b[k]);
  return s;
}

// overlap = (1 + 2 ci1g + gci2g) det0^2, gci2g = sum ci2g o x; one CTA per walker
__global__ void cisd_overlap_kernel(int nv, const double2* __restrict__ x, const double2* __restrict__ cg,
                                    const double2* __restrict__ wsc,
                                    const double2* __restrict__ det2, double2* __restrict__ out) {
  __shared__ double2 red[32];
  const int b = blockIdx.x;
  double2 gs = cmk(0.0, 0.0);
  for (int e = threadIdx.x; e < nv; e += blockDim.x) {
    const size_t k = (size_t)b * nv + e;
    cfma(gs, cg[k], x[k]);
  }
  gs = block_sum2(gs, red);
  if (threadIdx.x == 0) {
    const double2 ci1g = wsc[(size_t)b * 8 + 0];
    out[b] = cmul(cmk(1.0 + 2.0 * ci1g.x + gs.x, 2.0 * ci1g.y + gs.y), det2[b]);
  }
}

// force bias: (2 lg (1 + 2 ci1g + gci2g) - 2 lcs) / ov,  lcs = lci1g + lci2g
__global__ void cisd_fb_kernel(int W, int G, const double2* __restrict__ wsc, const double2* __restrict__ lg,
                               const double2* __restrict__ lcs, double2* __restrict__ fb) {
  const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (k >= (size_t)W * G) return;
  const int b = (int)(k / G);
  const double2 ci1g = wsc[(size_t)b * 8 + 0], gci2g = wsc[(size_t)b * 8 + 1];
  const double2 ov = cmk(1.0 + 2.0 * ci1g.x + gci2g.x, 2.0 * ci1g.y + gci2g.y);
  const double2 f = cmk(2.0 * ci1g.x + gci2g.x, 2.0 * ci1g.y + gci2g.y);  // (ov - 1)
  // 2 lg + 4 ci1g lg + 2 gci2g lg = 2 lg (1 + 2 ci1g + gci2g) = 2 lg ov
  const double2 a = cmul(lg[k], cmk(2.0 * (1.0 + f.x), 2.0 * f.y));
  const double2 c = lcs[k];
  fb[k] = cdiv(cmk(a.x - 2.0 * c.x, a.y - 2.0 * c.y), ov);
}

// mixed-estimator 1-RDM (trot/meas/cisd.py:772-820): gamma = G0 - (ci1_green + ci2_green) / ov,
// G0[i][j] = G[j][i] for j < n, 0 otherwise
__global__ void cisd_rdm1_kernel(int N, int n, const double2* __restrict__ green, const double2* __restrict__ ms,
                                 const double2* __restrict__ wsc, double2* __restrict__ out) {
  const int b = blockIdx.y;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N * N) return;
  const int i = e / N, j = e % N;
  const double2 ci1g = wsc[(size_t)b * 8 + 0], gci2g = wsc[(size_t)b * 8 + 1];
  const double2 ov = cmk(1.0 + 2.0 * ci1g.x + gci2g.x, 2.0 * ci1g.y + gci2g.y);
  const size_t k = (size_t)b * N * N + e;
  const double2 corr = cdiv(ms[k], ov);
  const double2 g0 = j < n ? green[(size_t)b * n * N + (size_t)j * N + i] : cmk(0.0, 0.0);
  out[k] = csub(g0, corr);
}

// phaseless weights from the CISD overlaps of the propagated walkers
__global__ void cisd_weight_kernel(TrotterArgs a, const double2* __restrict__ ov_new) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < a.W) phaseless_update(a, b, ov_new[b]);
}

// local energy (trot/meas/cisd.py:608-769)
__global__ void __launch_bounds__(256)
cisd_energy_kernel(int G, int nchunk, double h0, const double2* __restrict__ wsc, const double2* __restrict__ hg2,
                   const double2* __restrict__ lg, const double2* __restrict__ lcs,
                   const double2* __restrict__ gpart, const double2* __restrict__ l2part,
                   double2* __restrict__ energy, const int* __restrict__ status) {
  __shared__ double2 red[32];
  const int b = blockIdx.x;
  if (status[0] != 0) {  // a tensor-core product of this call timed out: no numbers
    const double nan = __longlong_as_double(0x7FF8000000000000ll);
    if (threadIdx.x == 0) energy[b] = cmk(nan, nan);
    return;
  }
  double2 lglg = cmk(0.0, 0.0), lslg = cmk(0.0, 0.0);
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double2 x = lg[(size_t)b * G + g];
    cfma(lglg, x, x);
    cfma(lslg, lcs[(size_t)b * G + g], x);
  }
  double2 p[4] = {cmk(0.0, 0.0), cmk(0.0, 0.0), cmk(0.0, 0.0), cmk(0.0, 0.0)};
  for (int c = threadIdx.x; c < nchunk; c += blockDim.x)
    for (int k = 0; k < 4; ++k) p[k] = cadd(p[k], gpart[((size_t)b * nchunk + c) * 4 + k]);
  lglg = block_sum2(lglg, red);
  lslg = block_sum2(lslg, red);
  for (int k = 0; k < 4; ++k) p[k] = block_sum2(p[k], red);
  if (threadIdx.x == 0) {
    const double2 ci1g = wsc[(size_t)b * 8 + 0], gci2g = wsc[(size_t)b * 8 + 1];
    const double2 e1_1_2 = wsc[(size_t)b * 8 + 2], e1_2_2 = wsc[(size_t)b * 8 + 3];
    double2 l2ci2 = cmk(0.0, 0.0);
    for (int c = 0; c < kL2Parts; ++c) l2ci2 = cadd(l2ci2, l2part[(size_t)b * kL2Parts + c]);
    const double2 hg = hg2[b];  // 2 hg
    // one body
    const double2 e1 = cadd(cadd(cadd(hg, cmul(cscale(ci1g, 2.0), hg)), e1_1_2),
                            cadd(cmul(hg, gci2g), e1_2_2));
    // two body; the lci1g . lg terms (2 e2_1_2 = -4 lci1g . lg) and the lci2g . lg term
    // (4 e2_2_2_1 = -4 lci2g . lg) are summed as -4 lcs . lg
    const double2 e2_0 = csub(cscale(lglg, 2.0), p[0]);
    const double2 e2_1 = cadd(cmul(cscale(e2_0, 2.0), ci1g), cscale(csub(p[1], p[2]), 2.0));
    const double2 e2_2 = cadd(cadd(cmul(e2_0, gci2g), cscale(p[3], 2.0)), l2ci2);
    const double2 e2 = cadd(cadd(cadd(e2_0, e2_1), e2_2), cscale(lslg, -4.0));
    const double2 ov = cmk(1.0 + 2.0 * ci1g.x + gci2g.x, 2.0 * ci1g.y + gci2g.y);
    const double2 e = cdiv(cadd(e1, e2), ov);
    energy[b] = cmk(e.x + h0, e.y);
  }
}

// ------------------------------------------------------------------ orchestration
static size_t cisd_mats_smem(int N, int n, int v) { return (size_t)(n * N + n * v + 2 * N * n) * sizeof(double2); }
static size_t cisd_gamma_smem(int N, int n) {
  return (size_t)(2 * n * N + N * N + 2 * n * n) * sizeof(double2) + (size_t)N * N * sizeof(double);
}

static size_t cisd_gamma_f32_smem(int N, int n) {
  // GsT, C1, AT (complex float-float, rows padded to n + 1), A + RdT (padded), Lc (float-float)
  // + Gf, P2f, GLf (float2)
  const size_t ns = (size_t)n + 1;
  return (N * ns + 2 * n * ns + (size_t)n * n) * 16 + (N * ns + (size_t)N * n) * 8 +
         (size_t)(3 * n * N) * sizeof(float2);
}

// need_ham: the force bias / energy / step also read h1, chol and lci1
static int check_cisd(const trot_cisd* c, int W, bool need_ham = true) {
  if (!c) { set_error("null CISD context"); return TROT_ERR_NULL_PTR; }
  if (W <= 0 || W > 65535 || c->norb <= 0 || c->nocc <= 0 || c->nvir <= 0 || c->nocc + c->nvir != c->norb ||
      c->nchol <= 0) {
    set_error("bad CISD sizes W=%d N=%d n=%d v=%d G=%d (need nocc + nvir == norb)", W, c->norb, c->nocc, c->nvir,
              c->nchol);
    return TROT_ERR_BAD_SHAPE;
  }
  if (!c->ci1 || !c->ci2m || !c->mo || (need_ham && (!c->h1 || !c->chol || !c->lci1))) {
    set_error("null CISD context array");
    return TROT_ERR_NULL_PTR;
  }
  if ((c->l2ci2_precision != TROT_FP64 && c->l2ci2_precision != TROT_MIXED) ||
      (c->gl_precision != TROT_FP64 && c->gl_precision != TROT_MIXED)) {
    set_error("CISD: bad precision selector");
    return TROT_ERR_BAD_DTYPE;
  }
  if (need_ham && c->l2ci2_precision == TROT_MIXED) {
    const int nv = c->nocc * c->nvir;
    if (!c->ci2_image) { set_error("CISD: mixed l2ci2 needs ci2_image"); return TROT_ERR_NULL_PTR; }
    if (c->nvpad < nv || c->nvpad % 64 || c->ncpad < nv || c->ncpad % 128) {
      set_error("CISD: ci2_image padding nvpad=%d ncpad=%d for nocc*nvir=%d", c->nvpad, c->ncpad, nv);
      return TROT_ERR_BAD_SHAPE;
    }
  }
  if (c->nocc > 64 || cisd_mats_smem(c->norb, c->nocc, c->nvir) > 200 * 1024 ||
      cisd_gamma_smem(c->norb, c->nocc) > 200 * 1024 ||
      (c->gl_precision == TROT_MIXED && cisd_gamma_f32_smem(c->norb, c->nocc) > 200 * 1024)) {
    set_error("CISD tile of N=%d, n=%d exceeds shared memory", c->norb, c->nocc);
    return TROT_ERR_UNSUPPORTED;
  }
  return TROT_OK;
}

static Spins cisd_spins(const trot_cisd* c) {
  Spins sp{};
  sp.nspin = 1;
  sp.n[0] = c->nocc;
  sp.mult[0] = 2;
  sp.off[0] = 0;
  sp.off[1] = c->nocc;
  sp.ntot = c->nocc;
  sp.mo[0] = c->mo;
  sp.rot_h1[0] = c->h1;  // rows [0, n) of h1: 2 sum G o h1[:n, :] = 2 hg
  sp.rot_chol[0] = nullptr;
  return sp;
}

// one timed kernel launch: CISD_LAUNCH("name", kernel, grid, block, smem, stream, args...)
#define CISD_LAUNCH(name, kernel, grid, block, smem, st, ...)   \
  TROT_TIMED(name, st, ([&]() -> int {                          \
    kernel<<<grid, block, smem, st>>>(__VA_ARGS__);             \
    TROT_CHECK_LAUNCH(name);                                    \
    return TROT_OK;                                             \
  })())

// green, x, C_c / C_e, scalars; stage 0 = overlap only, 1 = + N x N matrices and chol contractions, 2 = + energy terms
static int cisd_run(const trot_cisd* c, int W, const double2* w, CisdBuffers& b, int stage, cudaStream_t st) {
  const int N = c->norb, n = c->nocc, v = c->nvir, G = c->nchol, nv = n * v;
  Spins sp = cisd_spins(c);
  if (stage > 0) cudaMemsetAsync(b.status, 0, sizeof(int), st);  // this call's word; the sticky one persists
  TROT_TIMED("cisd_green", st, launch_green(sp, W, N, w, nullptr, b.green, b.det2, b.hg2, st));
  CISD_LAUNCH("cisd_x", cisd_x_kernel, W, 256, 0, st, N, n, v, b.green, c->ci1, b.x,
              stage >= 1 ? b.ci1g1 : nullptr, b.wsc);
  TROT_TIMED("cisd_ci2g", st,
             launch_zgemm_cr_splitk(W, nv, nv, 1.0, b.x, nv, c->ci2m, nv, false, b.cg, nv, false, b.kpart,
                                    cisd_splitk(W, nv, nv), st));
  if (stage == 0) return TROT_OK;
  const size_t smem = cisd_mats_smem(N, n, v);
  if (smem > 40 * 1024) cudaFuncSetAttribute(cisd_mats_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  CISD_LAUNCH("cisd_mats", cisd_mats_kernel, W, 256, smem, st, N, n, v, b.green, c->ci1, b.cg, b.x, c->h1, b.ms,
              b.m2, b.p2, b.wsc);
  // lg = rot_chol . G  (rot_chol rows g: chol[g][:n][:] = first n N entries of chol_flat row g)
  TROT_TIMED("cisd_chol_gemm", st,
             launch_zgemm_cr_splitk(W, G, n * N, 1.0, b.green, n * N, c->chol, N * N, true, b.lg, G, false, b.kpart,
                                    cisd_splitk(W, G, n * N), st));
  // lcs = (ci1_green + ci2_green) . chol^T: one (W, N^2) x (N^2, G) FP64 product, over the packed
  // upper triangle when every chol[g] is symmetric.
  // (FP32-class products here, as the reference's mixed_real_dtype contraction, move
  // the local energy by ~1e-3 Ha at N=60, G=300: too far from FP64.)
  if (c->chol_symmetric) {
    const int P = N * (N + 1) / 2;
    const size_t gnn = (size_t)G * N * N, wnn = (size_t)W * N * N;
    CISD_LAUNCH("cisd_lci_gemm", cisd_pack_chol_kernel, (unsigned)std::min<size_t>((gnn + 255) / 256, 152 * 16), 256,
                0, st, N, G, c->chol, b.lp);
    CISD_LAUNCH("cisd_lci_gemm", cisd_pack_ms_kernel, (unsigned)std::min<size_t>((wnn + 255) / 256, 152 * 16), 256, 0,
                st, N, W, b.ms, b.msp);
    TROT_TIMED("cisd_lci_gemm", st,
               launch_zgemm_cr_splitk(W, G, P, 1.0, b.msp, P, b.lp, P, true, b.lcs, G, false, b.kpart,
                                      cisd_splitk(W, G, P), st));
  } else {
    TROT_TIMED("cisd_lci_gemm", st,
               launch_zgemm_cr_splitk(W, G, N * N, 1.0, b.ms, N * N, c->chol, N * N, true, b.lcs, G, false,
                                      b.kpart, cisd_splitk(W, G, N * N), st));
  }
  if (stage == 1) return TROT_OK;
  const int nch = cisd_chunks(G);
  if (c->gl_precision == TROT_MIXED) {
    const size_t smem2 = cisd_gamma_f32_smem(N, n);
    cudaFuncSetAttribute(cisd_gamma_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
    const size_t gnn = (size_t)G * N * n;
    CISD_LAUNCH("cisd_chol_forms", cisd_chol_forms_kernel, (unsigned)std::min<size_t>((gnn + 255) / 256, 152 * 16),
                256, 0, st, N, n, G, c->chol, c->lci1, b.rd, b.lc);
    // gl = G L_g for all walkers and Cholesky vectors: one split-BF16 tensor-core product
    // (FP32-class, the reference's float32 gl), rows (walker, p), columns (g, j)
    const int kp = (int)cisd_gl_kpad(N), np = (int)cisd_gl_npad(N, G);
    const size_t nimg = (size_t)np * kp;
    CISD_LAUNCH("cisd_gl_tc", cisd_gl_image_kernel, (unsigned)std::min<size_t>((nimg + 255) / 256, 152 * 16), 256, 0,
                st, N, G, kp, np, c->chol, b.glimg);
    TROT_TIMED("cisd_gl_tc", st, launch_split3_gemm(W * n, N, kp, np, b.green, b.glimg, b.glq, b.gld, b.status, st));
    CISD_LAUNCH("cisd_gamma_f32", cisd_gamma_f32_kernel, dim3(nch, W), 256, smem2, st, N, n, v, G, b.green, b.gld, np,
                b.rd, b.lc, b.p2, b.ci1g1, b.xg, b.gpart);
  } else {
    const size_t smem2 = cisd_gamma_smem(N, n);
    cudaFuncSetAttribute(cisd_gamma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
    CISD_LAUNCH("cisd_gamma", cisd_gamma_kernel, dim3(nch, W), 256, smem2, st, N, n, v, G, b.green, c->chol, c->lci1,
                b.m2, b.ci1g1, b.xg, b.gpart);
  }
  if (c->l2ci2_precision == TROT_MIXED) {
    TROT_TIMED("cisd_l2ci2_tc", st,
               launch_split3_gemm(W * G, nv, c->nvpad, c->ncpad, b.xg, c->ci2_image, b.xq, b.yd, b.status, st));
    CISD_LAUNCH("cisd_l2_reduce", cisd_l2_reduce_tc_kernel, dim3(kL2Parts, W), 256, 0, st, G, nv, c->ncpad, b.xg,
                b.yd, b.l2part);
    return TROT_OK;
  }
  if ((size_t)W * G > 65535u * 64u) { set_error("CISD: W*G too large"); return TROT_ERR_UNSUPPORTED; }
  TROT_TIMED("cisd_l2ci2", st,
             launch_zgemm_cr(W * G, nv, nv, 1.0, b.xg, nv, c->ci2m, nv, false, b.y, nv, false, st));
  CISD_LAUNCH("cisd_l2_reduce", cisd_l2_reduce_kernel, dim3(kL2Parts, W), 256, 0, st, G, nv, b.xg, b.y, b.l2part);
  return TROT_OK;
}

}  // namespace trot

using namespace trot;

extern "C" {

size_t trot_cisd_workspace_size(const trot_cisd* c, int n_walkers, int op) {
  if (check_cisd(c, n_walkers, false) != TROT_OK) return 0;
  if (op != TROT_OP_OVERLAP && op != TROT_OP_FORCE_BIAS && op != TROT_OP_LOCAL_ENERGY && op != TROT_OP_PROP_STEP) {
    set_error("CISD workspace: unsupported op %d", op);
    return 0;
  }
  Carver cv(nullptr, 0);
  CisdBuffers b;
  return carve_cisd(c, n_walkers, op, cv, b) + 256;
}

int trot_cisd_overlap(const trot_cisd* c, int W, const double* walkers, double* out, void* ws, size_t ws_bytes,
                      void* stream) {
  TROT_TRY(check_cisd(c, W, false));
  if (!walkers || !out) { set_error("null walkers or output"); return TROT_ERR_NULL_PTR; }
  Carver cv(ws, ws_bytes);
  CisdBuffers b;
  carve_cisd(c, W, TROT_OP_OVERLAP, cv, b);
  if (!cv.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, cv.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  TROT_TRY(cisd_run(c, W, (const double2*)walkers, b, 0, st));
  cisd_overlap_kernel<<<W, 256, 0, st>>>(c->nocc * c->nvir, b.x, b.cg, b.wsc, b.det2, (double2*)out);
  TROT_CHECK_LAUNCH("cisd_overlap_kernel");
  return TROT_OK;
}

int trot_cisd_force_bias(const trot_cisd* c, int W, const double* walkers, double* out, void* ws, size_t ws_bytes,
                         void* stream) {
  TROT_TRY(check_cisd(c, W));
  if (!walkers || !out) { set_error("null walkers or output"); return TROT_ERR_NULL_PTR; }
  Carver cv(ws, ws_bytes);
  CisdBuffers b;
  carve_cisd(c, W, TROT_OP_FORCE_BIAS, cv, b);
  if (!cv.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, cv.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  TROT_TRY(cisd_run(c, W, (const double2*)walkers, b, 1, st));
  const size_t n = (size_t)W * c->nchol;
  cisd_fb_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(W, c->nchol, b.wsc, b.lg, b.lcs, (double2*)out);
  TROT_CHECK_LAUNCH("cisd_fb_kernel");
  return TROT_OK;
}

int trot_cisd_local_energy(const trot_cisd* c, int W, const double* walkers, double* out, void* ws,
                           size_t ws_bytes, void* stream) {
  TROT_TRY(check_cisd(c, W));
  if (!walkers || !out) { set_error("null walkers or output"); return TROT_ERR_NULL_PTR; }
  Carver cv(ws, ws_bytes);
  CisdBuffers b;
  carve_cisd(c, W, TROT_OP_LOCAL_ENERGY, cv, b);
  if (!cv.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, cv.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  TROT_TRY(cisd_run(c, W, (const double2*)walkers, b, 2, st));
  cisd_energy_kernel<<<W, 256, 0, st>>>(c->nchol, cisd_chunks(c->nchol), c->h0, b.wsc, b.hg2, b.lg, b.lcs,
                                        b.gpart, b.l2part, (double2*)out, b.status);
  TROT_CHECK_LAUNCH("cisd_energy_kernel");
  return TROT_OK;
}

int trot_cisd_rdm1(const trot_cisd* c, int W, const double* walkers, double* out, void* ws, size_t ws_bytes,
                   void* stream) {
  TROT_TRY(check_cisd(c, W));
  if (!walkers || !out) { set_error("null walkers or output"); return TROT_ERR_NULL_PTR; }
  Carver cv(ws, ws_bytes);
  CisdBuffers b;
  carve_cisd(c, W, TROT_OP_FORCE_BIAS, cv, b);
  if (!cv.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, cv.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  TROT_TRY(cisd_run(c, W, (const double2*)walkers, b, 1, st));
  const int N = c->norb;
  cisd_rdm1_kernel<<<dim3((N * N + 255) / 256, W), 256, 0, st>>>(N, c->nocc, b.green, b.ms, b.wsc,
                                                                (double2*)out);
  TROT_CHECK_LAUNCH("cisd_rdm1_kernel");
  return TROT_OK;
}

/* One phaseless step with the CISD trial (trot/prop/afqmc.py:79-144 with the
 * CISD meas ops): force bias and optional local energy of the incoming
 * walkers, shifted fields, VHS, Taylor propagation with one-body half steps
 * (FP64), CISD overlaps of the new walkers, phaseless weights, population
 * shift.  `prop` supplies the propagation context (TROT_RHF_R, FP64). */
int trot_cisd_prop_step(const trot_cisd* c, const trot_system* prop, const trot_state* state, const double* fields,
                        double* energy_out, void* ws, size_t ws_bytes, void* stream) {
  if (!prop || !state || !fields) { set_error("null system, state or fields"); return TROT_ERR_NULL_PTR; }
  const int W = prop->n_walkers;
  TROT_TRY(check_cisd(c, W));
  if (prop->kind != TROT_RHF_R || prop->norb != c->norb || prop->nchol != c->nchol || prop->nocc_a != c->nocc) {
    set_error("CISD step: propagation context must be restricted with norb %d, nchol %d, nocc %d", c->norb,
              c->nchol, c->nocc);
    return TROT_ERR_BAD_SHAPE;
  }
  if (prop->precision != TROT_FP64 && !(prop->precision == TROT_MIXED && prop->mixed)) {
    set_error("CISD step: propagation precision must be FP64, or mixed with a trot_mixed context");
    return TROT_ERR_BAD_DTYPE;
  }
  if (!prop->exp_h1_half || !prop->chol_flat || !prop->mf_shifts_im) {
    set_error("CISD step: null propagation context array");
    return TROT_ERR_NULL_PTR;
  }
  if (prop->n_exp_terms < 1 || prop->n_exp_terms > 16) { set_error("bad n_exp_terms"); return TROT_ERR_BAD_SHAPE; }
  if (!state->walkers_a || !state->weights || !state->overlaps || !state->scalars || !state->node_encounters) {
    set_error("null state buffer");
    return TROT_ERR_NULL_PTR;
  }
  Carver cv(ws, ws_bytes);
  CisdBuffers b;
  carve_cisd(c, W, TROT_OP_PROP_STEP, cv, b);
  if (!cv.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, cv.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  // mixed propagation: the tensor-core Trotter path gets its own workspace after the CISD buffers
  const size_t cisd_bytes = (cv.used + 255) & ~(size_t)255;
  size_t prop_bytes = 0;
  if (prop->precision == TROT_MIXED) {
    prop_bytes = trot_workspace_size(prop, TROT_OP_APPLY_TROTTER);
    if (prop_bytes == 0) return TROT_ERR_BAD_SHAPE;
    if (cisd_bytes + prop_bytes > ws_bytes) {
      set_error("workspace too small: %zu < %zu", ws_bytes, cisd_bytes + prop_bytes);
      return TROT_ERR_WORKSPACE_TOO_SMALL;
    }
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int N = c->norb, G = c->nchol;
  double2* w = (double2*)state->walkers_a;
  // 1. force bias (and local energy) of the incoming walkers
  TROT_TRY(cisd_run(c, W, w, b, energy_out ? 2 : 1, st));
  const size_t wg = (size_t)W * G;
  CISD_LAUNCH("cisd_fb", cisd_fb_kernel, (unsigned)((wg + 255) / 256), 256, 0, st, W, G, b.wsc, b.lg, b.lcs,
              b.fb);
  if (energy_out)
    CISD_LAUNCH("cisd_energy", cisd_energy_kernel, W, 256, 0, st, G, cisd_chunks(G), c->h0, b.wsc, b.hg2, b.lg,
                b.lcs, b.gpart, b.l2part, (double2*)energy_out, b.status);
  // 2. shifted fields, 3. VHS, 4. propagation in place
  TROT_TIMED("fields", st,
             launch_fields(W, G, prop->sqrt_dt, b.fb, prop->mf_shifts_im, fields, b.xs, b.shift_term, b.fb_term, st));
  Spins sp = make_spins(prop);
  TrotterArgs a{};
  a.W = W; a.N = N; a.G = G; a.nterms = prop->n_exp_terms; a.sqrt_dt = prop->sqrt_dt; a.expH = prop->exp_h1_half;
  a.in_a = w; a.out_a = w;
  if (prop->precision == TROT_MIXED) {
    TROT_TRY(trot_apply_trotter(prop, (const double*)w, nullptr, (const double*)b.xs, (double*)w, nullptr,
                                static_cast<char*>(ws) + cisd_bytes, ws_bytes - cisd_bytes, stream));
    // the propagation's status block sits at the start of its workspace region
    TROT_TRY(launch_status_merge(reinterpret_cast<const int*>(static_cast<char*>(ws) + cisd_bytes), b.status, st));
  } else {
    TROT_TIMED("vhs_fp64", st,
               launch_zgemm_cr(W, N * N, G, 1.0, b.xs, G, prop->chol_flat, N * N, false, b.vhs, N * N, false, st));
    a.vhs = b.vhs;
    TROT_TIMED("trotter_fp64", st, launch_trotter(sp, a, st));
  }
  // 5. CISD overlaps of the new walkers, weights, population shift
  TROT_TRY(cisd_run(c, W, w, b, 0, st));
  CISD_LAUNCH("cisd_overlap", cisd_overlap_kernel, W, 256, 0, st, c->nocc * c->nvir, b.x, b.cg, b.wsc, b.det2,
              b.ov_new);
  a.overlaps = (double2*)state->overlaps; a.weights = state->weights; a.scalars = state->scalars;
  a.shift_term = b.shift_term; a.fb_term = b.fb_term; a.node_flag = b.node_flag;
  a.dt = prop->dt; a.h0_prop = prop->h0_prop; a.w_floor = prop->weight_floor; a.w_cap = prop->weight_cap;
  CISD_LAUNCH("cisd_weight", cisd_weight_kernel, (W + 127) / 128, 128, 0, st, a, b.ov_new);
  TROT_TIMED("step_finalize", st,
             launch_step_finalize(W, state->weights, state->scalars, (long long*)state->node_encounters, b.node_flag,
                                  prop->pop_control_damping, prop->dt, st, b.status));
  return TROT_OK;
}

}  // extern "C"
