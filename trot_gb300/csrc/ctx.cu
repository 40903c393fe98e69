// One-time propagation and measurement constants on the device.
//
// Propagation context (trot/runtime_layout.py:125-197, the host twin of
// trot/prop/chol_afqmc_ops.py:103-127), with rho the spin-summed trial 1-RDM:
//   t_g        = sum_ij L_g[i][j] rho[j][i]          (mf_shifts = i t_g)
//   h0_prop    = -h0 - 1/2 sum_g mf_g^2 = -h0 + 1/2 sum_g t_g^2
//   h1_eff     = h1 - 1/2 sum_g L_g L_g + sum_g t_g L_g
//   exp_h1_half = expm(-dt/2 h1_eff)
// The matrix exponential is scaling and squaring of a degree-16 Taylor
// polynomial: s = the smallest power of two with ||A||_1 / 2^s <= 1/2, the
// Taylor sum of B = A / 2^s by Horner's rule (remainder < 0.5^17 / 17! ~ 2e-20
// relative), then s squarings.  s is chosen on the device, so the launches are a
// fixed sequence (no host round trip; squarings past s return at once).
//
// Half rotation (trot/runtime_layout.py:200-245; trot/meas/rhf.py:308-319):
//   rot_h1 = C^T h1 (n, N),  rot_chol[g] = C^T L_g (n, N)   for a real trial C (N, n).
// CISD (trot/runtime_layout.py:248-292; trot/meas/cisd.py:92-110):
//   lci1[g][i][p] = sum_t L_g[i][nocc + t] ci1[p][t]   (G, N, nocc).
#include "kernels.h"

namespace trot {

static constexpr int kCtxT = 32;        // output tile of the FP64 matrix products
static constexpr int kTaylorDeg = 16;
static constexpr int kMaxSquarings = 40;

struct CtxBuffers {
  int* status;   // [0] status, [1] number of squarings s
  double *a, *p0, *p1, *part;
};

static void ctx_slices(int N, int G, int& S, int& gper) {
  const int tiles = ((N + kCtxT - 1) / kCtxT) * ((N + kCtxT - 1) / kCtxT);
  S = (2 * 152 + tiles - 1) / tiles;
  if (S > G) S = G;
  if (S < 1) S = 1;
  gper = (G + S - 1) / S;
  S = (G + gper - 1) / gper;
}

static size_t carve_ctx(int N, int G, Carver& c, CtxBuffers& b) {
  int S, gper;
  ctx_slices(N, G, S, gper);
  const size_t nn = (size_t)N * N;
  b.status = c.status();  // 64 ints
  b.a = c.take<double>(nn);
  b.p0 = c.take<double>(nn);
  b.p1 = c.take<double>(nn);
  b.part = c.take<double>((size_t)S * nn);
  return c.used;
}

// t_g = sum_ij L_g[i][j] rho[j][i]; one block per g, fixed-order reduction
__global__ void ctx_mf_kernel(int N, const double* __restrict__ chol, const double* __restrict__ rho,
                              double* __restrict__ t) {
  __shared__ double2 red[32];
  const int g = blockIdx.x;
  const double* L = chol + (size_t)g * N * N;
  double acc = 0.0;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    const int i = e / N, j = e - i * N;
    acc = fma(L[e], rho[(size_t)j * N + i], acc);
  }
  const double2 s = block_sum2(cmk(acc, 0.0), red);
  if (threadIdx.x == 0) t[g] = s.x;
}

// h0_prop = -h0 + 1/2 sum_g t_g^2
__global__ void ctx_h0_kernel(int G, double h0, const double* __restrict__ t, double* __restrict__ h0_prop) {
  __shared__ double2 red[32];
  double acc = 0.0;
  for (int g = threadIdx.x; g < G; g += blockDim.x) acc = fma(t[g], t[g], acc);
  const double2 s = block_sum2(cmk(acc, 0.0), red);
  if (threadIdx.x == 0) *h0_prop = -h0 + 0.5 * s.x;
}

// part[s][i][j] = sum_{g in slice s} (t_g L_g[i][j] - 1/2 sum_k L_g[i][k] L_g[k][j]);
// grid (j tiles, i tiles, slices), 256 threads: thread (ty, tx) owns rows ty + 8r of column tx.
__global__ void __launch_bounds__(256) ctx_v_partial_kernel(int N, int G, int gper, const double* __restrict__ chol,
                                                            const double* __restrict__ t, double* __restrict__ part) {
  __shared__ double As[kCtxT][kCtxT + 1], Bs[kCtxT][kCtxT + 1];
  const int j0 = blockIdx.x * kCtxT, i0 = blockIdx.y * kCtxT, sl = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double quad[4] = {0.0, 0.0, 0.0, 0.0}, lin[4] = {0.0, 0.0, 0.0, 0.0};
  const int g0 = sl * gper, g1 = min(G, g0 + gper);
  for (int g = g0; g < g1; ++g) {
    const double* L = chol + (size_t)g * N * N;
    for (int k0 = 0; k0 < N; k0 += kCtxT) {
#pragma unroll
      for (int r = ty; r < kCtxT; r += 8) {
        const int i = i0 + r, k = k0 + tx, kk = k0 + r, j = j0 + tx;
        As[r][tx] = (i < N && k < N) ? L[(size_t)i * N + k] : 0.0;
        Bs[r][tx] = (kk < N && j < N) ? L[(size_t)kk * N + j] : 0.0;
      }
      __syncthreads();
#pragma unroll 8
      for (int k = 0; k < kCtxT; ++k) {
        const double bv = Bs[k][tx];
#pragma unroll
        for (int r = 0; r < 4; ++r) quad[r] = fma(As[ty + 8 * r][k], bv, quad[r]);
      }
      __syncthreads();
    }
    const double tg = t[g];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = i0 + ty + 8 * r, j = j0 + tx;
      if (i < N && j < N) lin[r] = fma(tg, L[(size_t)i * N + j], lin[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty + 8 * r, j = j0 + tx;
    if (i < N && j < N) part[((size_t)sl * N + i) * N + j] = lin[r] - 0.5 * quad[r];
  }
}

// A = -dt/2 (h1 + sum_s part[s]) in slice order
__global__ void ctx_heff_kernel(int N, int S, double dt, const double* __restrict__ h1, const double* __restrict__ part,
                                double* __restrict__ A) {
  const size_t nn = (size_t)N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x) {
    double v = h1[e];
    for (int s = 0; s < S; ++s) v += part[(size_t)s * nn + e];
    A[e] = -0.5 * dt * v;
  }
}

// P = I (Horner's starting value)
__global__ void ctx_eye_kernel(int n, double* __restrict__ P) {
  const size_t nn = (size_t)n * n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x)
    P[e] = (e / n == e % n) ? 1.0 : 0.0;
}

// ||A||_1 (max column sum) -> number of squarings; status on a non-finite or huge norm
__global__ void ctx_norm_kernel(int N, const double* __restrict__ A, int* __restrict__ status) {
  __shared__ double red[256];
  double m = 0.0;
  bool finite = true;
  for (int j = threadIdx.x; j < N; j += blockDim.x) {
    double c = 0.0;
    for (int i = 0; i < N; ++i) c += fabs(A[(size_t)i * N + j]);
    if (!(c <= 1.7e308)) finite = false;  // NaN or inf
    m = fmax(m, c);
  }
  red[threadIdx.x] = finite ? m : -1.0;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double x = red[threadIdx.x], y = red[threadIdx.x + o];
      red[threadIdx.x] = (x < 0.0 || y < 0.0) ? -1.0 : fmax(x, y);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double nrm = red[0];
    int s = 0;
    if (nrm < 0.0) {
      status[0] = TROT_ERR_NUMERIC_GUARD;
    } else {
      while (nrm > 0.5 && s < kMaxSquarings) { nrm *= 0.5; ++s; }
      if (nrm > 0.5) status[0] = TROT_ERR_NUMERIC_GUARD;
    }
    status[1] = s;
  }
}

// mode 0 (Horner): Z = I + (A Y) * (2^-s * kinv);  mode 1 (squaring number q): Z = Y Y if q < s.
// grid (j tiles, i tiles), 256 threads.
__global__ void __launch_bounds__(256) ctx_gemm_kernel(int N, int mode, int q, double kinv,
                                                       const double* __restrict__ A, const double* __restrict__ Y,
                                                       double* __restrict__ Z, const int* __restrict__ status) {
  const int s = status[1];
  if (mode == 1 && q >= s) return;
  const double* X = mode == 0 ? A : Y;
  __shared__ double As[kCtxT][kCtxT + 1], Bs[kCtxT][kCtxT + 1];
  const int j0 = blockIdx.x * kCtxT, i0 = blockIdx.y * kCtxT;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < N; k0 += kCtxT) {
#pragma unroll
    for (int r = ty; r < kCtxT; r += 8) {
      const int i = i0 + r, k = k0 + tx, kk = k0 + r, j = j0 + tx;
      As[r][tx] = (i < N && k < N) ? X[(size_t)i * N + k] : 0.0;
      Bs[r][tx] = (kk < N && j < N) ? Y[(size_t)kk * N + j] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < kCtxT; ++k) {
      const double bv = Bs[k][tx];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] = fma(As[ty + 8 * r][k], bv, acc[r]);
    }
    __syncthreads();
  }
  const double scale = mode == 0 ? ldexp(kinv, -s) : 1.0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty + 8 * r, j = j0 + tx;
    if (i < N && j < N) Z[(size_t)i * N + j] = (mode == 0 ? (i == j ? 1.0 : 0.0) : 0.0) + acc[r] * scale;
  }
}

// exp_h1_half = P[s & 1] (Horner leaves its sum in P0; squaring q reads P[q & 1])
__global__ void ctx_final_kernel(int N, const double* __restrict__ P0, const double* __restrict__ P1,
                                 const int* __restrict__ status, double* __restrict__ out) {
  const double* P = (status[1] & 1) ? P1 : P0;
  const size_t nn = (size_t)N * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nn; e += (size_t)gridDim.x * blockDim.x)
    out[e] = P[e];
}

// out[g][p][j] = sum_i C[i][p] M_g[i][j] for p in [p0, p0 + 16): grid (G, ceil(n / 16)), 128 threads
// over j; C rows staged in shared memory 128 at a time.
__global__ void __launch_bounds__(128) ctx_rotate_kernel(int N, int n, const double* __restrict__ C,
                                                         const double* __restrict__ M, double* __restrict__ out) {
  __shared__ double Cs[128][16];
  const int g = blockIdx.x, p0 = blockIdx.y * 16;
  const int np = min(16, n - p0);
  const double* Mg = M + (size_t)g * N * N;
  double* og = out + (size_t)g * n * N;
  for (int jb = 0; jb < N; jb += 128) {
    const int j = jb + threadIdx.x;
    double acc[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) acc[q] = 0.0;
    for (int ib = 0; ib < N; ib += 128) {
      const int ni = min(128, N - ib);
      __syncthreads();
      for (int e = threadIdx.x; e < 128 * 16; e += 128) {
        const int r = e >> 4, q = e & 15;
        Cs[r][q] = (r < ni && q < np) ? C[(size_t)(ib + r) * n + p0 + q] : 0.0;
      }
      __syncthreads();
      if (j < N) {
        for (int r = 0; r < ni; ++r) {
          const double m = Mg[(size_t)(ib + r) * N + j];
#pragma unroll
          for (int q = 0; q < 16; ++q) acc[q] = fma(Cs[r][q], m, acc[q]);
        }
      }
    }
    if (j < N) {
#pragma unroll
      for (int q = 0; q < 16; ++q)
        if (q < np) og[(size_t)(p0 + q) * N + j] = acc[q];
    }
  }
}

// lci1[g][i][p] = sum_t L_g[i][nocc + t] ci1[p][t]; one block per g, threads over (i, p)
__global__ void ctx_lci1_kernel(int N, int nocc, const double* __restrict__ ci1, const double* __restrict__ chol,
                                double* __restrict__ lci1) {
  const int g = blockIdx.x, nv = N - nocc;
  const double* L = chol + (size_t)g * N * N;
  for (int e = threadIdx.x; e < N * nocc; e += blockDim.x) {
    const int i = e / nocc, p = e - i * nocc;
    double acc = 0.0;
    for (int t = 0; t < nv; ++t) acc = fma(L[(size_t)i * N + nocc + t], ci1[(size_t)p * nv + t], acc);
    lci1[((size_t)g * N + i) * nocc + p] = acc;
  }
}

// M (2N x 2N) = [[A^T, Gb], [0, A^T]]: expm(M)'s upper-right block is the
// adjoint of the Frechet derivative of expm at A applied to Gb (for the
// Frobenius inner product the adjoint of L(A, .) is L(A^T, .); Higham,
// "Functions of Matrices", 2008, Thm. 3.6 and sec. 3.2).
// The upper-right block is linear in Gb: it is scaled to max |Gb| = 1 (keeping
// ||M||_1 and so the number of squarings small) and scaled back on the way out.
__global__ void ctx_absmax_kernel(size_t n, const double* __restrict__ x, double* __restrict__ out) {
  __shared__ double red[256];
  double m = 0.0;
  for (size_t e = threadIdx.x; e < n; e += blockDim.x) m = fmax(m, fabs(x[e]));
  red[threadIdx.x] = m;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + o]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] > 0.0 ? red[0] : 1.0;
}

__global__ void ctx_frechet_build_kernel(int N, const double* __restrict__ A, const double* __restrict__ Gb,
                                         const double* __restrict__ gscale, double* __restrict__ M) {
  const int n2 = 2 * N;
  const double inv = 1.0 / *gscale;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)n2 * n2;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n2), j = (int)(e % n2);
    double v = 0.0;
    if (i < N && j < N) v = A[(size_t)j * N + i];
    else if (i < N) v = Gb[(size_t)i * N + (j - N)] * inv;
    else if (j >= N) v = A[(size_t)(j - N) * N + (i - N)];
    M[e] = v;
  }
}

// g_h1[i][j] += scale * gscale * E[i][N + j]
__global__ void ctx_frechet_take_kernel(int N, const double* __restrict__ E, double scale,
                                        const double* __restrict__ gscale, double* __restrict__ g) {
  const double sc = scale * *gscale;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < (size_t)N * N;
       e += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / N), j = (int)(e % N);
    g[e] += sc * E[(size_t)i * 2 * N + N + j];
  }
}

// out = expm(A) for a real n x n matrix on the device; status[0] is set to
// TROT_ERR_NUMERIC_GUARD on a non-finite or huge norm, status[1] receives s.
// p0, p1: n x n scratch.  Used by the propagation context and its adjoint.
int launch_expm(int n, const double* A, double* out, double* p0, double* p1, int* status, cudaStream_t st) {
  const size_t nn = (size_t)n * n;
  const int eb = (int)((nn + 255) / 256 < 1024 ? (nn + 255) / 256 : 1024);
  const int nt = (n + kCtxT - 1) / kCtxT;
  ctx_norm_kernel<<<1, 256, 0, st>>>(n, A, status);
  TROT_CHECK_LAUNCH("ctx_norm_kernel");
  ctx_eye_kernel<<<eb, 256, 0, st>>>(n, p0);
  TROT_CHECK_LAUNCH("ctx_eye_kernel");
  double* P[2] = {p0, p1};
  // Horner: T <- I + B T / k for k = 16 .. 1, ping-pong P0 -> P1 -> ... -> P0 (16 steps)
  for (int idx = 0; idx < kTaylorDeg; ++idx) {
    const int k = kTaylorDeg - idx;
    ctx_gemm_kernel<<<dim3(nt, nt), 256, 0, st>>>(n, 0, 0, 1.0 / k, A, P[idx & 1], P[(idx + 1) & 1], status);
    TROT_CHECK_LAUNCH("ctx_gemm_kernel");
  }
  static_assert((kTaylorDeg & 1) == 0, "Horner must end in P0");
  for (int q = 0; q < kMaxSquarings; ++q) {
    ctx_gemm_kernel<<<dim3(nt, nt), 256, 0, st>>>(n, 1, q, 1.0, nullptr, P[q & 1], P[(q + 1) & 1], status);
    TROT_CHECK_LAUNCH("ctx_gemm_kernel");
  }
  ctx_final_kernel<<<eb, 256, 0, st>>>(n, p0, p1, status, out);
  TROT_CHECK_LAUNCH("ctx_final_kernel");
  return TROT_OK;
}

}  // namespace trot

using namespace trot;

extern "C" {

size_t trot_prop_ctx_workspace_size(int norb, int nchol) {
  if (norb < 1 || nchol < 1) { set_error("bad shape: norb %d, nchol %d", norb, nchol); return 0; }
  Carver c(nullptr, 0);
  CtxBuffers b;
  return carve_ctx(norb, nchol, c, b) + 256;
}

int trot_build_prop_ctx(int norb, int nchol, double h0, double dt, const double* h1, const double* chol,
                        const double* rdm1, double* mf_im, double* h0_prop, double* exp_h1_half, void* ws,
                        size_t ws_bytes, void* stream) {
  if (!h1 || !chol || !rdm1 || !mf_im || !h0_prop || !exp_h1_half || !ws) {
    set_error("null input, output or workspace");
    return TROT_ERR_NULL_PTR;
  }
  if (norb < 1 || nchol < 1) { set_error("bad shape: norb %d, nchol %d", norb, nchol); return TROT_ERR_BAD_SHAPE; }
  if (!(dt > 0.0) || !(dt < 1e300)) { set_error("bad time step %g", dt); return TROT_ERR_BAD_SHAPE; }
  const int N = norb, G = nchol;
  Carver c(ws, ws_bytes);
  CtxBuffers b;
  carve_ctx(N, G, c, b);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  int S, gper;
  ctx_slices(N, G, S, gper);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(b.status, 0, 2 * sizeof(int), st);
  if (e != cudaSuccess) return cuda_status(e, "trot_build_prop_ctx memset");
  ctx_mf_kernel<<<G, 256, 0, st>>>(N, chol, rdm1, mf_im);
  TROT_CHECK_LAUNCH("ctx_mf_kernel");
  ctx_h0_kernel<<<1, 256, 0, st>>>(G, h0, mf_im, h0_prop);
  TROT_CHECK_LAUNCH("ctx_h0_kernel");
  const int nt = (N + kCtxT - 1) / kCtxT;
  ctx_v_partial_kernel<<<dim3(nt, nt, S), 256, 0, st>>>(N, G, gper, chol, mf_im, b.part);
  TROT_CHECK_LAUNCH("ctx_v_partial_kernel");
  const size_t nn = (size_t)N * N;
  const int eb = (int)((nn + 255) / 256 < 1024 ? (nn + 255) / 256 : 1024);
  ctx_heff_kernel<<<eb, 256, 0, st>>>(N, S, dt, h1, b.part, b.a);
  TROT_CHECK_LAUNCH("ctx_heff_kernel");
  TROT_TRY(launch_expm(N, b.a, exp_h1_half, b.p0, b.p1, b.status, st));
  return TROT_OK;
}

size_t trot_prop_ctx_vjp_workspace_size(int norb, int nchol) {
  if (norb < 1 || nchol < 1) { set_error("bad shape: norb %d, nchol %d", norb, nchol); return 0; }
  Carver c(nullptr, 0);
  CtxBuffers b;
  carve_ctx(norb, nchol, c, b);
  const size_t m = (size_t)4 * norb * norb;
  c.take<double>(nchol);      // mean-field traces
  for (int k = 0; k < 4; ++k) c.take<double>(m);  // M, P0, P1, expm(M)
  return c.used + 256;
}

int trot_prop_ctx_vjp(int norb, int nchol, double dt, const double* h1, const double* chol, const double* rdm1,
                      const double* g_exp_h1_half, double* g_h1, void* ws, size_t ws_bytes, void* stream) {
  if (!h1 || !chol || !rdm1 || !g_exp_h1_half || !g_h1 || !ws) {
    set_error("null input, output or workspace");
    return TROT_ERR_NULL_PTR;
  }
  if (norb < 1 || nchol < 1) { set_error("bad shape: norb %d, nchol %d", norb, nchol); return TROT_ERR_BAD_SHAPE; }
  if (!(dt > 0.0) || !(dt < 1e300)) { set_error("bad time step %g", dt); return TROT_ERR_BAD_SHAPE; }
  const int N = norb, G = nchol;
  Carver c(ws, ws_bytes);
  CtxBuffers b;
  carve_ctx(N, G, c, b);
  const size_t m = (size_t)4 * N * N;
  double* t = c.take<double>(G);
  double* M = c.take<double>(m);
  double* q0 = c.take<double>(m);
  double* q1 = c.take<double>(m);
  double* E = c.take<double>(m);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  int S, gper;
  ctx_slices(N, G, S, gper);
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(b.status, 0, 2 * sizeof(int), st);
  if (e != cudaSuccess) return cuda_status(e, "trot_prop_ctx_vjp memset");
  ctx_mf_kernel<<<G, 256, 0, st>>>(N, chol, rdm1, t);
  TROT_CHECK_LAUNCH("ctx_mf_kernel");
  const int nt = (N + kCtxT - 1) / kCtxT;
  ctx_v_partial_kernel<<<dim3(nt, nt, S), 256, 0, st>>>(N, G, gper, chol, t, b.part);
  TROT_CHECK_LAUNCH("ctx_v_partial_kernel");
  const size_t nn = (size_t)N * N;
  const int eb = (int)((nn + 255) / 256 < 1024 ? (nn + 255) / 256 : 1024);
  ctx_heff_kernel<<<eb, 256, 0, st>>>(N, S, dt, h1, b.part, b.a);
  TROT_CHECK_LAUNCH("ctx_heff_kernel");
  const int eb2 = (int)((m + 255) / 256 < 1024 ? (m + 255) / 256 : 1024);
  double* gscale = reinterpret_cast<double*>(b.status + 8);
  ctx_absmax_kernel<<<1, 256, 0, st>>>(nn, g_exp_h1_half, gscale);
  TROT_CHECK_LAUNCH("ctx_absmax_kernel");
  ctx_frechet_build_kernel<<<eb2, 256, 0, st>>>(N, b.a, g_exp_h1_half, gscale, M);
  TROT_CHECK_LAUNCH("ctx_frechet_build_kernel");
  TROT_TRY(launch_expm(2 * N, M, E, q0, q1, b.status, st));
  // A = -dt/2 h1_eff and h1_eff = h1 + (terms without h1): dJ/dh1 = -dt/2 dJ/dA
  ctx_frechet_take_kernel<<<eb, 256, 0, st>>>(N, E, -0.5 * dt, gscale, g_h1);
  TROT_CHECK_LAUNCH("ctx_frechet_take_kernel");
  return TROT_OK;
}

int trot_half_rotate(int norb, int nchol, int nocc, const double* mo, const double* h1, const double* chol,
                     double* rot_h1, double* rot_chol, void* stream) {
  if (!mo || (!h1 && !chol) || (h1 && !rot_h1) || (chol && !rot_chol)) {
    set_error("null input or output");
    return TROT_ERR_NULL_PTR;
  }
  if (norb < 1 || nocc < 1 || nocc > norb || (chol && nchol < 1)) {
    set_error("bad shape: norb %d, nchol %d, nocc %d", norb, nchol, nocc);
    return TROT_ERR_BAD_SHAPE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned pb = (unsigned)((nocc + 15) / 16);
  if (h1) {
    ctx_rotate_kernel<<<dim3(1, pb), 128, 0, st>>>(norb, nocc, mo, h1, rot_h1);
    TROT_CHECK_LAUNCH("ctx_rotate_kernel");
  }
  if (chol) {
    ctx_rotate_kernel<<<dim3(nchol, pb), 128, 0, st>>>(norb, nocc, mo, chol, rot_chol);
    TROT_CHECK_LAUNCH("ctx_rotate_kernel");
  }
  return TROT_OK;
}

int trot_cisd_lci1(int norb, int nchol, int nocc, const double* ci1, const double* chol, double* lci1, void* stream) {
  if (!ci1 || !chol || !lci1) { set_error("null input or output"); return TROT_ERR_NULL_PTR; }
  if (norb < 2 || nchol < 1 || nocc < 1 || nocc >= norb) {
    set_error("bad shape: norb %d, nchol %d, nocc %d", norb, nchol, nocc);
    return TROT_ERR_BAD_SHAPE;
  }
  ctx_lci1_kernel<<<nchol, 256, 0, (cudaStream_t)stream>>>(norb, nocc, ci1, chol, lci1);
  TROT_CHECK_LAUNCH("ctx_lci1_kernel");
  return TROT_OK;
}

}  // extern "C"
