// FP64 kernels of the phaseless step and the local energy.
#include "kernels.h"
#include "step_tail.cuh"

namespace trot {

// ------------------------------------------------------------------ field shifts
// trot/prop/afqmc.py:99-103:
//   s = -sqrt(dt) (i fb - mf),  xs = x - s,
//   shift_term = sum_g xs mf,   fb_term = sum_g (x s - s^2 / 2)
// mf = i * mf_im (purely imaginary).  One CTA per walker.
__global__ void __launch_bounds__(256)
fields_kernel(int G, double sqrt_dt, const double2* __restrict__ fb, const double* __restrict__ mf_im,
              const double* __restrict__ x, double2* __restrict__ xs, double2* __restrict__ shift_term,
              double2* __restrict__ fb_term) {
  __shared__ double2 red[32];
  const int b = blockIdx.x;
  double2 st = cmk(0.0, 0.0), ft = cmk(0.0, 0.0);
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double2 f = fb[(size_t)b * G + g];
    const double2 mf = cmk(0.0, mf_im[g]);
    const double2 ifb = cmk(-f.y, f.x);
    const double2 s = cscale(csub(ifb, mf), -sqrt_dt);
    const double xv = x[(size_t)b * G + g];
    const double2 xsv = cmk(xv - s.x, -s.y);
    xs[(size_t)b * G + g] = xsv;
    st = cadd(st, cmul(xsv, mf));
    ft = cadd(ft, csub(cscale(s, xv), cscale(cmul(s, s), 0.5)));
  }
  st = block_sum2(st, red);
  ft = block_sum2(ft, red);
  if (threadIdx.x == 0) {
    shift_term[b] = st;
    fb_term[b] = ft;
  }
}

int launch_fields(int W, int G, double sqrt_dt, const double2* fb, const double* mf_im, const double* x,
                  double2* xs, double2* shift_term, double2* fb_term, cudaStream_t st) {
  fields_kernel<<<W, 256, 0, st>>>(G, sqrt_dt, fb, mf_im, x, xs, shift_term, fb_term);
  TROT_CHECK_LAUNCH("fields_kernel");
  return TROT_OK;
}

// ------------------------------------------------------------------ Trotter propagation
// Per walker (trot/prop/chol_afqmc_ops.py:198-222, trot/prop/utils.py:20-30):
//   w1 = E w;  out = w1, term = w1;  term = (i sqrt(dt) / k) V term, out += term  (k = 1..K);
//   w' = E out.
// Both spins share one VHS, so their columns are concatenated (N x ntot).
// In step mode the kernel then computes the new overlap and the phaseless
// importance weight of the walker (trot/prop/afqmc.py:108-130).
static constexpr int kTrotThreads = 256;

// out[p][j] = sum_q E[p][q] in[q][j]   (E real, global)
__device__ void real_mm(int N, int nc, const double* __restrict__ E, const double2* in, double2* out) {
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) {
    const int p = e / nc, j = e % nc;
    const double* Er = E + (size_t)p * N;
    double2 acc = cmk(0.0, 0.0);
    for (int q = 0; q < N; ++q) crfma(acc, Er[q], in[q * nc + j]);
    out[e] = acc;
  }
}

__global__ void __launch_bounds__(kTrotThreads)
trotter_kernel(Spins sp, TrotterArgs a) {
  extern __shared__ double2 smem[];
  __shared__ double2 red[32];
  __shared__ int piv;
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int N = a.N, nc = sp.ntot;
  double2* O = smem;            // accumulator
  double2* T = O + N * nc;      // current term
  double2* T2 = T + N * nc;     // next term
  // load walker columns (both spins) into T2
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    const double2* w = (s == 0 ? a.in_a : a.in_b) + (size_t)b * N * n;
    for (int e = tid; e < N * n; e += nt) T2[(e / n) * nc + sp.off[s] + e % n] = w[e];
  }
  __syncthreads();
  real_mm(N, nc, a.expH, T2, O);
  __syncthreads();
  for (int e = tid; e < N * nc; e += nt) T[e] = O[e];
  __syncthreads();
  const double2* V = a.vhs + (size_t)b * N * N;
  for (int k = 1; k <= a.nterms; ++k) {
    const double c = a.sqrt_dt / (double)k;  // (i sqrt_dt) / k = (0, c)
    for (int e = tid; e < N * nc; e += nt) {
      const int p = e / nc, j = e % nc;
      const double2* Vr = V + (size_t)p * N;
      double2 acc = cmk(0.0, 0.0);
      for (int q = 0; q < N; ++q) cfma(acc, Vr[q], T[q * nc + j]);
      const double2 t = cmk(-c * acc.y, c * acc.x);
      T2[e] = t;
      O[e] = cadd(O[e], t);
    }
    __syncthreads();
    double2* tmp = T; T = T2; T2 = tmp;
  }
  // w' = E out  -> T2, then to global
  real_mm(N, nc, a.expH, O, T2);
  __syncthreads();
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    double2* w = (s == 0 ? a.out_a : a.out_b) + (size_t)b * N * n;
    for (int e = tid; e < N * n; e += nt) w[e] = T2[(e / n) * nc + sp.off[s] + e % n];
  }
  if (a.overlaps == nullptr) return;
  overlap_and_weight(sp, a, N, nc, T2, O, &piv, red);
}

int launch_trotter(const Spins& sp, const TrotterArgs& a, cudaStream_t st) {
  size_t smem = (size_t)3 * a.N * sp.ntot * sizeof(double2);
  if (smem > 220 * 1024) {
    set_error("trotter: 3 walker tiles of %zu bytes exceed shared memory", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 40 * 1024)
    cudaFuncSetAttribute(trotter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  trotter_kernel<<<a.W, kTrotThreads, smem, st>>>(sp, a);
  TROT_CHECK_LAUNCH("trotter_kernel");
  return TROT_OK;
}

// ------------------------------------------------------------------ population control
// trot/prop/afqmc.py:126,132-134: nodes += count(flag); E_shift = e_est - damping log(max(mean w, 1e-300)) / dt
__global__ void __launch_bounds__(1024)
step_finalize_kernel(int W, double* __restrict__ weights, double* __restrict__ scalars,
                     long long* __restrict__ nodes, const int* __restrict__ node_flag, double damping, double dt,
                     const int* __restrict__ status) {
  __shared__ double2 red[32];
  if (status && status[0] != 0) {  // a tensor-core kernel of this step timed out: no numbers
    const double nan = __longlong_as_double(0x7FF8000000000000ll);
    for (int i = threadIdx.x; i < W; i += blockDim.x) weights[i] = nan;
    if (threadIdx.x == 0) scalars[0] = nan;
    return;
  }
  double2 acc = cmk(0.0, 0.0);  // (sum w, node count)
  for (int i = threadIdx.x; i < W; i += blockDim.x) {
    acc.x += weights[i];
    acc.y += (double)node_flag[i];
  }
  acc = block_sum2(acc, red);
  if (threadIdx.x == 0) {
    double avg = acc.x / (double)W;
    if (!(avg >= 1.0e-300)) avg = avg != avg ? avg : 1.0e-300;
    scalars[0] = scalars[1] - damping * (log(avg) / dt);
    nodes[0] += (long long)acc.y;
  }
}

int launch_step_finalize(int W, double* weights, double* scalars, long long* nodes, const int* node_flag,
                         double damping, double dt, cudaStream_t st, const int* status) {
  step_finalize_kernel<<<1, 1024, 0, st>>>(W, weights, scalars, nodes, node_flag, damping, dt, status);
  TROT_CHECK_LAUNCH("step_finalize_kernel");
  return TROT_OK;
}

// ------------------------------------------------------------------ exchange energy
// sum_g sum_ij f_gij f_gji with f_g = rot_chol_g G^T  (trot/meas/rhf.py:33-60,
// trot/meas/uhf.py:220-225), per walker and per chunk of Cholesky vectors;
// multiplicities folded in: partial[b][chunk] = sum_s mult_s exc_s.
static constexpr int kExcChunk = 16;

int exchange_chunks(int G) { return (G + kExcChunk - 1) / kExcChunk; }

__global__ void __launch_bounds__(256)
exchange_kernel(Spins sp, int N, int G, const double2* __restrict__ green, double2* __restrict__ partial) {
  extern __shared__ double2 smem[];
  __shared__ double2 red[32];
  const int chunk = blockIdx.x, b = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int g0 = chunk * kExcChunk, g1 = min(G, g0 + kExcChunk);
  double2 acc_all = cmk(0.0, 0.0);
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    double2* Gs = smem;                             // n x N
    double2* F = Gs + n * N;                        // n x n
    double* R = reinterpret_cast<double*>(F + n * n);  // n x N
    const double2* gsrc = green + (size_t)b * sp.ntot * N + (size_t)sp.off[s] * N;
    __syncthreads();
    for (int e = tid; e < n * N; e += nt) Gs[e] = gsrc[e];
    double2 acc = cmk(0.0, 0.0);
    for (int g = g0; g < g1; ++g) {
      const double* Rg = sp.rot_chol[s] + (size_t)g * n * N;
      __syncthreads();
      for (int e = tid; e < n * N; e += nt) R[e] = Rg[e];
      __syncthreads();
      for (int e = tid; e < n * n; e += nt) {
        const int i = e / n, j = e % n;
        double2 f = cmk(0.0, 0.0);
        for (int p = 0; p < N; ++p) crfma(f, R[i * N + p], Gs[j * N + p]);
        F[e] = f;
      }
      __syncthreads();
      for (int e = tid; e < n * n; e += nt) {
        const int i = e / n, j = e % n;
        cfma(acc, F[i * n + j], F[j * n + i]);
      }
    }
    acc = block_sum2(acc, red);
    acc_all = cadd(acc_all, cscale(acc, (double)sp.mult[s]));
  }
  if (tid == 0) partial[(size_t)b * gridDim.x + chunk] = acc_all;
}

int launch_exchange(const Spins& sp, int W, int N, int G, const double2* green, double2* partial,
                    cudaStream_t st) {
  int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  size_t smem = (size_t)(nmax * N + nmax * nmax) * sizeof(double2) + (size_t)nmax * N * sizeof(double);
  if (smem > 200 * 1024) {
    set_error("exchange: tile of %zu bytes exceeds shared memory", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 40 * 1024)
    cudaFuncSetAttribute(exchange_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid(exchange_chunks(G), W);
  exchange_kernel<<<grid, 256, smem, st>>>(sp, N, G, green, partial);
  TROT_CHECK_LAUNCH("exchange_kernel");
  return TROT_OK;
}

// E = h0 + e1 + 1/2 sum_g fb_g^2 - 1/2 sum_chunks partial   (fb already carries the spin multiplicity;
// e1 comes in e1_parts parts of W values each, added in order)
__global__ void __launch_bounds__(256)
energy_combine_kernel(int G, int nchunks, double h0, const double2* __restrict__ fb,
                      const double2* __restrict__ e1, int e1_parts, const double2* __restrict__ partial,
                      double2* __restrict__ energy, const int* __restrict__ status,
                      const ExFixed* __restrict__ xfixed) {
  __shared__ double2 red[32];
  const int b = blockIdx.x;
  if (status && status[0] != 0) {  // the exchange / force-bias kernel timed out: no numbers
    const double nan = __longlong_as_double(0x7FF8000000000000ll);
    if (threadIdx.x == 0) energy[b] = cmk(nan, nan);
    return;
  }
  double2 c = cmk(0.0, 0.0), x = cmk(0.0, 0.0);
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double2 f = fb[(size_t)b * G + g];
    cfma(c, f, f);
  }
  if (xfixed) {
    const double nan = __longlong_as_double(0x7FF8000000000000ll);
    for (int k = threadIdx.x; k < nchunks; k += blockDim.x) {
      const ExFixed f = xfixed[(size_t)b * nchunks + k];
      double v[2];
      for (int c = 0; c < 2; ++c)  // v 2^-s, with 2^-s formed from its exponent bits (|s| < 1000)
        v[c] = f.s[c] == kExchangeNonFinite ? nan
                                             : (double)f.v[c] * __longlong_as_double((long long)(1023 - f.s[c]) << 52);
      x = cadd(x, cmk(v[0], v[1]));
    }
  } else {
    for (int k = threadIdx.x; k < nchunks; k += blockDim.x) x = cadd(x, partial[(size_t)b * nchunks + k]);
  }
  c = block_sum2(c, red);
  x = block_sum2(x, red);
  if (threadIdx.x == 0) {
    double2 e = e1[b];
    for (int k = 1; k < e1_parts; ++k) e = cadd(e, e1[(size_t)k * gridDim.x + b]);
    energy[b] = cmk(h0 + e.x + 0.5 * c.x - 0.5 * x.x, e.y + 0.5 * c.y - 0.5 * x.y);
  }
}

int launch_energy_combine(int W, int G, int nchunks, double h0, const double2* fb, const double2* e1, int e1_parts,
                          const double2* partial, double2* energy, cudaStream_t st, const int* status,
                          const ExFixed* xfixed) {
  energy_combine_kernel<<<W, 256, 0, st>>>(G, nchunks, h0, fb, e1, e1_parts, partial, energy, status, xfixed);
  TROT_CHECK_LAUNCH("energy_combine_kernel");
  return TROT_OK;
}

__global__ void status_merge_kernel(const int* __restrict__ src, int* __restrict__ dst) {
  const int v = src[0];
  if (v != 0) {
    dst[0] = v;
    dst[3] = v;
  }
}

int launch_status_merge(const int* src, int* dst, cudaStream_t st) {
  status_merge_kernel<<<1, 1, 0, st>>>(src, dst);
  TROT_CHECK_LAUNCH("status_merge_kernel");
  return TROT_OK;
}

}  // namespace trot
