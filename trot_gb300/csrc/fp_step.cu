// Free-projection step (trot/prop/afqmc_fp.py:18-72): unshifted fields, the
// Trotter action with the propagation context's terms (10 in the reference),
// per-walker constants exp(-sqrt(dt) shift + dt h0_prop) spread over the walker
// columns, QR norms prod_j |R_jj| (trot/walkers.py:182-207), weights times the
// norms, comb resampling, and the resampled weights divided by the selected
// walkers' norms.  Overlaps, the energy shift and node count are unchanged.
#include "kernels.h"
#include "profile.h"

namespace trot {

// shift_term = sum_g x_g mf_g = i s (mf purely imaginary); constants c = exp(-sqrt(dt) i s + dt h0_prop);
// croot = c^(1/n_total) = exp(log(c) / n_total) with the principal logarithm (as complex ** in numpy/jax)
__global__ void fp_fields_kernel(int G, double sqrt_dt, double dt, double h0_prop, int n_total,
                                 const double* __restrict__ x, const double* __restrict__ mf_im,
                                 double2* __restrict__ xs, double2* __restrict__ croot) {
  __shared__ double2 red[32];
  const int b = blockIdx.x;
  double2 acc = cmk(0.0, 0.0);
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const double v = x[(size_t)b * G + g];
    xs[(size_t)b * G + g] = cmk(v, 0.0);
    acc.x += v * mf_im[g];
  }
  acc = block_sum2(acc, red);
  if (threadIdx.x == 0) {
    const double2 c = cexp(cmk(dt * h0_prop, -sqrt_dt * acc.x));
    const double2 lg = cmk(log(hypot(c.x, c.y)), atan2(c.y, c.x));
    croot[b] = cexp(cscale(lg, 1.0 / (double)n_total));
  }
}

__global__ void fp_scale_kernel(size_t per_walker, const double2* __restrict__ croot, double2* __restrict__ w) {
  const int b = blockIdx.y;
  const double2 c = croot[b];
  double2* wb = w + (size_t)b * per_walker;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per_walker; e += (size_t)gridDim.x * blockDim.x)
    wb[e] = cmul(wb[e], c);
}

__global__ void fp_weights_kernel(int W, const double* __restrict__ weights, const double2* __restrict__ norm,
                                  double* __restrict__ wnew) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < W) wnew[b] = weights[b] * norm[b].x;
}

__global__ void fp_finalize_kernel(int W, const double* __restrict__ wsr, const double2* __restrict__ norm,
                                   const long long* __restrict__ idx, double* __restrict__ weights) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < W) weights[k] = wsr[k] / norm[idx[k]].x;
}

struct FpBuffers {
  double2 *xs, *croot, *norm, *ga, *gb;
  double *wnew, *wsr, *cw;
  long long* idx;
};

static size_t carve_fp(const trot_system* s, const Spins& sp, Carver& c, FpBuffers& f) {
  const size_t W = s->n_walkers, N = s->norb, G = s->nchol;
  f = FpBuffers{};
  f.xs = c.take<double2>(W * G);
  f.croot = c.take<double2>(W);
  f.norm = c.take<double2>(W);
  f.wnew = c.take<double>(W);
  f.wsr = c.take<double>(W);
  f.cw = c.take<double>(W);
  f.idx = c.take<long long>(W);
  f.ga = c.take<double2>(W * N * sp.n[0]);
  if (sp.nspin == 2) f.gb = c.take<double2>(W * N * sp.n[1]);
  return c.used;
}

static size_t trotter_bytes(const trot_system* s) {
  return (trot_workspace_size(s, TROT_OP_APPLY_TROTTER) + 255) & ~(size_t)255;
}

}  // namespace trot

using namespace trot;

extern "C" {

size_t trot_fp_workspace_size(const trot_system* s) {
  const size_t tb = trotter_bytes(s);
  if (tb == 0) return 0;
  Spins sp = make_spins(s);
  Carver c(nullptr, 0);
  FpBuffers f;
  return tb + carve_fp(s, sp, c, f) + 256;
}

int trot_fp_step(const trot_system* s, const trot_state* state, const double* fields, const double* zeta_dev,
                 void* ws, size_t ws_bytes, void* stream) {
  if (!s || !state || !fields || !zeta_dev) { set_error("null system, state, fields or zeta"); return TROT_ERR_NULL_PTR; }
  if (!state->walkers_a || (s->kind != TROT_RHF_R && !state->walkers_b) || !state->weights) {
    set_error("null state buffer");
    return TROT_ERR_NULL_PTR;
  }
  if (!s->mf_shifts_im) { set_error("null propagation context"); return TROT_ERR_NULL_PTR; }
  const size_t tb = trotter_bytes(s);
  if (tb == 0) return TROT_ERR_BAD_SHAPE;  // trot_workspace_size recorded the reason
  if (ws_bytes < tb) { set_error("workspace too small: %zu < %zu", ws_bytes, tb); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  Spins sp = make_spins(s);
  Carver c(ws ? static_cast<char*>(ws) + tb : nullptr, ws_bytes - tb);
  FpBuffers f;
  carve_fp(s, sp, c, f);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, tb + c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaStream_t st = (cudaStream_t)stream;
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  const int n_total = sp.nspin == 2 ? sp.n[0] + sp.n[1] : 2 * sp.n[0];
  double2* wa = (double2*)state->walkers_a;
  double2* wb = (double2*)state->walkers_b;
  fp_fields_kernel<<<W, 256, 0, st>>>(G, s->sqrt_dt, s->dt, s->h0_prop, n_total, fields, s->mf_shifts_im, f.xs,
                                      f.croot);
  TROT_CHECK_LAUNCH("fp_fields_kernel");
  TROT_TRY(trot_apply_trotter(s, (const double*)wa, (const double*)wb, (const double*)f.xs, (double*)wa, (double*)wb,
                              ws, tb, stream));
  for (int q = 0; q < sp.nspin; ++q) {
    const size_t per = (size_t)N * sp.n[q];
    fp_scale_kernel<<<dim3((unsigned)((per + 255) / 256), W), 256, 0, st>>>(per, f.croot, q == 0 ? wa : wb);
    TROT_CHECK_LAUNCH("fp_scale_kernel");
  }
  TROT_TIMED("qr_norm", st, launch_qr(sp, W, N, wa, wb, f.norm, st, false));
  fp_weights_kernel<<<(W + 255) / 256, 256, 0, st>>>(W, state->weights, f.norm, f.wnew);
  TROT_CHECK_LAUNCH("fp_weights_kernel");
  TROT_TRY(launch_sr(sp, W, N, f.wnew, zeta_dev, 0.0, wa, wb, f.ga, f.gb, f.wsr, f.idx, f.cw, st));
  fp_finalize_kernel<<<(W + 255) / 256, 256, 0, st>>>(W, f.wsr, f.norm, f.idx, state->weights);
  TROT_CHECK_LAUNCH("fp_finalize_kernel");
  cudaError_t e = cudaMemcpyAsync(wa, f.ga, (size_t)W * N * sp.n[0] * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && sp.nspin == 2)
    e = cudaMemcpyAsync(wb, f.gb, (size_t)W * N * sp.n[1] * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "trot_fp_step copy");
  return TROT_OK;
}

}  // extern "C"
