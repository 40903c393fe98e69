// extern "C" entry points (include/trot_gb300.h): argument checks, workspace
// carving and the launch sequence of each op.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "kernels.h"
#include "mixed.h"
#include "profile.h"

namespace trot {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("%s: %s", where, cudaGetErrorString(e));
  return TROT_ERR_CUDA;
}

Spins make_spins(const trot_system* s) {
  Spins sp{};
  if (s->kind == TROT_RHF_R) {
    sp.nspin = 1;
    sp.n[0] = s->nocc_a; sp.n[1] = 0;
    sp.mult[0] = 2; sp.mult[1] = 0;
    sp.mo[0] = s->mo_a; sp.rot_h1[0] = s->rot_h1_a; sp.rot_chol[0] = s->rot_chol_a;
  } else {
    sp.nspin = 2;
    sp.n[0] = s->nocc_a; sp.n[1] = s->nocc_b;
    sp.mult[0] = sp.mult[1] = 1;
    const bool uhf = s->kind == TROT_UHF_U;
    sp.mo[0] = s->mo_a; sp.mo[1] = uhf ? s->mo_b : s->mo_a;
    sp.rot_h1[0] = s->rot_h1_a; sp.rot_h1[1] = uhf ? s->rot_h1_b : s->rot_h1_a;
    sp.rot_chol[0] = s->rot_chol_a; sp.rot_chol[1] = uhf ? s->rot_chol_b : s->rot_chol_a;
  }
  sp.off[0] = 0;
  sp.off[1] = sp.n[0];
  sp.ntot = sp.n[0] + sp.n[1];
  return sp;
}

// Workspace layout shared by size query and the ops.
static size_t carve_step(const trot_system* s, const Spins& sp, Carver& c, StepBuffers& b, int op) {
  const size_t W = s->n_walkers, N = s->norb, G = s->nchol;
  b = StepBuffers{};
  if (op == TROT_OP_SR) { c.take<double>(W); return c.used; }
  if (op == TROT_OP_QR) return c.used;
  b.green = c.take<double2>(W * sp.ntot * N);
  b.e1 = c.take<double2>(W);
  b.fb = c.take<double2>(W * G);
  if (op == TROT_OP_LOCAL_ENERGY || op == TROT_OP_PROP_STEP) b.exc = c.take<double2>(W * exchange_chunks((int)G));
  if (op == TROT_OP_APPLY_TROTTER || op == TROT_OP_PROP_STEP) {
    b.vhs = c.take<double2>(W * N * N);
    if (s->chol_packed) b.vp = c.take<double2>(W * (N * (N + 1) / 2));
  }
  if (op == TROT_OP_PROP_STEP) {
    b.xs = c.take<double2>(W * G);
    b.shift_term = c.take<double2>(W);
    b.fb_term = c.take<double2>(W);
    b.node_flag = c.take<int>(W);
  }
  return c.used;
}

static int check_system(const trot_system* s) {
  if (!s) { set_error("null system"); return TROT_ERR_NULL_PTR; }
  if (s->kind < TROT_RHF_R || s->kind > TROT_UHF_U) { set_error("bad kind %d", s->kind); return TROT_ERR_BAD_SHAPE; }
  if (s->n_walkers <= 0 || s->norb <= 0 || s->nchol < 0 || s->nocc_a <= 0 || s->nocc_a > s->norb) {
    set_error("bad sizes W=%d N=%d G=%d na=%d", s->n_walkers, s->norb, s->nchol, s->nocc_a);
    return TROT_ERR_BAD_SHAPE;
  }
  if (s->kind != TROT_RHF_R && (s->nocc_b <= 0 || s->nocc_b > s->norb)) {
    set_error("bad nocc_b=%d", s->nocc_b);
    return TROT_ERR_BAD_SHAPE;
  }
  if (s->kind == TROT_RHF_U && s->nocc_a != s->nocc_b) {
    set_error("RHF trial requires nocc_a == nocc_b (got %d, %d)", s->nocc_a, s->nocc_b);
    return TROT_ERR_BAD_SHAPE;
  }
  if (s->n_walkers > 65535) { set_error("n_walkers=%d > 65535", s->n_walkers); return TROT_ERR_UNSUPPORTED; }
  if (s->precision != TROT_FP64 && s->precision != TROT_MIXED) {
    set_error("bad precision %d", s->precision);
    return TROT_ERR_BAD_DTYPE;
  }
  if (!s->mo_a || (s->kind == TROT_UHF_U && !s->mo_b)) { set_error("null trial coefficients"); return TROT_ERR_NULL_PTR; }
  return TROT_OK;
}

static int check_walkers(const trot_system* s, const void* wa, const void* wb) {
  if (!wa || (s->kind != TROT_RHF_R && !wb)) { set_error("null walker pointer"); return TROT_ERR_NULL_PTR; }
  return TROT_OK;
}

static int check_meas(const trot_system* s, bool need_h1) {
  if (!s->rot_chol_a || (s->kind == TROT_UHF_U && !s->rot_chol_b)) { set_error("null rot_chol"); return TROT_ERR_NULL_PTR; }
  if (need_h1 && (!s->rot_h1_a || (s->kind == TROT_UHF_U && !s->rot_h1_b))) { set_error("null rot_h1"); return TROT_ERR_NULL_PTR; }
  return TROT_OK;
}

static int check_prop(const trot_system* s) {
  if (!s->exp_h1_half || !s->chol_flat || !s->mf_shifts_im) { set_error("null propagation context"); return TROT_ERR_NULL_PTR; }
  if (s->n_exp_terms < 0 || s->n_exp_terms > 64) { set_error("bad n_exp_terms %d", s->n_exp_terms); return TROT_ERR_BAD_SHAPE; }
  if (s->precision == TROT_MIXED && !s->mixed) { set_error("mixed precision needs trot_mixed_prepare context"); return TROT_ERR_NULL_PTR; }
  return TROT_OK;
}


// force bias from the half Green's functions: fb = sum_s mult_s rot_chol_s G_s
static int force_bias_from_green(const trot_system* s, const Spins& sp, const double2* green, double2* fb,
                                 cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, G = s->nchol, K = sp.ntot * N;
  for (int q = 0; q < sp.nspin; ++q) {
    TROT_TRY(launch_zgemm_cr(W, G, sp.n[q] * N, (double)sp.mult[q], green + (size_t)sp.off[q] * N, K,
                             sp.rot_chol[q], sp.n[q] * N, true, fb, G, q > 0, st));
  }
  return TROT_OK;
}

// ------------------------------------------------------------------ block rdm1 observable
// Chunks of walkers per Green's-function row, so that rows x chunks covers the GPU.
static int rdm1_chunks(const trot_system* s, const Spins& sp) {
  const int want = (2 * 152 + sp.ntot - 1) / sp.ntot;
  return std::max(1, std::min(std::min(64, want), s->n_walkers));
}

static size_t rdm1_workspace_size(const trot_system* s, const Spins& sp) {
  return (size_t)rdm1_chunks(s, sp) * sp.ntot * s->norb * sizeof(double2);
}

// part[c][row][p] = sum over the walkers of chunk c (in order) of wt_w G_w[row][p]
__global__ void rdm1_partial_kernel(int W, int rows, int N, int wchunk, const double2* __restrict__ green,
                                    const double* __restrict__ weights, double2* __restrict__ part) {
  const int row = blockIdx.x, c = blockIdx.y;
  const int w0 = c * wchunk, w1 = min(W, w0 + wchunk);
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    double2 acc = cmk(0.0, 0.0);
    for (int w = w0; w < w1; ++w) acc = cadd(acc, cscale(green[((size_t)w * rows + row) * N + p], weights[w]));
    part[((size_t)c * rows + row) * N + p] = acc;
  }
}

// out[s][p][q] = sum_i Gbar_s[i][p] conj(C_s[q][i]) / w_sum with Gbar = sum_c part[c] (fixed order)
__global__ void rdm1_finish_kernel(Spins sp, int N, int nchunk, const double2* __restrict__ part,
                                   const double* __restrict__ obs, double2* __restrict__ out) {
  extern __shared__ double2 gbar[];  // [n]
  const int so = blockIdx.x, p = blockIdx.y;
  const int s = sp.nspin == 1 ? 0 : so;
  const int n = sp.n[s], off = sp.off[s];
  const double* C = sp.mo[s];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double2 acc = cmk(0.0, 0.0);
    for (int c = 0; c < nchunk; ++c) acc = cadd(acc, part[((size_t)c * sp.ntot + off + i) * N + p]);
    gbar[i] = acc;
  }
  __syncthreads();
  const double wsum = obs[1];
  for (int q = threadIdx.x; q < N; q += blockDim.x) {
    double2 v = cmk(0.0, 0.0);
    for (int i = 0; i < n; ++i) v = cadd(v, cscale(gbar[i], C[(size_t)q * n + i]));
    out[((size_t)so * N + p) * N + q] = wsum == 0.0 ? cmk(0.0, 0.0) : cmk(v.x / wsum, v.y / wsum);
  }
}

}  // namespace trot

using namespace trot;

extern "C" {

const char* trot_last_error(void) { return g_err; }
int trot_abi_version(void) { return TROT_ABI_VERSION; }

size_t trot_workspace_size(const trot_system* s, int op) {
  if (check_system(s) != TROT_OK) return 0;
  Spins sp = make_spins(s);
  Carver c(nullptr, 0);
  StepBuffers b;
  if (op == TROT_OP_RDM1) return rdm1_workspace_size(s, sp) + 256;
  if (s->precision == TROT_MIXED && op != TROT_OP_SR && op != TROT_OP_QR) {
    if (!s->mixed) return 0;
    return mixed_workspace_size(s, op) + 256;
  }
  size_t n = carve_step(s, sp, c, b, op);
  return n + 256;
}

int trot_block_rdm1(const trot_system* s, const double* green, const double* weights, const double* obs,
                    double* rdm1_out, void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  if (!green || !weights || !obs || !rdm1_out || !ws) { set_error("null rdm1 buffer"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  const size_t need = rdm1_workspace_size(s, sp) + 256;
  if (ws_bytes < need) {
    set_error("workspace too small: %zu < %zu", ws_bytes, need);
    return TROT_ERR_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int W = s->n_walkers, N = s->norb, nchunk = rdm1_chunks(s, sp);
  const int wchunk = (W + nchunk - 1) / nchunk;
  double2* part = reinterpret_cast<double2*>(static_cast<char*>(ws) + 256);
  rdm1_partial_kernel<<<dim3(sp.ntot, nchunk), 128, 0, st>>>(W, sp.ntot, N, wchunk, (const double2*)green, weights,
                                                            part);
  TROT_CHECK_LAUNCH("rdm1_partial_kernel");
  const int nmax = std::max(sp.n[0], sp.n[1]);
  rdm1_finish_kernel<<<dim3(2, N), 128, (size_t)nmax * sizeof(double2), st>>>(sp, N, nchunk, part, obs,
                                                                            (double2*)rdm1_out);
  TROT_CHECK_LAUNCH("rdm1_finish_kernel");
  return TROT_OK;
}

int trot_overlap(const trot_system* s, const double* wa, const double* wb, double* out, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  if (!out) { set_error("null output"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  return launch_green(sp, s->n_walkers, s->norb, (const double2*)wa, (const double2*)wb, nullptr,
                      (double2*)out, nullptr, (cudaStream_t)stream);
}

int trot_half_green(const trot_system* s, const double* wa, const double* wb, double* green_out,
                    double* overlaps_out, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  if (!green_out) { set_error("null output"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  return launch_green(sp, s->n_walkers, s->norb, (const double2*)wa, (const double2*)wb, (double2*)green_out,
                      (double2*)overlaps_out, nullptr, (cudaStream_t)stream);
}

int trot_force_bias(const trot_system* s, const double* wa, const double* wb, double* out, void* ws,
                    size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  TROT_TRY(check_meas(s, false));
  if (!out) { set_error("null output"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  cudaStream_t st = (cudaStream_t)stream;
  if (s->precision == TROT_MIXED)
    return mixed_force_bias(s, sp, (const double2*)wa, (const double2*)wb, (double2*)out, ws, ws_bytes, st);
  Carver c(ws, ws_bytes);
  StepBuffers b;
  carve_step(s, sp, c, b, TROT_OP_FORCE_BIAS);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  TROT_TRY(launch_green(sp, s->n_walkers, s->norb, (const double2*)wa, (const double2*)wb, b.green, nullptr,
                        nullptr, st));
  return force_bias_from_green(s, sp, b.green, (double2*)out, st);
}

int trot_local_energy(const trot_system* s, const double* wa, const double* wb, double* out, void* ws,
                      size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  TROT_TRY(check_meas(s, true));
  if (!out) { set_error("null output"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  cudaStream_t st = (cudaStream_t)stream;
  if (s->precision == TROT_MIXED)
    return mixed_local_energy(s, sp, (const double2*)wa, (const double2*)wb, (double2*)out, ws, ws_bytes, st);
  Carver c(ws, ws_bytes);
  StepBuffers b;
  carve_step(s, sp, c, b, TROT_OP_LOCAL_ENERGY);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  TROT_TRY(launch_green(sp, W, N, (const double2*)wa, (const double2*)wb, b.green, nullptr, b.e1, st));
  TROT_TRY(force_bias_from_green(s, sp, b.green, b.fb, st));
  TROT_TRY(launch_exchange(sp, W, N, G, b.green, b.exc, st));
  return launch_energy_combine(W, G, exchange_chunks(G), s->h0, b.fb, b.e1, 1, b.exc, (double2*)out, st);
}

int trot_apply_trotter(const trot_system* s, const double* wa, const double* wb, const double* xs,
                       double* oa, double* ob, void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  TROT_TRY(check_walkers(s, oa, ob));
  TROT_TRY(check_prop(s));
  if (!xs) { set_error("null fields"); return TROT_ERR_NULL_PTR; }
  Spins sp = make_spins(s);
  cudaStream_t st = (cudaStream_t)stream;
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  TrotterArgs a{};
  a.W = W; a.N = N; a.G = G; a.nterms = s->n_exp_terms; a.sqrt_dt = s->sqrt_dt; a.expH = s->exp_h1_half;
  a.in_a = (const double2*)wa; a.in_b = (const double2*)wb; a.out_a = (double2*)oa; a.out_b = (double2*)ob;
  if (s->precision == TROT_MIXED) return mixed_apply_trotter(s, sp, (const double2*)xs, a, ws, ws_bytes, st);
  Carver c(ws, ws_bytes);
  StepBuffers b;
  carve_step(s, sp, c, b, TROT_OP_APPLY_TROTTER);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  TROT_TRY(launch_vhs64(W, N, G, (const double2*)xs, s->chol_flat, s->chol_packed, b.vp, b.vhs, st));
  a.vhs = b.vhs;
  return launch_trotter(sp, a, st);
}

int trot_prop_step(const trot_system* s, const trot_state* state, const double* fields, double* energy_out,
                   void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  if (!state) { set_error("null state"); return TROT_ERR_NULL_PTR; }
  TROT_TRY(check_walkers(s, state->walkers_a, state->walkers_b));
  TROT_TRY(check_meas(s, energy_out != nullptr));
  TROT_TRY(check_prop(s));
  if (!state->weights || !state->overlaps || !state->scalars || !state->node_encounters || !fields) {
    set_error("null state buffer or fields");
    return TROT_ERR_NULL_PTR;
  }
  Spins sp = make_spins(s);
  cudaStream_t st = (cudaStream_t)stream;
  if (s->precision == TROT_MIXED)
    return mixed_prop_step(s, sp, state, fields, (double2*)energy_out, ws, ws_bytes, st);
  Carver c(ws, ws_bytes);
  StepBuffers b;
  carve_step(s, sp, c, b, TROT_OP_PROP_STEP);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  double2* wa = (double2*)state->walkers_a;
  double2* wb = (double2*)state->walkers_b;
  // 1. Green's functions (+ one-body energy) of the current walkers
  TROT_TIMED("green", st, launch_green(sp, W, N, wa, wb, b.green, nullptr, energy_out ? b.e1 : nullptr, st));
  // 2. force bias
  TROT_TIMED("force_bias_fp64", st, force_bias_from_green(s, sp, b.green, b.fb, st));
  // 3. optional local energy of the current walkers (reuses G and fb)
  if (energy_out) {
    TROT_TIMED("exchange_fp64", st, launch_exchange(sp, W, N, G, b.green, b.exc, st));
    TROT_TIMED("energy_combine", st,
               launch_energy_combine(W, G, exchange_chunks(G), s->h0, b.fb, b.e1, 1, b.exc, (double2*)energy_out, st));
  }
  // 4. shifted fields
  TROT_TIMED("fields", st, launch_fields(W, G, s->sqrt_dt, b.fb, s->mf_shifts_im, fields, b.xs, b.shift_term, b.fb_term, st));
  // 5. VHS
  TROT_TIMED("vhs_fp64", st, launch_vhs64(W, N, G, b.xs, s->chol_flat, s->chol_packed, b.vp, b.vhs, st));
  // 6. propagation + overlaps + weights
  TrotterArgs a{};
  a.W = W; a.N = N; a.G = G; a.nterms = s->n_exp_terms; a.sqrt_dt = s->sqrt_dt; a.expH = s->exp_h1_half;
  a.vhs = b.vhs; a.in_a = wa; a.in_b = wb; a.out_a = wa; a.out_b = wb;
  a.overlaps = (double2*)state->overlaps; a.weights = state->weights; a.scalars = state->scalars;
  a.shift_term = b.shift_term; a.fb_term = b.fb_term; a.node_flag = b.node_flag;
  a.dt = s->dt; a.h0_prop = s->h0_prop; a.w_floor = s->weight_floor; a.w_cap = s->weight_cap;
  TROT_TIMED("trotter_fp64", st, launch_trotter(sp, a, st));
  // 7. population-control shift, node count
  TROT_TIMED("step_finalize", st, launch_step_finalize(W, state->weights, state->scalars, (long long*)state->node_encounters,
                                                       b.node_flag, s->pop_control_damping, s->dt, st));
  return TROT_OK;
}

int trot_workspace_status(const void* workspace, int* status_out) {
  if (!workspace || !status_out) { set_error("null pointer"); return TROT_ERR_NULL_PTR; }
  cudaError_t e = cudaMemcpy(status_out, workspace, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "trot_workspace_status");
  return TROT_OK;
}

int trot_workspace_timeouts(void* workspace, int clear, int* status_out) {
  if (!workspace || !status_out) { set_error("null pointer"); return TROT_ERR_NULL_PTR; }
  int* sticky = static_cast<int*>(workspace) + 3;
  cudaError_t e = cudaMemcpy(status_out, sticky, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e, "trot_workspace_timeouts");
  if (clear) {
    const int zero = 0;
    e = cudaMemcpy(sticky, &zero, sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_status(e, "trot_workspace_timeouts clear");
  }
  return TROT_OK;
}

int trot_orthonormalize(const trot_system* s, double* wa, double* wb, double* norm_out, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, wa, wb));
  Spins sp = make_spins(s);
  cudaStream_t st = (cudaStream_t)stream;
  TROT_TIMED("qr", st, launch_qr(sp, s->n_walkers, s->norb, (double2*)wa, (double2*)wb, (double2*)norm_out, st));
  return TROT_OK;
}

int trot_sr_resample(const trot_system* s, const double* weights_in, const double* zeta_dev, double zeta,
                     const double* ina,
                     const double* inb, double* outa, double* outb, double* weights_out, int64_t* idx_out,
                     void* ws, size_t ws_bytes, void* stream) {
  TROT_TRY(check_system(s));
  TROT_TRY(check_walkers(s, ina, inb));
  TROT_TRY(check_walkers(s, outa, outb));
  if (!weights_in || !weights_out || !idx_out) { set_error("null SR buffer"); return TROT_ERR_NULL_PTR; }
  if (!zeta_dev && !(zeta >= 0.0 && zeta < 1.0)) { set_error("zeta %g outside [0, 1)", zeta); return TROT_ERR_BAD_SHAPE; }
  if (ina == outa || (inb && inb == outb)) { set_error("SR input and output walkers must differ"); return TROT_ERR_BAD_SHAPE; }
  Spins sp = make_spins(s);
  Carver c(ws, ws_bytes);
  double* cw = c.take<double>(s->n_walkers);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  return launch_sr(sp, s->n_walkers, s->norb, weights_in, zeta_dev, zeta, (const double2*)ina, (const double2*)inb,
                   (double2*)outa, (double2*)outb, weights_out, (long long*)idx_out, cw, (cudaStream_t)stream);
}

}  // extern "C"
