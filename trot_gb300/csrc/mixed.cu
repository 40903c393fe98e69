// Mixed-precision (tensor-core) path of the phaseless step and local energy.
//
//  * half Green's functions, LU / log-det, overlaps, weights, energy sums: FP64;
//  * f_g = rot_chol_g G^T for all g (exchange and, through its trace, the force
//    bias / Coulomb term): exact-slice BF16 products on tcgen05 tensor cores,
//    combined in float-float (FP32 pairs) arithmetic — near-FP64 accuracy;
//  * VHS = x_shifted . chol: 3-term BF16 split on tcgen05, FP32 accumulation;
//  * one-body half steps and the Taylor series: FP32 on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "ff.cuh"
#include "mixed.h"
#include "profile.h"
#include "step_tail.cuh"
#include "tc.cuh"

namespace trot {

static constexpr int kMaxOccGJ = 16;  // largest n of the warp Gauss-Jordan kernels (perm scratch)

// ------------------------------------------------------------------ Green's functions in float-float
// Same quantities as green_kernel (green.cu): M_s = C_s^T w_s, M_s^{-1} by FP64
// Gauss-Jordan, G_s = (w_s M_s^{-1})^T and e1 = sum_s mult_s sum G_s o rot_h1_s, with
// the two N x n^2 products in float-float (FP32 pairs, ~2^-44 relative) on the FP32
// pipe: this GPU's FP64 pipe retires about two FMAs per clock per SM, so an FP64 M_s
// alone would cost more than the rest of the kernel.  One CTA per (walker, spin).
__global__ void __launch_bounds__(256)
green_ff_kernel(Spins sp, int N, const double2* __restrict__ wa, const double2* __restrict__ wb,
                double2* __restrict__ green, double2* __restrict__ e1_out) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ double2 red[32];
  __shared__ int perm[kMaxOccGJ];
  const int b = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  ffc* Wf = reinterpret_cast<ffc*>(smem_raw);                    // N x n
  ff* Cf = reinterpret_cast<ff*>(Wf + (size_t)N * nmax);          // N x n
  double2* Md = reinterpret_cast<double2*>(Cf + (size_t)N * nmax + ((N * nmax) & 1));  // n x n, then M^{-1}
  ffc* Mif = reinterpret_cast<ffc*>(Md + nmax * nmax);            // n x n
  ff e1r{0.f, 0.f}, e1i{0.f, 0.f};
  {
    const int n = s ? sp.n[1] : sp.n[0];
    const double2* w = (s == 0 ? wa : wb) + (size_t)b * N * n;
    const double* C = s ? sp.mo[1] : sp.mo[0];
    __syncthreads();
    for (int e = tid; e < N * n; e += nt) {
      const double2 x = w[e];
      Wf[e] = ffc{ff_from_d(x.x), ff_from_d(x.y)};
      Cf[e] = ff_from_d(C[e]);
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
      // M[i][j] = sum_p C[p][i] w[p][j] in float-float on the FP32 pipe (four accumulator pairs over
      // p mod 4 against the latency chains, combined in a fixed order)
      const int i = e / n, j = e % n;
      ff ar[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      ff ai[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      int p = 0;
      for (; p + 4 <= N; p += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const ff c = Cf[(p + u) * n + i];
          const ffc x = Wf[(p + u) * n + j];
          ff_mad(ar[u], c, x.re);
          ff_mad(ai[u], c, x.im);
        }
      }
      for (; p < N; ++p) {
        const ff c = Cf[p * n + i];
        const ffc x = Wf[p * n + j];
        ff_mad(ar[0], c, x.re);
        ff_mad(ai[0], c, x.im);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        ar[u] = ff_fast(ar[u].hi, ar[u].lo);
        ai[u] = ff_fast(ai[u].hi, ai[u].lo);
      }
      const ff sr = ff_add(ff_add(ar[0], ar[1]), ff_add(ar[2], ar[3]));
      const ff si = ff_add(ff_add(ai[0], ai[1]), ff_add(ai[2], ai[3]));
      Md[e] = make_double2(ff_d(sr), ff_d(si));
    }
    __syncthreads();
    // M^{-1} in place, FP64, by one warp (warp-synchronous phases; the other warps wait here)
    if (tid < 32) warp_gauss_jordan(Md, n, true, perm);
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) Mif[e] = ffc{ff_from_d(Md[e].x), ff_from_d(Md[e].y)};
    __syncthreads();
    const double* H = s ? sp.rot_h1[1] : sp.rot_h1[0];
    double2* gout = green + (size_t)b * sp.ntot * N + (size_t)(s ? sp.off[1] : 0) * N;
    const float m = (float)(s ? sp.mult[1] : sp.mult[0]);
    for (int e = tid; e < n * N; e += nt) {
      const int i = e / N, p = e % N;
      ff gr{0.f, 0.f}, gi{0.f, 0.f};
      for (int j = 0; j < n; ++j) {
        const ffc x = Wf[p * n + j], y = Mif[j * n + i];
        ff_mad(gr, x.re, y.re);
        ff_mad(gr, ff{-x.im.hi, -x.im.lo}, y.im);
        ff_mad(gi, x.re, y.im);
        ff_mad(gi, x.im, y.re);
      }
      gr = ff_fast(gr.hi, gr.lo);
      gi = ff_fast(gi.hi, gi.lo);
      gout[e] = make_double2(ff_d(gr), ff_d(gi));
      if (H) {
        const ff h = ff_from_d(H[e]);
        e1r = ff_add(e1r, ff_mul(h, ff{gr.hi * m, gr.lo * m}));
        e1i = ff_add(e1i, ff_mul(h, ff{gi.hi * m, gi.lo * m}));
      }
    }
  }
  if (e1_out) {
    double2 v = make_double2(ff_d(e1r), ff_d(e1i));
    v = block_sum2(v, red);
    if (tid == 0) e1_out[(size_t)s * gridDim.x + b] = v;
  }
}

static int launch_green_ff(const Spins& sp, int W, int N, const double2* wa, const double2* wb, double2* green,
                           double2* e1_out, cudaStream_t st) {
  const int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  const size_t smem = (size_t)N * nmax * (sizeof(ffc) + sizeof(ff)) + 16 + (size_t)nmax * nmax * 2 * 16;
  if (nmax > kMaxOccGJ) {
    set_error("green_ff: nocc %d > %d", nmax, kMaxOccGJ);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 200 * 1024) {
    set_error("green_ff: %zu bytes of shared memory needed", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  if (smem > 40 * 1024) cudaFuncSetAttribute(green_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  green_ff_kernel<<<dim3(W, sp.nspin), 256, smem, st>>>(sp, N, wa, wb, green, e1_out);
  TROT_CHECK_LAUNCH("green_ff_kernel");
  return TROT_OK;
}

// ------------------------------------------------------------------ layouts
static constexpr size_t kTcImgBytes = 3 * 128 * 256 * 2;  // [Vr | Vi] operand image of one walker (192 KB)
static constexpr int kKP = 128;       // padded orbital dimension of the exact product
static constexpr int kKS = kKP / 16;  // K16 steps of the exact product
static constexpr int kGroups = 5;     // accumulators for t + u = 0..4
static constexpr int kSlices = 5;
static constexpr int kMaxOcc = 16;    // largest n the exchange epilogue handles
// FP16 digit format of the exact product (trot_mixed.digit_format 2): Cholesky rows
// 2^eA sum_t qA_t 2^-(9 + 9t), Green's-function rows 2^eB sum_u qB_u 2^-(8 + 9u), five
// planes each; digit products of order d = t + u carry 2^(eA + eB - 17 - 9d).  Four planes
// (products d <= 3) are not enough: the exchange sum cancels strongly, and the error of
// the individual terms (2^-35 of their size) reached 3e-5 Ha on walkers near the trial.  Both operands are
// stored per K16 step: [plane][rows][16] blocks in core-matrix order (see tile16_idx).
static constexpr int kDigitFormat = 2;
static constexpr int kRotTopBits = 9, kGreenTopBits = 8, kLowBits = 9;
static constexpr int kGreenBits = kGreenTopBits + kLowBits * (kSlices - 1);  // 44 fixed-point bits per row
static constexpr uint32_t kAStep = (uint32_t)kSlices * 128 * 16 * 2;  // 20480 B: the 5 rot planes of one K16 step
static constexpr uint32_t kAImg = (uint32_t)kKS * kAStep;             // 163840 B: a whole 128-row Cholesky tile

// Element (r, k) of a [rows x 16] K-major block in core-matrix order (8 rows x 8 K per
// 128-byte core matrix; core matrices 128 B apart along K, 256 B apart along rows):
// 16-bit index (r/8)*128 + (k/8)*64 + (r%8)*8 + k%8.  Descriptor LBO 128 B, SBO 256 B.
TROT_HD uint32_t tile16_idx(int r, int k) {
  return (uint32_t)((r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7));
}

// Walker tiles of the exchange product: the Green's-function rows (walker b, j, c) of
// P = WBT * 2 n_pad columns; the five digit planes of a tile are stacked along the MMA's
// N dimension (planes 0..4-t in one MMA with rot plane t), so P <= 51 and 2 x 5P TMEM
// columns (double-buffered accumulators) fit the 512 columns.
TROT_HD int ex_npad(int n) { return n <= 4 ? 4 : n <= 8 ? 8 : n <= 12 ? 12 : 16; }
TROT_HD int ex_cols(int n_pad) { return n_pad == 16 ? 32 : 48; }

struct SpinLayout {
  int n, n_pad, S, P, WB, ntiles;  // columns per walker S = 2 n_pad, per tile P = WB S; walker tiles
  int gb, nblk, blk_off;        // Cholesky vectors per 128-row tile, tiles, offset in the partial array
};

static SpinLayout spin_layout(const trot_system* s, const Spins& sp, int q) {
  SpinLayout L{};
  L.n = sp.n[q];
  L.n_pad = ex_npad(L.n);
  L.S = 2 * L.n_pad;
  L.P = ex_cols(L.n_pad);
  L.WB = L.P / L.S;
  L.ntiles = (s->n_walkers + L.WB - 1) / L.WB;
  const int mq = (s->kind == TROT_UHF_U) ? q : 0;
  L.gb = s->mixed->gammas_per_block[mq];
  L.nblk = s->mixed->n_blocks[mq];
  L.blk_off = q == 0 ? 0 : s->mixed->n_blocks[0];
  return L;
}

struct MixedBuffers {
  double2* green;
  double2* e1;
  uint16_t* gq[2];   // per spin: [tile][K16 step][5 planes x P rows][16] in core-matrix order
  int32_t* ge[2];    // per spin: [tile][P] row exponents
  float4* cs[2];     // per spin: traces c_g per (walker, g) as float-float (re.hi, re.lo, im.hi, im.lo)
  ExFixed* xpart;    // exchange partial sums per (walker, Cholesky tile)
  double2* fb;
  double2* xs;
  double2 *shift_term, *fb_term;
  uint16_t* xq;
  float* vhs;
  uint16_t* vimg;  // [Vr | Vi] operand images of the tensor-core Trotter kernel
  double2* ov_new; // overlaps of the propagated walkers (tensor-core Trotter, step mode)
  double2* ovp;    // det(M_s)^mult_s per (spin, walker) of the propagated walkers
  int* node_flag;
  int* status;
  int nblk_total, mpad;
};

static size_t carve_mixed(const trot_system* s, const Spins& sp, Carver& c, MixedBuffers& m, int op) {
  const size_t W = s->n_walkers, N = s->norb, G = s->nchol;
  m = MixedBuffers{};
  if (op == TROT_OP_SR || op == TROT_OP_QR) return c.used;
  m.status = c.status();
  const bool meas = op == TROT_OP_FORCE_BIAS || op == TROT_OP_LOCAL_ENERGY || op == TROT_OP_PROP_STEP;
  if (meas) {
    m.green = c.take<double2>(W * sp.ntot * N);
    m.e1 = c.take<double2>(2 * W);  // one-body energy per (spin, walker)
    m.nblk_total = 0;
    for (int q = 0; q < sp.nspin; ++q) {
      SpinLayout L = spin_layout(s, sp, q);
      m.gq[q] = c.take<uint16_t>((size_t)L.ntiles * kKS * kSlices * L.P * 16);
      m.ge[q] = c.take<int32_t>((size_t)L.ntiles * L.P);
      m.cs[q] = c.take<float4>(W * G);
      m.nblk_total += L.nblk;
    }
    m.xpart = c.take<ExFixed>(W * m.nblk_total);
    m.fb = c.take<double2>(W * G);
  }
  if (op == TROT_OP_APPLY_TROTTER || op == TROT_OP_PROP_STEP) {
    m.mpad = (int)((2 * W + 127) / 128 * 128);
    m.xs = c.take<double2>(W * G);
    m.xq = c.take<uint16_t>((size_t)s->mixed->vhs_slices * m.mpad * s->mixed->gpad);
    m.vhs = c.take<float>((size_t)m.mpad * s->mixed->n2pad);
    if (s->mixed->exp_h1_half_img) {
      m.vimg = c.take<uint16_t>(W * (kTcImgBytes / 2));
      m.ov_new = c.take<double2>(W);
      m.ovp = c.take<double2>(2 * W);
    }
    m.shift_term = c.take<double2>(W);
    m.fb_term = c.take<double2>(W);
    m.node_flag = c.take<int>(W);
  }
  return c.used;
}

size_t mixed_workspace_size(const trot_system* s, int op) {
  if (!s->mixed) return 0;
  Spins sp = make_spins(s);
  Carver c(nullptr, 0);
  MixedBuffers m;
  return carve_mixed(s, sp, c, m, op);
}

// rint(x 2^s) (round half to even) by integer operations, for |x 2^s| < 2^62; zero and
// subnormal x give 0 (the callers scale the row maximum to 2^40).
TROT_D long long rint_scaled(double x, int s) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((u >> 52) & 0x7FF);
  if (ex == 0 || ex == 0x7FF) return 0;
  const unsigned long long M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const int sh = 1075 - ex - s;  // x 2^s = M 2^(ex - 1075 + s)
  unsigned long long q;
  if (sh <= 0) {
    q = M << (-sh);
  } else if (sh >= 64) {
    q = 0;
  } else {
    q = M >> sh;
    const unsigned long long r = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (r > half || (r == half && (q & 1ull))) ++q;
  }
  return (u >> 63) ? -(long long)q : (long long)q;
}

// ------------------------------------------------------------------ Green's function digits
// Rows (b, spin, j, c in {re, im}) of the half Green's function over orbitals p, as
// exact integer FP16 digits: v = round(x 2^(44 - e)) (|v| <= 2^44, e the smallest
// integer with max |x| <= 2^e), an 8-bit leading digit q_0 = round(v / 2^36) (|q_0| <=
// 256) and balanced 9-bit digits q_1..q_4 (|q| <= 256), so x ~= 2^e sum_t q_t 2^-(8 +
// 9 t).  Written straight into the exchange kernel's B operand image: per walker tile
// (P columns: walker bl, j, c at bl*2*n_pad + 2 j + c), per K16 step, the 5 digit planes
// stacked as 5P rows (plane u at rows u*P ..) of 16 orbitals in core-matrix order; padding
// rows (j >= n, walkers past W) and orbitals p >= N are zero.  One CTA per tile.
__global__ void __launch_bounds__(256)
green_slices_kernel(int N, int n, int n_pad, int P, int WB, int W, int ntot, int off,
                    const double2* __restrict__ green, uint16_t* __restrict__ gq, int32_t* __restrict__ ge) {
  const int tile = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = 2 * n_pad;
  const size_t unit = (size_t)kSlices * P * 16;  // 16-bit entries per K16 step of the tile
  uint16_t* out = gq + (size_t)tile * kKS * unit;
  for (int row = warp; row < P; row += blockDim.x >> 5) {
    const int bl = row / S, rr = row % S;
    const int b = tile * WB + bl;
    const int j = rr >> 1, c = rr & 1;
    const bool valid = bl < WB && b < W && j < n;
    const double* src = valid ? reinterpret_cast<const double*>(green + (size_t)b * ntot * N + (size_t)(off + j) * N)
                              : nullptr;
    double x[kKP / 32];
    unsigned long long mx = 0;
#pragma unroll
    for (int k = 0; k < kKP / 32; ++k) {
      const int p = lane + 32 * k;
      x[k] = (valid && p < N) ? src[2 * p + c] : 0.0;
      const unsigned long long bits = (unsigned long long)__double_as_longlong(x[k]) & 0x7FFFFFFFFFFFFFFFull;
      mx = bits > mx ? bits : mx;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long t = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = t > mx ? t : mx;
    }
    // e = the smallest integer with max |x| <= 2^e, from the bits of the maximum
    const int E = (int)((mx >> 52) & 0x7FF);
    const bool nonfinite = E == 0x7FF;  // the row's digits become NaN, so its products are NaN
    int e = 0;
    if (mx != 0 && !nonfinite) e = E == 0 ? -1022 : (E - 1023) + ((mx & 0xFFFFFFFFFFFFFull) != 0 ? 1 : 0);
    if (lane == 0) ge[(size_t)tile * P + row] = e;
#pragma unroll
    for (int k = 0; k < kKP / 32; ++k) {
      const int p = lane + 32 * k;
      long long v = rint_scaled(x[k], kGreenBits - e);
      uint16_t* dst = out + (size_t)(p >> 4) * unit;
#pragma unroll
      for (int t = 0; t < kSlices; ++t) {
        const int sh = kLowBits * (kSlices - 1 - t);
        const long long d = sh > 0 ? ((v + (1ll << (sh - 1))) >> sh) : v;  // |d| <= 256 for every t
        v -= d << sh;
        const __half h = __int2half_rn((int)d);
        dst[tile16_idx(t * P + row, p & 15)] = nonfinite ? (uint16_t)0x7E00u : __half_as_ushort(h);
      }
    }
  }
}

// ------------------------------------------------------------------ exact exchange / trace kernel
// f_g = rot_chol_g G^T (n x n per Cholesky vector g and walker) from exact FP16 digit
// products on tcgen05, then per walker the exchange sum_g sum_ij f_gij f_gji
// (trot/meas/rhf.py:33-60) and the traces c_g = sum_i f_gii (Coulomb / force bias,
// trot/meas/rhf.py:119-125).
//
// A persistent CTA walks work items = (Cholesky tile: gb vectors x n orbitals = up to
// 128 MMA rows (g, i), run of walker tiles of P columns).  Warp 16 (one lane) is the
// producer.  The rot_chol digits of the item's tile (5 planes x 128 rows x 128 orbitals)
// stay in shared memory, loaded per K16 step (20 KB chunks; each chunk is refilled for the
// next item as soon as the last MMAs that read it have completed, so items do not drain
// the tensor pipe); the Green's-function digits of each walker tile stream through a ring
// of K16 steps (5 planes x P rows each).  Per K16 step the producer issues five MMAs:
// rot plane t against Green's-function planes 0..4-t stacked along N (N = (5 - t) P),
// which accumulates product (t, u) into TMEM group t + u (columns (t + u) P of the tile's
// accumulator buffer) - exactly for t + u <= 1, where every partial sum stays below 2^24.
// Two accumulator buffers (5P columns each, at columns 0 and 256) let the MMAs of the next
// tile run during the epilogue of this one.
//
// Warps 0-15 are the epilogue, one walker of the tile at a time: warp w reads TMEM lane
// quadrant w % 4 (rows r = (g, i)) and the columns of orbitals j in [JH (w / 4), JH (w / 4
// + 1)) of the walker, re and im; it rebuilds f_g[i][j] = 2^(eA + eB - 17) sum_d 2^(-9 d)
// A_d in float-float, stages f in shared memory for the transposed products f_gji, and
// reduces the exchange and the traces in fixed order.
struct ExArgs {
  SpinLayout L;
  int G, W, mult;
  int tiles_per_item, chunks, n_items;  // work item = (Cholesky tile, run of walker tiles)
  const uint16_t* rot_img;   // [nblk][kKS][5][128][16] core-matrix order
  const int32_t* rot_e;      // [nblk][128]
  const uint16_t* green_img; // [ntiles][kKS][5 P][16] core-matrix order
  const int32_t* green_e;    // [ntiles][P]
  float4* cs;
  ExFixed* xpart;
  int nblk_total;
  int* status;
  int test_timeout_polls;  // > 0: the producer's first wait is on a barrier nothing arrives on
};

static constexpr int kExLoaders = 2;     // loader warps: bulk copies issued by one warp complete one after
                                        // another (~700 cycles each), copies of different warps overlap
static constexpr int kExThreads = 32 * (18 + kExLoaders);  // 16 epilogue warps, the MMA warp, the reducer, the loaders
static constexpr int kExEpi = 512;      // epilogue threads
static constexpr int kExSync = 544;     // epilogue + reducer: the per-tile and per-walker barriers
static constexpr int kExKU = 1;         // K16 steps per ring unit (one 7.5 KB bulk copy at P = 48)
static constexpr int kExSlots = 4;      // ring of Green's-function units (two per loader warp)
// unit g goes to slot g % kExSlots and loader g % kExLoaders: every slot is refilled by one loader only,
// which the loaders' bounded drain on the timeout path relies on
static_assert(kExSlots % kExLoaders == 0, "exchange kernel: ring slots per loader");

// One epilogue warp's exchange sum of a walker: fixed-point values V[c] with scale 2^-s[c]
// (s[c] = kExNonFinite: a lane's value was not finite).
struct ExWarpSum {
  long long v[2];
  int s[2];
  int pad[2];
};

static constexpr int kExNonFinite = kExchangeNonFinite;

// Sum over the warp of float-float values as a fixed-point int64 with the warp's own scale:
// returns V with sum ~= V 2^-s (|V| < 2^54), s = kExNonFinite if a lane is not finite.
// Each lane's value x 2^s (|x 2^s| < 2^48) is split into three int32 parts summed exactly by
// redux.sync; only FP32 / int32 conversions are used (64-bit conversions run on the FP64 pipe).
TROT_D long long ex_warp_sum(ff x, int& s_out) {
  const unsigned E = __reduce_max_sync(0xffffffffu, (__float_as_uint(x.hi) >> 23) & 0xFFu);
  if (E == 0xFFu) {
    s_out = kExNonFinite;
    return 0;
  }
  const int s = 174 - (int)E;  // |x| < 2^(E - 126)
  const float f1 = pow2f(max(-126, min(127, s >> 1))), f2 = pow2f(max(-126, min(127, s - (s >> 1))));
  const float h = __fmul_rn(__fmul_rn(x.hi, f1), f2), l = __fmul_rn(__fmul_rn(x.lo, f1), f2);
  const float hA = rintf(h * 5.9604644775390625e-08f);      // h / 2^24, |hA| <= 2^24
  const int A = (int)hA;
  const int B = __float2int_rn(__fmaf_rn(-hA, 16777216.f, h));  // h - hA 2^24 is exact, |B| <= 2^23
  const int Lo = __float2int_rn(l);                             // |Lo| <= 2^25
  const int SA = __reduce_add_sync(0xffffffffu, A), SB = __reduce_add_sync(0xffffffffu, B);
  const int SL = __reduce_add_sync(0xffffffffu, Lo);
  s_out = s;
  return ((long long)SA << 24) + (long long)SB + (long long)SL;
}

template <int NP>
struct ExShape {
  static constexpr int P = NP == 16 ? 32 : 48;        // columns per digit plane (= ex_cols)
  static constexpr int WBT = P / (2 * NP);            // walkers per tile
  static constexpr int JH = NP / 4;                   // orbitals j per epilogue thread
  static constexpr uint32_t UB = (uint32_t)kSlices * P * 32;  // one K16 step of a walker tile
  static constexpr int FS = NP + 1;                   // staging row stride (padded against bank conflicts)
  static constexpr int KPT = (NP / 2 + 4) / 4;        // exchange pair offsets k per epilogue thread
  static constexpr size_t offRing = kAImg;
  static constexpr uint32_t UU = kExKU * UB;                                   // one ring unit
  static constexpr size_t offF = offRing + (size_t)kExSlots * UU;              // re, im: [128][FS] ff each
  static constexpr size_t offRed = offF + (size_t)2 * 128 * FS * sizeof(ff);   // [16 warps] per-warp exchange sums
  static constexpr size_t offBar = offRed + (size_t)16 * 32;                    // 34 mbarriers / words
  static constexpr size_t bytes = offBar + 40 * 8 + 1024;                      // + base alignment
};

template <int NP>
__global__ void __launch_bounds__(kExThreads, 1) exchange_exact_kernel(ExArgs a) {
  using X = ExShape<NP>;
  constexpr int P = X::P, WBT = X::WBT, JH = X::JH, FS = X::FS;
  constexpr uint32_t UB = X::UB, UU = X::UU;
  constexpr int kUnits = kKS / kExKU;  // ring units per walker tile
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  unsigned char* sA = base;
  unsigned char* ring = base + X::offRing;
  ff* sF = reinterpret_cast<ff*>(base + X::offF);
  ExWarpSum* sRed = reinterpret_cast<ExWarpSum*>(base + X::offRed);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + X::offBar);
  static_assert(2 * kKS + 2 * kExSlots + 10 <= 40, "exchange kernel: barrier table");
  uint64_t* a_full = bars;                         // [kKS] chunk k of the Cholesky tile has landed
  uint64_t* a_free = bars + kKS;                   // [kKS] the MMAs reading chunk k of the item are done
  uint64_t* full = bars + 2 * kKS;                 // [kExSlots]
  uint64_t* empty = full + kExSlots;               // [kExSlots]
  uint64_t* acc_full = empty + kExSlots;           // [2] a tile's accumulators are complete
  uint64_t* acc_empty = acc_full + 2;              // [2] the epilogue has read them out of TMEM
  uint64_t* never = acc_empty + 2;                 // nothing but the abort path's commit arrives on it
  uint32_t* tslot = reinterpret_cast<uint32_t*>(never + 1);
  volatile int* flag = reinterpret_cast<volatile int*>(never + 2);        // epilogue go/stop broadcast
  volatile int* abort_flag = reinterpret_cast<volatile int*>(never + 3);  // a producer gave up: epilogue stops

  const SpinLayout& L = a.L;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if ((int)blockIdx.x >= a.n_items) return;

  if (warp == 16) tc::tmem_alloc(tslot, 512);
  if (tid == kExEpi) {
    for (int k = 0; k < kKS; ++k) {
      tc::mbar_init(&a_full[k], 1);
      tc::mbar_init(&a_free[k], 1);
    }
    for (int k = 0; k < kExSlots; ++k) {
      tc::mbar_init(&full[k], 1);
      tc::mbar_init(&empty[k], 1);
    }
    for (int k = 0; k < 2; ++k) {
      tc::mbar_init(&acc_full[k], 1);
      tc::mbar_init(&acc_empty[k], 16);
    }
    tc::mbar_init(never, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;

  if (warp == 16) {
    // ------------------------------------------------ MMA issuer (one lane)
    if (lane == 0) {
      bool ok = true;
      uint32_t idesc[kSlices];
#pragma unroll
      for (int t = 0; t < kSlices; ++t) idesc[t] = tc::idesc_f16_f32(128, (kSlices - t) * P);
      // both operands: LBO 128 B (K-adjacent core matrices), SBO 256 B (8-row groups), so the
      // descriptors share their high word and only the start-address words advance
      const uint64_t ad0 = tc::smem_desc(tc::smem_u32(sA), 128, 256);
      const uint64_t bd0 = tc::smem_desc(tc::smem_u32(ring), 128, 256);
      const uint32_t adlo = (uint32_t)ad0, bdlo = (uint32_t)bd0, dhi = (uint32_t)(ad0 >> 32);
      int gs = 0, tg = 0, kitem = 0;  // CTA-wide unit / tile / item counters
      // status-path test (TROT_TUNE_TEST_TIMEOUT): a bounded wait on a barrier nothing
      // arrives on runs out before any MMA is issued
      if (a.test_timeout_polls > 0) ok = tc::mbar_wait(never, 0u, (uint32_t)a.test_timeout_polls);
      for (int item = blockIdx.x; item < a.n_items && ok; item += gridDim.x, ++kitem) {
        const int t0 = (item % a.chunks) * a.tiles_per_item, t1 = min(L.ntiles, t0 + a.tiles_per_item);
        const int ntl = t1 - t0;
        for (int i = 0; i < ntl && ok; ++i) {
          const int tgi = tg + i, buf = tgi & 1;
          // the epilogue has read this accumulator buffer's previous tile out of TMEM
          if (tgi >= 2) {
            ok = tc::mbar_wait(&acc_empty[buf], (uint32_t)(((tgi >> 1) - 1) & 1));
            if (!ok) break;
          }
          const uint32_t dcol = taddr + (uint32_t)(buf * 256);
          for (int k = 0; k < kKS; ++k, ++gs) {
            if (i == 0) {
              ok = tc::mbar_wait(&a_full[k], (uint32_t)(kitem & 1));
              if (!ok) break;
            }
            const int ug = gs / kExKU, slot = ug % kExSlots, kj = gs % kExKU;
            if (kj == 0) {
              ok = tc::mbar_wait(&full[slot], (uint32_t)((ug / kExSlots) & 1));
              if (!ok) break;
            }
            tc::fence_after_sync();
            const uint32_t alo = adlo + (uint32_t)(k * kAStep / 16);
            const uint32_t blo = bdlo + (uint32_t)((slot * UU + kj * UB) / 16);
#pragma unroll
            for (int t = 0; t < kSlices; ++t)
              tc::mma_bf16_lo(dcol + (uint32_t)(t * P), alo + (uint32_t)(t * 256), blo, dhi, idesc[t],
                              (k > 0 || t > 0) ? 1u : 0u);
            if (kj == kExKU - 1) tc::mma_commit(&empty[slot]);
            if (i == ntl - 1) tc::mma_commit(&a_free[k]);  // chunk k of the Cholesky tile may be refilled
          }
          if (ok) tc::mma_commit(&acc_full[buf]);
        }
        tg += ntl;
      }
      if (!ok) {
        report_timeout(a.status);
        *abort_flag = 1;
        // the issued MMAs complete (a commit on a barrier nothing else arrives on) before the
        // epilogue is released: its next accumulator wait completes and it stops
        tc::mma_commit(never);
        tc::mbar_wait(never, 0u, 1000000u);
        tc::mbar_arrive(&acc_full[0]);
        tc::mbar_arrive(&acc_full[1]);
      }
    }
    __syncwarp();
  } else if (warp >= 18) {
    // ------------------------------------------------ loaders (one lane per warp): Green's-function K16
    // step pairs into the ring as slots free up (unit g by loader g % kExLoaders), and (loader 0) the next
    // item's Cholesky chunks as soon as the MMAs reading each chunk completed; non-blocking tests
    // (test_wait), so no stream waits on another
    if (lane == 0) {
      const int w = warp - 18;
      bool ok = a.test_timeout_polls == 0;
      // B stream: item bi, unit bu of it, global unit bg; A stream: item ai (ka-th of this CTA), chunk ak
      int bi = blockIdx.x, bu = 0, bg = 0;
      int ai = w == 0 ? blockIdx.x : a.n_items, ka = 0, ak = 0;
      uint32_t idle = 0, pend_mask = 0, pend_par = 0;
      int last_b = -1;  // this loader's last issued unit
      auto units_of = [&](int item) {
        const int t0 = (item % a.chunks) * a.tiles_per_item;
        return (min(L.ntiles, t0 + a.tiles_per_item) - t0) * kUnits;
      };
      int btot = bi < a.n_items ? units_of(bi) : 0;
      auto advance_b = [&]() {
        ++bg;
        if (++bu == btot) {
          bu = 0;
          bi += gridDim.x;
          btot = bi < a.n_items ? units_of(bi) : 0;
        }
      };
      while (bi < a.n_items && bg % kExLoaders != w) advance_b();
      while (ok && (bi < a.n_items || ai < a.n_items)) {
        bool progress = false;
        if (bi < a.n_items) {
          const int slot = bg % kExSlots;
          if (bg < kExSlots || tc::mbar_test_wait(&empty[slot], (uint32_t)((bg / kExSlots - 1) & 1))) {
            const int t0 = (bi % a.chunks) * a.tiles_per_item;
            const int ti = t0 + bu / kUnits, tk = (bu % kUnits) * kExKU;
            tc::mbar_expect_tx(&full[slot], UU);
            tc::bulk_g2s(ring + (size_t)slot * UU, a.green_img + ((size_t)ti * kKS + tk) * (UB / 2), UU, &full[slot]);
            last_b = bg;
            do advance_b(); while (bi < a.n_items && bg % kExLoaders != w);
            progress = true;
          }
        }
        if (ai < a.n_items && (ka == 0 || tc::mbar_test_wait(&a_free[ak], (uint32_t)((ka - 1) & 1)))) {
          const int blk = ai / a.chunks;
          tc::mbar_expect_tx(&a_full[ak], kAStep);
          tc::bulk_g2s(sA + (size_t)ak * kAStep, a.rot_img + ((size_t)blk * kAImg + (size_t)ak * kAStep) / 2, kAStep,
                       &a_full[ak]);
          pend_mask |= 1u << ak;
          pend_par = (pend_par & ~(1u << ak)) | ((uint32_t)(ka & 1) << ak);
          if (++ak == kKS) {
            ak = 0;
            ai += gridDim.x;
            ++ka;
          }
          progress = true;
        }
        if (progress) {
          idle = 0;
        } else if (++idle > 100000000u || *abort_flag) {  // ~1-2 s of non-blocking polls
          ok = false;
        }
      }
      if (!ok) {
        if (a.test_timeout_polls == 0) report_timeout(a.status);
        // bounded drain of this loader's copies in flight before the CTA releases its memory
        for (int u = last_b; u >= 0 && u > last_b - kExSlots; u -= kExLoaders)
          tc::mbar_wait(&full[u % kExSlots], (uint32_t)((u / kExSlots) & 1), 1000000u);
        for (int k = 0; k < kKS; ++k)
          if (pend_mask & (1u << k)) tc::mbar_wait(&a_full[k], (pend_par >> k) & 1u, 1000000u);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------ epilogue: 16 warps (lane quarter q, orbital range h)
    // and the reducer (warp 17): traces from the staged diagonals, then the walker's exchange
    // from the 16 warp sums, while the epilogue warps move on to the next walker
    constexpr int KPT = X::KPT;
    const bool reducer = warp == 17;
    const int q = warp & 3, h = (warp >> 2) & 3;
    const int r = q * 32 + lane;
    const int n = L.n;
    const int i = r % n, gl = r / n;
    const int j0 = h * JH;
    const uint32_t tlane = taddr + ((uint32_t)(q * 32) << 16);
    ff* sFr = sF;
    ff* sFi = sF + 128 * FS;
    // Exchange sum_ij f_ij f_ji over unordered pairs: row i takes the pairs (i, (i + k) mod n)
    // for k = h, h + 4, ... <= n / 2; weight 2 where 0 < k < n - k (the pair's other order is
    // never visited), 1 for k = 0 and k = n / 2 (visited from both of its rows)
    const int nk = n / 2 + 1;
    bool stop = false;
    int tgl = 0;  // CTA-wide tile counter (accumulator buffer and phase)
    for (int item = blockIdx.x; item < a.n_items && !stop; item += gridDim.x) {
      const int blk = item / a.chunks;
      const int t0 = (item % a.chunks) * a.tiles_per_item, t1 = min(L.ntiles, t0 + a.tiles_per_item);
      const int ntl = t1 - t0;
      const int nvec = min(L.gb, a.G - blk * L.gb);
      const int rows_valid = nvec * n;
      const bool rvalid = r < rows_valid;
      const float sa = pow2f(a.rot_e[(size_t)blk * 128 + r] - kRotTopBits);
      for (int it = 0; it < ntl; ++it, ++tgl) {
        const int tile = t0 + it, buf = tgl & 1;
        // this thread's Green's-function exponents of the tile, loaded before the accumulator wait
        // (green_e holds P entries for every tile, so the loads stay in bounds for partial tiles)
        int ebr[WBT][JH][2];
        if (!reducer) {
          const int32_t* eB = a.green_e + (size_t)tile * P;
#pragma unroll
          for (int bl = 0; bl < WBT; ++bl)
#pragma unroll
            for (int jj = 0; jj < JH; ++jj)
#pragma unroll
              for (int c = 0; c < 2; ++c) ebr[bl][jj][c] = __ldg(eB + bl * 2 * NP + 2 * (j0 + jj) + c);
        }
        if (tid == 0) *flag = (tc::mbar_wait(&acc_full[buf], (uint32_t)((tgl >> 1) & 1)) && *abort_flag == 0) ? 1 : 0;
        tc::named_bar(1, kExSync);
        if (!*flag) {
          if (tid == 0) report_timeout(a.status);
          stop = true;
          break;
        }
        tc::fence_after_sync();
        const int nw = min(WBT, a.W - tile * WBT);
#pragma unroll
        for (int bl = 0; bl < WBT; ++bl) {
          if (bl >= nw) break;  // uniform across the CTA
          const int b = tile * WBT + bl;
          if (!reducer) {
            const int cb = bl * 2 * NP + 2 * j0;  // this thread's first column: (j0, re)
            uint32_t raw[kGroups][2 * JH];
#pragma unroll
            for (int d = 0; d < kGroups; ++d)
#pragma unroll
              for (int x = 0; x < JH; ++x)
                tc::tmem_ld2(tlane + (uint32_t)(buf * 256 + d * P + cb + 2 * x), raw[d][2 * x], raw[d][2 * x + 1]);
            tc::tmem_wait_ld();
            if (bl == nw - 1) {  // the tile's last walker is in registers: release the buffer
              tc::fence_before_sync();
              __syncwarp();
              if (lane == 0) tc::mbar_arrive(&acc_empty[buf]);
            }
#pragma unroll
            for (int jj = 0; jj < JH; ++jj)
#pragma unroll
              for (int c = 0; c < 2; ++c) {
                float g[kGroups];
#pragma unroll
                for (int d = 0; d < kGroups; ++d) {
                  uint32_t v = raw[d][2 * jj + c];
                  asm volatile("" : "+r"(v));  // consume after tcgen05.wait::ld
                  g[d] = __uint_as_float(v);
                }
                // sum_d 2^(-9 d) A_d: the 2^-9d scalings are exact, the leading pair error-free
                ff x = ff_two_sum(g[0], g[1] * 1.953125e-03f);
                float lo = x.lo;
#pragma unroll
                for (int d = 2; d < kGroups; ++d) lo += g[d] * pow2f(-9 * d);
                x = ff_fast(x.hi, lo);
                // times 2^(eA - 9) 2^(eB - 8), as two exact power-of-two factors
                const float sb = pow2f(ebr[bl][jj][c] - kGreenTopBits);
                (c == 0 ? sFr : sFi)[r * FS + j0 + jj] = ff{x.hi * sa * sb, x.lo * sa * sb};
              }
          }
          tc::named_bar(1, kExSync);
          if (!reducer) {
            // exchange products over this row's pairs; f_ij and f_ji both from the staging rows
            const int brow = gl * n;
            ff xr{0.f, 0.f}, xi{0.f, 0.f};
            if (rvalid) {
#pragma unroll
              for (int kk = 0; kk < KPT; ++kk) {
                const int k = h + 4 * kk;
                if (k >= nk) break;
                int j = i + k;
                if (j >= n) j -= n;
                ff ar = sFr[r * FS + j], ai = sFi[r * FS + j];
                const ff br = sFr[(brow + j) * FS + i], bi = sFi[(brow + j) * FS + i];
                if (k != 0 && 2 * k != n) {  // exact doubling
                  ar = ff{2.f * ar.hi, 2.f * ar.lo};
                  ai = ff{2.f * ai.hi, 2.f * ai.lo};
                }
                // (a + ib)(c + id) = (ac - bd) + i(ad + bc)
                ff_mad(xr, ar, br);
                ff_mad(xr, ff{-ai.hi, -ai.lo}, bi);
                ff_mad(xi, ar, bi);
                ff_mad(xi, ai, br);
              }
            }
            int sx0, sx1;
            const long long V0 = ex_warp_sum(ff_fast(xr.hi, xr.lo), sx0);
            const long long V1 = ex_warp_sum(ff_fast(xi.hi, xi.lo), sx1);
            if (lane == 0) sRed[warp] = ExWarpSum{{V0, V1}, {sx0, sx1}, {0, 0}};
          } else {
            // traces c_g = sum_i f_gii of the tile's vectors, float-float in fixed order: S lanes
            // per vector (a power of two) sum every S-th diagonal term, then S-lane shuffles
            int S = 1;
            while (S * 2 * nvec <= 32) S *= 2;
            for (int v0 = 0; v0 < nvec; v0 += 32 / S) {
              const int v = v0 + lane / S, sub = lane % S;
              ff tr{0.f, 0.f}, ti{0.f, 0.f};
              if (v < nvec)
                for (int ii = sub; ii < n; ii += S) {
                  const int rr = v * n + ii;
                  tr = ff_add(tr, sFr[rr * FS + ii]);
                  ti = ff_add(ti, sFi[rr * FS + ii]);
                }
              for (int o = S / 2; o > 0; o >>= 1) {
                tr = ff_add(tr, ff_shfl_xor(tr, o));
                ti = ff_add(ti, ff_shfl_xor(ti, o));
              }
              if (sub == 0 && v < nvec) a.cs[(size_t)b * a.G + blk * L.gb + v] = make_float4(tr.hi, tr.lo, ti.hi, ti.lo);
            }
          }
          tc::named_bar(1, kExSync);
          if (reducer) {
            // the 16 warp sums (lanes 0-15: re, 16-31: im) aligned to the coarsest scale of each
            // half, then one exact integer sum per half; converted to FP64 by the energy combine
            const int c = lane >> 4;
            long long V = sRed[lane & 15].v[c];
            const int sw = sRed[lane & 15].s[c];
            const unsigned badm = __ballot_sync(0xffffffffu, sw == kExNonFinite);
            int smin = sw == kExNonFinite ? 0x7fffffff : sw;
            for (int o = 8; o > 0; o >>= 1) smin = min(smin, __shfl_xor_sync(0xffffffffu, smin, o));
            const int sh = sw == kExNonFinite ? 62 : sw - smin;
            V = sh >= 62 ? 0ll : (sh > 0 ? (V + (1ll << (sh - 1))) >> sh : V);
            for (int o = 8; o > 0; o >>= 1) V += __shfl_xor_sync(0xffffffffu, V, o);
            if ((lane & 15) == 0) {
              ExFixed* out = a.xpart + (size_t)b * a.nblk_total + L.blk_off + blk;
              const bool bad = ((badm >> (16 * c)) & 0xFFFFu) != 0;
              out->v[c] = V * a.mult;
              out->s[c] = (bad || smin == 0x7fffffff) ? (bad ? kExNonFinite : 0) : smin;
            }
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 16) tc::tmem_dealloc(taddr, 512);
}

// fb = sum_s mult_s c_s   (complex, W x G)
// (the traces arrive as float-float pairs (re.hi, re.lo, im.hi, im.lo))
__global__ void fb_combine_kernel(int n, int nspin, int m0, int m1, const float4* __restrict__ c0,
                                  const float4* __restrict__ c1, double2* __restrict__ fb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float4 a = c0[k];
  double2 v = cscale(cmk(ff_d(ff{a.x, a.y}), ff_d(ff{a.z, a.w})), (double)m0);
  if (nspin == 2) {
    const float4 b = c1[k];
    v = cadd(v, cscale(cmk(ff_d(ff{b.x, b.y}), ff_d(ff{b.z, b.w})), (double)m1));
  }
  fb[k] = v;
}

// ------------------------------------------------------------------ VHS
// VHS rows (walker b, re/im) = sum over g of x_shifted[b][g] L_g, as
// D = sum_{t + u <= 2} X_t . Lt_u^T with 3-term bf16 splits, FP32 accumulation.
// Operands are stored as shared-memory images per K chunk of 64:
//   X: [mtile][kchunk][slice][128][64]  (mtile = 128 rows (b, re/im))
//   L: [ntile][kchunk][slice][128][64]  (ntile = 128 orbital pairs pq)
// each 128 x 64 slice tile in core-matrix order (tc::tile_off).
static constexpr int kVK = 64;
static constexpr uint32_t kVSlice = 128 * kVK * 2;        // 16 KB
static constexpr uint32_t kVStage = 6 * kVSlice;          // 3 X + 3 L slices: 96 KB
static constexpr int kVThreads = 160;                     // 4 epilogue warps + 1 producer warp
static constexpr size_t kVhsSmem = 2 * (size_t)kVStage + 16 * 8 + 1024;

// Shifted fields -> 3-term bf16 split in the X image layout.
__global__ void x_slices_kernel(int W, int G, int gpad, int mpad, const double2* __restrict__ xs,
                                uint16_t* __restrict__ xq) {
  const int nkc = gpad / kVK;
  const size_t total = (size_t)mpad * gpad;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int row = (int)(e / gpad), g = (int)(e % gpad);
    const int b = row >> 1, c = row & 1;
    float x = 0.f;
    if (b < W && g < G) {
      const double2 v = xs[(size_t)b * G + g];
      x = (float)(c ? v.y : v.x);
    }
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
    const int mt = row >> 7, rr = row & 127, kc = g / kVK, kk = g % kVK;
    const size_t base = (((size_t)mt * nkc + kc) * 3) * (kVSlice / 2) + tc::tile_off(rr, kk) / 2;
    xq[base] = *reinterpret_cast<const uint16_t*>(&h);
    xq[base + kVSlice / 2] = *reinterpret_cast<const uint16_t*>(&m);
    xq[base + kVSlice] = *reinterpret_cast<const uint16_t*>(&l);
  }
}

__global__ void __launch_bounds__(kVThreads, 1)
vhs_gemm_kernel(int mtiles, int ntiles, int gpad, int n2pad, const uint16_t* __restrict__ xq,
                const uint16_t* __restrict__ lq, float* __restrict__ D, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + 2 * kVStage);
  uint64_t* full = bars;           // [2] stages
  uint64_t* empty = bars + 2;      // [2]
  uint64_t* acc_full = bars + 4;   // [2]
  uint64_t* acc_empty = bars + 6;  // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 8);
  int* flag = reinterpret_cast<int*>(bars + 9);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkc = gpad / kVK;
  // this CTA's tiles: linear index over (mtile, ntile), strided by the grid
  const int ntot = mtiles * ntiles;
  if (warp == 4) tc::tmem_alloc(tslot, 256);
  if (tid == 128) {
    for (int k = 0; k < 2; ++k) {
      tc::mbar_init(&full[k], 1);
      tc::mbar_init(&empty[k], 1);
      tc::mbar_init(&acc_full[k], 1);
      tc::mbar_init(&acc_empty[k], 4);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  if (warp == 4) {
    if (lane == 0) {
      bool ok = true;
      const uint32_t idesc = tc::idesc_bf16_f32(128, 128);
      const uint32_t su = tc::smem_u32(base);
      int chunk = 0;  // global K-chunk counter of this CTA (stage = chunk & 1)
      int nt = 0;     // tiles of this CTA
      for (int tl = blockIdx.x; tl < ntot && ok; tl += gridDim.x, ++nt) {
        const int mt = tl / ntiles, ntl = tl % ntiles;
        const int abuf = nt & 1;
        if (nt >= 2) ok = tc::mbar_wait(&acc_empty[abuf], (uint32_t)(((nt - 2) / 2) & 1));
        for (int kc = 0; kc < nkc && ok; ++kc, ++chunk) {
          const int st = chunk & 1;
          if (chunk >= 2) ok = tc::mbar_wait(&empty[st], (uint32_t)(((chunk - 2) / 2) & 1));
          if (!ok) break;
          unsigned char* dst = base + (size_t)st * kVStage;
          tc::mbar_expect_tx(&full[st], kVStage);
          tc::bulk_g2s(dst, xq + ((size_t)mt * nkc + kc) * 3 * (kVSlice / 2), 3 * kVSlice, &full[st]);
          tc::bulk_g2s(dst + 3 * kVSlice, lq + ((size_t)ntl * nkc + kc) * 3 * (kVSlice / 2), 3 * kVSlice,
                       &full[st]);
          // MMAs of the previous chunk were issued already; now wait for this chunk's data
          ok = tc::mbar_wait(&full[st], (uint32_t)((chunk / 2) & 1));
          if (!ok) break;
          tc::fence_after_sync();
          const uint64_t s0d = tc::smem_desc(su + (uint32_t)st * kVStage, 128, 1024);
          const uint32_t slo = (uint32_t)s0d, dhi = (uint32_t)(s0d >> 32);  // A and B share the high word
          const uint32_t dcol = taddr + (uint32_t)(abuf * 128);
#pragma unroll
          for (int t = 0; t < 3; ++t)
#pragma unroll
            for (int u = 0; t + u <= 2; ++u)
#pragma unroll
              for (int ks = 0; ks < kVK / 16; ++ks)
                tc::mma_bf16_lo(dcol, slo + (uint32_t)((t * kVSlice + ks * 256) >> 4),
                                slo + (uint32_t)(((3 + u) * kVSlice + ks * 256) >> 4), dhi, idesc,
                                (kc | t | u | ks) ? 1u : 0u);
          tc::mma_commit(&empty[st]);
        }
        if (ok) tc::mma_commit(&acc_full[abuf]);
      }
      if (!ok) {
        report_timeout(status);
        for (int k = 0; k < 2; ++k) tc::mbar_wait(&empty[k], 0u, 1000000u);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warp q reads TMEM lanes 32q..32q+31 (rows of the tile)
    int nt = 0;
    for (int tl = blockIdx.x; tl < ntot; tl += gridDim.x, ++nt) {
      const int mt = tl / ntiles, ntl = tl % ntiles;
      const int abuf = nt & 1;
      if (tid == 0) *flag = tc::mbar_wait(&acc_full[abuf], (uint32_t)((nt / 2) & 1)) ? 1 : 0;
      tc::named_bar(1, 128);
      if (!*flag) {
        if (tid == 0) report_timeout(status);
        break;
      }
      tc::fence_after_sync();
      const uint32_t trow = taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(abuf * 128);
      float* drow = D + (size_t)(mt * 128 + warp * 32 + lane) * n2pad + (size_t)ntl * 128;
      for (int c = 0; c < 8; ++c) {
        float v[16];
        tc::tmem_ld16(trow + c * 16, v);
        float4* d4 = reinterpret_cast<float4*>(drow + c * 16);
        d4[0] = make_float4(v[0], v[1], v[2], v[3]);
        d4[1] = make_float4(v[4], v[5], v[6], v[7]);
        d4[2] = make_float4(v[8], v[9], v[10], v[11]);
        d4[3] = make_float4(v[12], v[13], v[14], v[15]);
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acc_empty[abuf]);
      tc::named_bar(1, 128);  // flag reuse
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 4) tc::tmem_dealloc(taddr, 256);
}

// ------------------------------------------------------------------ FP32 Trotter propagation
// Same algorithm as the FP64 trotter_kernel with float2 arithmetic: the walker's
// VHS (complex N x N, from rows (2b, 2b+1) of D) is staged in shared memory.
// Register-tiled products for the FP32 propagation: each thread owns a block
// of RP rows x RJ columns of the N x nc output.
static constexpr int kRP = 4, kRJ = 2;

// out = E in   (E real N x N in global memory, in / out N x nc in shared memory)
__device__ void real_mm32(int N, int nc, const float* __restrict__ E, const float2* in, float2* out) {
  const int pt = (N + kRP - 1) / kRP, jt = (nc + kRJ - 1) / kRJ;
  for (int tt = threadIdx.x; tt < pt * jt; tt += blockDim.x) {
    const int p0 = (tt / jt) * kRP, j0 = (tt % jt) * kRJ;
    float2 acc[kRP][kRJ];
#pragma unroll
    for (int a = 0; a < kRP; ++a)
#pragma unroll
      for (int c = 0; c < kRJ; ++c) acc[a][c] = make_float2(0.f, 0.f);
    for (int q = 0; q < N; ++q) {
      float e[kRP];
      float2 x[kRJ];
#pragma unroll
      for (int a = 0; a < kRP; ++a) e[a] = p0 + a < N ? __ldg(E + (size_t)(p0 + a) * N + q) : 0.f;
#pragma unroll
      for (int c = 0; c < kRJ; ++c) x[c] = j0 + c < nc ? in[q * nc + j0 + c] : make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < kRP; ++a)
#pragma unroll
        for (int c = 0; c < kRJ; ++c) {
          acc[a][c].x = fmaf(e[a], x[c].x, acc[a][c].x);
          acc[a][c].y = fmaf(e[a], x[c].y, acc[a][c].y);
        }
    }
#pragma unroll
    for (int a = 0; a < kRP; ++a)
#pragma unroll
      for (int c = 0; c < kRJ; ++c)
        if (p0 + a < N && j0 + c < nc) out[(p0 + a) * nc + j0 + c] = acc[a][c];
  }
}

// T2 = (i coef) V T ; O += T2   (V complex N x N, T / T2 / O N x nc, all in shared memory)
__device__ void taylor_term32(int N, int nc, const float2* V, const float2* T, float coef, float2* T2, float2* O) {
  const int pt = (N + kRP - 1) / kRP, jt = (nc + kRJ - 1) / kRJ;
  for (int tt = threadIdx.x; tt < pt * jt; tt += blockDim.x) {
    const int p0 = (tt / jt) * kRP, j0 = (tt % jt) * kRJ;
    float2 acc[kRP][kRJ];
#pragma unroll
    for (int a = 0; a < kRP; ++a)
#pragma unroll
      for (int c = 0; c < kRJ; ++c) acc[a][c] = make_float2(0.f, 0.f);
    for (int q = 0; q < N; ++q) {
      float2 v[kRP], x[kRJ];
#pragma unroll
      for (int a = 0; a < kRP; ++a) v[a] = p0 + a < N ? V[(p0 + a) * N + q] : make_float2(0.f, 0.f);
#pragma unroll
      for (int c = 0; c < kRJ; ++c) x[c] = j0 + c < nc ? T[q * nc + j0 + c] : make_float2(0.f, 0.f);
#pragma unroll
      for (int a = 0; a < kRP; ++a)
#pragma unroll
        for (int c = 0; c < kRJ; ++c) {
          acc[a][c].x = fmaf(v[a].x, x[c].x, acc[a][c].x);
          acc[a][c].x = fmaf(-v[a].y, x[c].y, acc[a][c].x);
          acc[a][c].y = fmaf(v[a].x, x[c].y, acc[a][c].y);
          acc[a][c].y = fmaf(v[a].y, x[c].x, acc[a][c].y);
        }
    }
#pragma unroll
    for (int a = 0; a < kRP; ++a)
#pragma unroll
      for (int c = 0; c < kRJ; ++c)
        if (p0 + a < N && j0 + c < nc) {
          const int e = (p0 + a) * nc + j0 + c;
          const float2 t = make_float2(-coef * acc[a][c].y, coef * acc[a][c].x);
          T2[e] = t;
          O[e] = make_float2(O[e].x + t.x, O[e].y + t.y);
        }
  }
}

// column of V[p][q] in the VHS GEMM output: p N + q, or its packed upper-triangle
// column k(min, max) when the Cholesky image is packed (symmetric L: V is symmetric)
__device__ __forceinline__ size_t vhs_col(int p, int q, int N, int packed) {
  if (!packed) return (size_t)p * N + q;
  if (p > q) {
    const int t = p;
    p = q;
    q = t;
  }
  return (size_t)p * N - (size_t)p * (p - 1) / 2 + (q - p);
}

struct Trot32Args {
  TrotterArgs t;
  const float* vhs;
  int n2pad, packed;
  const float* expH32;
};

__global__ void __launch_bounds__(256) trotter32_kernel(Spins sp, Trot32Args a32) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ double2 red[32];
  __shared__ int piv;
  const TrotterArgs& a = a32.t;
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  const int N = a.N, nc = sp.ntot;
  // regions rounded to 16 bytes so the FP64 (double2) views below stay aligned for any N
  const size_t vbytes = ((size_t)N * N * sizeof(float2) + 15) & ~(size_t)15;
  const size_t tbytes = ((size_t)N * nc * sizeof(float2) + 15) & ~(size_t)15;
  float2* V = reinterpret_cast<float2*>(smem_raw);  // N x N
  float2* O = reinterpret_cast<float2*>(smem_raw + vbytes);
  float2* T = reinterpret_cast<float2*>(smem_raw + vbytes + tbytes);
  float2* T2 = reinterpret_cast<float2*>(smem_raw + vbytes + 2 * tbytes);
  unsigned char* extra = smem_raw + vbytes + 3 * tbytes;
  const float* vre = a32.vhs + (size_t)(2 * b) * a32.n2pad;
  const float* vim = vre + a32.n2pad;
  for (int e = tid; e < N * N; e += nt) {
    const size_t c = vhs_col(e / N, e % N, N, a32.packed);
    V[e] = make_float2(vre[c], vim[c]);
  }
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    const double2* w = (s == 0 ? a.in_a : a.in_b) + (size_t)b * N * n;
    for (int e = tid; e < N * n; e += nt) {
      const double2 x = w[e];
      T2[(e / n) * nc + sp.off[s] + e % n] = make_float2((float)x.x, (float)x.y);
    }
  }
  __syncthreads();
  real_mm32(N, nc, a32.expH32, T2, O);
  __syncthreads();
  for (int e = tid; e < N * nc; e += nt) T[e] = O[e];
  __syncthreads();
  for (int k = 1; k <= a.nterms; ++k) {
    taylor_term32(N, nc, V, T, (float)(a.sqrt_dt / (double)k), T2, O);
    __syncthreads();
    float2* tmp = T; T = T2; T2 = tmp;
  }
  real_mm32(N, nc, a32.expH32, O, T2);
  __syncthreads();
  // FP64 copy of the propagated walker: in the (now free) VHS region when it
  // fits, else in the extra region after the three tiles; the LU scratch uses
  // the dead O and T tiles, which never overlap it.
  const size_t w2_bytes = (size_t)N * nc * sizeof(double2);
  double2* W2 = w2_bytes <= vbytes ? reinterpret_cast<double2*>(smem_raw) : reinterpret_cast<double2*>(extra);
  for (int e = tid; e < N * nc; e += nt) W2[e] = make_double2((double)T2[e].x, (double)T2[e].y);
  __syncthreads();
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    double2* w = (s == 0 ? a.out_a : a.out_b) + (size_t)b * N * n;
    for (int e = tid; e < N * n; e += nt) w[e] = W2[(e / n) * nc + sp.off[s] + e % n];
  }
  if (a.overlaps == nullptr) return;
  // n x n scratch over the dead O, T, T2 tiles (16-byte aligned, n^2 * 16 <= 2 * tbytes)
  double2* Ms = reinterpret_cast<double2*>(smem_raw + vbytes);
  overlap_and_weight(sp, a, N, nc, W2, Ms, &piv, red);
}

// ------------------------------------------------------------------ tensor-core Trotter propagation
// Same algorithm as trotter32_kernel with every product on the tensor cores:
//   step 0:          T0 = E w                      (E = exp(-dt/2 h1_eff), real)
//   steps k=1..K:    T_k = (i sqrt(dt)/k) V T_{k-1}, O = T0 + ... + T_K
//   step K+1:        w' = E O
// The A operand (128 rows p x K) is streamed from global memory in 32-wide K chunks of
// 3 BF16 slices (24 KB each): E (K = 128, 4 chunks, shared by all walkers) or the
// walker's [Vr | Vi] (8 chunks: 0-3 are Vr, 4-7 are Vi).  The B operand (NB rows x
// K = 128, 3 slices) holds the previous term T in shared memory, row 2j = Re T_j and row
// 2j + 1 = Im T_j.  A V step accumulates Vr B (chunks 0-3) and Vi B (chunks 4-7) into two
// TMEM accumulators D1, D2, and the epilogue forms V T = (D1[2j] - D2[2j+1]) +
// i (D1[2j+1] + D2[2j]); an E step uses D1 only.  3-term BF16 splits of both operands,
// products t + u <= 2 (6 MMAs per 16-wide K step), FP32 accumulation in TMEM (~2^-24
// relative, the FP32 path's accuracy).
// Warps: 0-15 epilogue (warp w: TMEM lanes / orbital rows 32 (w % 4) .., output columns of
// quarter w / 4, accumulating O in registers), warp 16 lane 0 issues the MMAs, warps 17-19
// lane 0 load A chunks into a ring of kTcStages<NB> slots (chunk c by loader c % 3; bulk copies of
// different warps are in flight together, copies of one warp complete one after another).
// Each CTA carries WPC walkers through the steps in lockstep: while the epilogue turns
// walker 0's accumulators into its next B operand the tensor core runs walker 1's step.
// The new overlaps and phaseless weights are computed afterwards by the float-float
// determinant kernel (overlap_weight_ff_kernel).
static constexpr int kTcLoaders = 3;
static constexpr int kTcEpi = 512;                              // epilogue threads (16 warps)
static constexpr int kTcThreads = kTcEpi + 32 * (1 + kTcLoaders);
static constexpr int kTcKC = 32;                                // K per A / B chunk
static constexpr uint32_t kTcSlice = 128 * kTcKC * 2;           // 8 KB: one slice of one A chunk
static constexpr uint32_t kTcChunk = 3 * kTcSlice;              // 24 KB
static constexpr int kTcWPC = 2;                                // walkers per CTA
static constexpr int kTcMaxStages = 9;

// B operand layout: K-major core matrices (8 rows x 16 B) with the K-adjacent ones 144 B
// apart (LBO) and 8-row groups 576 B apart (SBO).  The 16 B of padding per core matrix put
// the four 8-lane groups of an epilogue warp's stores (lanes = K) on distinct banks.
static constexpr uint32_t kTcBLbo = 144, kTcBSbo = 4 * kTcBLbo;
__host__ __device__ __forceinline__ uint32_t tc_b_off(int r, int k) {
  return (uint32_t)((r >> 3) * kTcBSbo + (k >> 3) * kTcBLbo + (r & 7) * 16 + (k & 7) * 2);
}

template <int NB>
struct TcShape {
  static constexpr uint32_t BSlice = (uint32_t)(NB / 8) * kTcBSbo;  // one slice of one K chunk
  static constexpr uint32_t BBytes = 4u * 3u * BSlice;                // B image of one walker (K = 128)
  static constexpr size_t budget = 227 * 1024 - 1024 - 128 - (size_t)kTcWPC * BBytes;
  // a multiple of the loader count, so every ring slot is refilled by one loader only
  static constexpr int fit = (int)(budget / kTcChunk);
  static constexpr int Stages = (fit > kTcMaxStages ? kTcMaxStages : fit) / kTcLoaders * kTcLoaders;
  static constexpr size_t smem = 128 + (size_t)Stages * kTcChunk + (size_t)kTcWPC * BBytes;
  // per walker two accumulators (Vr / E products, Vi products) of two column blocks each
  static constexpr int WalkerCols = 4 * NB;
  static constexpr uint32_t TmemCols = kTcWPC * WalkerCols <= 128 ? 128 : (kTcWPC * WalkerCols <= 256 ? 256 : 512);
  static_assert(Stages >= kTcLoaders, "tensor-core Trotter: ring");
  static_assert(smem <= 227 * 1024, "tensor-core Trotter shared memory");
  static_assert(kTcWPC * WalkerCols <= 512, "tensor-core Trotter TMEM columns");
};

struct TrotTcArgs {
  TrotterArgs t;
  const uint16_t* vimg;  // (W, 8 chunks, 3, 128, 32) bf16 image of [Vr | Vi]
  const uint16_t* eimg;  // (4 chunks, 3, 128, 32) bf16 image of E
  int* status;
};

__device__ __forceinline__ void split3_bf16(float x, uint16_t& h, uint16_t& m, uint16_t& l) {
  const __nv_bfloat16 bh = __float2bfloat16_rn(x);
  const float r1 = x - __bfloat162float(bh);
  const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
  const __nv_bfloat16 bl = __float2bfloat16_rn(r1 - __bfloat162float(bm));
  h = *reinterpret_cast<const uint16_t*>(&bh);
  m = *reinterpret_cast<const uint16_t*>(&bm);
  l = *reinterpret_cast<const uint16_t*>(&bl);
}

// B element (row j, k < 128) = x as 3 slices; B image = [kchunk][slice][NB rows][32]
template <int NB>
__device__ __forceinline__ void put_b(unsigned char* B, int j, int k, float x) {
  uint16_t h, m, l;
  split3_bf16(x, h, m, l);
  constexpr uint32_t sl = TcShape<NB>::BSlice;  // bytes of one slice of one chunk
  unsigned char* c = B + (size_t)(k / kTcKC) * 3 * sl + tc_b_off(j, k % kTcKC);
  *reinterpret_cast<uint16_t*>(c) = h;
  *reinterpret_cast<uint16_t*>(c + sl) = m;
  *reinterpret_cast<uint16_t*>(c + 2 * sl) = l;
}

// A chunk c of a CTA's sequence (steps x walkers x chunks): the source image address.
__device__ __forceinline__ const uint16_t* tc_chunk_src(const TrotTcArgs& g, int b0, int step, int wi, int kc,
                                                        int nterms) {
  const bool vterm = step > 0 && step <= nterms;
  return vterm ? g.vimg + ((size_t)(b0 + wi) * 8 + kc) * (kTcChunk / 2) : g.eimg + (size_t)kc * (kTcChunk / 2);
}

template <int NB>
__global__ void __launch_bounds__(kTcThreads, 1) trotter_tc_kernel(Spins sp, TrotTcArgs g) {
  using X = TcShape<NB>;
  constexpr int WPC = kTcWPC, S = X::Stages, NH = NB / 8;  // complex output columns per epilogue thread
  constexpr uint32_t kBBytes = X::BBytes;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2 * kTcMaxStages + 2 * WPC + 1];
  __shared__ uint32_t tslot;
  __shared__ volatile int abort_flag;
  __shared__ float coefs[18];  // sqrt(dt) / k rounded once from FP64 (the FP64 pipe is narrow: one division per k)
  // no swizzling: 128-byte alignment serves the bulk copies and the descriptors
  unsigned char* base = smem_raw + ((128 - (tc::smem_u32(smem_raw) & 127)) & 127);
  unsigned char* Abuf = base;                          // S x 24 KB
  unsigned char* Bbuf = base + (size_t)S * kTcChunk;   // WPC x kBBytes
  uint64_t* full = bars;                 // [S] an A chunk has landed
  uint64_t* empty = bars + S;            // [S] the MMAs reading the slot are done
  uint64_t* acc_full = bars + 2 * S;     // [WPC]
  uint64_t* b_ready = acc_full + WPC;    // [WPC]
  uint64_t* drain = b_ready + WPC;       // the abort path's commit
  const TrotterArgs& a = g.t;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int N = a.N, nc = sp.ntot, nterms = a.nterms;
  const int nsteps = nterms + 2;  // E, V x nterms, E
  const int b0 = blockIdx.x * WPC;
  const int nw = min(WPC, a.W - b0);
  if (warp == 16) tc::tmem_alloc(&tslot, X::TmemCols);
  if (tid < 18) coefs[tid] = tid == 0 ? 1.f : (float)(a.sqrt_dt / (double)tid);
  if (tid == kTcEpi) {
    for (int k = 0; k < S; ++k) {
      tc::mbar_init(&full[k], 1);
      tc::mbar_init(&empty[k], 1);
    }
    for (int wi = 0; wi < WPC; ++wi) {
      tc::mbar_init(&acc_full[wi], 1);
      tc::mbar_init(&b_ready[wi], kTcEpi);
    }
    tc::mbar_init(drain, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  {  // zero the B images: padding rows (j >= 2 nc) and K rows (p >= N) stay zero
    uint4* bz = reinterpret_cast<uint4*>(Bbuf);
    for (int e = tid; e < (int)(WPC * kBBytes / 16); e += kTcThreads) bz[e] = make_uint4(0u, 0u, 0u, 0u);
    tc::fence_proxy_async();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = tslot;
  if (warp == 16) {
    // ------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool ok = true;
      const uint32_t idesc2 = tc::idesc_bf16_f32(128, 2 * NB), idesc1 = tc::idesc_bf16_f32(128, NB);
      const uint32_t sa = tc::smem_u32(Abuf), sb = tc::smem_u32(Bbuf);
      constexpr uint32_t bsl = X::BSlice;
      const uint32_t bhi = (uint32_t)(tc::smem_desc(sb, kTcBLbo, kTcBSbo) >> 32);
      int c = 0;
      for (int step = 0; step < nsteps && ok; ++step) {
        const bool vterm = step > 0 && step <= nterms;
        const int nk = vterm ? 8 : 4;
        for (int wi = 0; wi < nw && ok; ++wi) {
          const uint32_t bw = sb + (uint32_t)wi * kBBytes;
          // this walker's B operand for the step is written by the epilogue
          ok = tc::mbar_wait(&b_ready[wi], (uint32_t)(step & 1));
          for (int kc = 0; kc < nk && ok; ++kc, ++c) {
            const int st = c % S;
            ok = tc::mbar_wait(&full[st], (uint32_t)((c / S) & 1));
            if (!ok) break;
            tc::fence_after_sync();
            const uint64_t a0 = tc::smem_desc(sa + (uint32_t)st * kTcChunk, 128, 512);
            const uint32_t alo = (uint32_t)a0, ahi = (uint32_t)(a0 >> 32);
            const int kb = kc & 3;
            const uint32_t blo = (uint32_t)tc::smem_desc(bw + (uint32_t)kb * 3 * bsl, kTcBLbo, kTcBSbo);
            const uint32_t dcol = taddr + (uint32_t)(wi * X::WalkerCols + (kc >= 4 ? 2 * NB : 0));
            // B slices 0 and 1 are adjacent rows of the B image, so one MMA of N = 2 NB takes both
            // (TMEM blocks X, Y of the accumulator): A_t [B_0; B_1] for t = 0, 1, 2, then A_0 B_2 into
            // block X.  Products t + u <= 2 plus A_2 B_1; four MMAs per 16-wide K step, each reading
            // its A slice once (the per-MMA A read from shared memory is what bounds these MMAs).
#pragma unroll
            for (int ks = 0; ks < kTcKC / 16; ++ks) {
              const uint32_t ak = alo + (uint32_t)((ks * 256) >> 4), bk = blo + (uint32_t)((ks * 2 * kTcBLbo) >> 4);
#pragma unroll
              for (int t = 0; t < 3; ++t)
                tc::mma_bf16_lo2(dcol, ak + (uint32_t)((t * kTcSlice) >> 4), ahi, bk, bhi, idesc2,
                                 (kb | ks | t) ? 1u : 0u);
              tc::mma_bf16_lo2(dcol, ak, ahi, bk + (uint32_t)((2 * bsl) >> 4), bhi, idesc1, 1u);
            }
            tc::mma_commit(&empty[st]);
          }
          if (ok) tc::mma_commit(&acc_full[wi]);
        }
      }
      if (!ok) {
        report_timeout(g.status);
        abort_flag = 1;
        // the MMAs already issued complete before the epilogue is released and TMEM is freed
        tc::mma_commit(drain);
        tc::mbar_wait(drain, 0u, 1000000u);
        for (int wi = 0; wi < WPC; ++wi) tc::mbar_arrive(&acc_full[wi]);
      }
    }
    __syncwarp();
  } else if (warp > 16) {
    // ------------------------------------------------ loaders: chunk c by loader c % kTcLoaders
    if (lane == 0) {
      const int w = warp - 17;
      bool ok = true;
      int last = -1;  // this loader's last issued chunk
      int c = 0;
      for (int step = 0; step < nsteps && ok; ++step) {
        const int nk = (step > 0 && step <= nterms) ? 8 : 4;
        for (int wi = 0; wi < nw && ok; ++wi)
          for (int kc = 0; kc < nk; ++kc, ++c) {
            if (c % kTcLoaders != w) continue;
            const int st = c % S;
            if (c >= S) {  // the MMAs of chunk c - S have read the slot
              const uint32_t par = (uint32_t)(((c / S) - 1) & 1);
              uint32_t polls = 0;
              while (!tc::mbar_try_wait(&empty[st], par))  // suspends between polls
                if (abort_flag || ++polls > 20000000u) {
                  ok = false;
                  break;
                }
              if (!ok) break;
            }
            tc::mbar_expect_tx(&full[st], kTcChunk);
            tc::bulk_g2s(Abuf + (size_t)st * kTcChunk, tc_chunk_src(g, b0, step, wi, kc, nterms), kTcChunk,
                         &full[st]);
            last = c;
          }
      }
      if (!ok) {
        if (!abort_flag) report_timeout(g.status);
        // bounded drain of this loader's copies in flight (its slots are its own: S is a
        // multiple of the loader count) before the CTA releases its shared memory
        for (int u = last; u >= 0 && u > last - S; u -= kTcLoaders)
          tc::mbar_wait(&full[u % S], (uint32_t)((u / S) & 1), 1000000u);
      }
    }
    __syncwarp();
  } else {
    // thread: orbital row p (TMEM lane), complex output columns j = jbase + jj, jj < NH
    const int q = warp & 3, h = warp >> 2;
    const int p = q * 32 + lane;
    const bool prow = p < N;
    const int jbase = h * NH;
    float orr[WPC][NH], oi[WPC][NH];
#pragma unroll
    for (int wi = 0; wi < WPC; ++wi)
#pragma unroll
      for (int jj = 0; jj < NH; ++jj) { orr[wi][jj] = 0.f; oi[wi][jj] = 0.f; }
    // step 0 operand: B[2j][p] = Re w[p][j], B[2j+1][p] = Im w[p][j]
    for (int wi = 0; wi < nw; ++wi) {
      unsigned char* B = Bbuf + (size_t)wi * kBBytes;
      const int b = b0 + wi;
#pragma unroll
      for (int jj = 0; jj < NH; ++jj) {
        const int j = jbase + jj;
        if (j < nc) {
          const int s = j < sp.n[0] ? 0 : 1, n = s ? sp.n[1] : sp.n[0], col = s ? j - sp.off[1] : j;
          const double2* w = (s == 0 ? a.in_a : a.in_b) + (size_t)b * N * n;
          const double2 x = prow ? w[(size_t)p * n + col] : make_double2(0.0, 0.0);
          put_b<NB>(B, 2 * j, p, d2f_bits(x.x));
          put_b<NB>(B, 2 * j + 1, p, d2f_bits(x.y));
        }
      }
      tc::fence_proxy_async();
      tc::fence_before_sync();
      tc::mbar_arrive(&b_ready[wi]);
    }
    bool ok = true;
    for (int step = 0; step < nsteps && ok; ++step) {
      const bool vterm = step > 0 && step <= nterms;
      const bool next_is_v = step < nterms;  // the operand built now feeds a V step
      const float coef = coefs[step < 18 ? step : 0];
#pragma unroll
      for (int wi = 0; wi < WPC; ++wi) {
        if (wi >= nw) break;
        if (!tc::mbar_wait(&acc_full[wi], (uint32_t)(step & 1)) || abort_flag) {
          if (!abort_flag) report_timeout(g.status);
          ok = false;
          break;
        }
        tc::fence_after_sync();
        float d[2 * NH];
        const uint32_t tl = taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(wi * X::WalkerCols + h * 2 * NH);
        {  // accumulator = block X + block Y
          uint32_t rx[2 * NH], ry[2 * NH];
#pragma unroll
          for (int c = 0; c < 2 * NH; c += 4) {
            tc::tmem_ld4_raw(tl + c, rx + c);
            tc::tmem_ld4_raw(tl + NB + c, ry + c);
          }
          tc::tmem_wait_ld();
#pragma unroll
          for (int c = 0; c < 2 * NH; ++c) {
            uint32_t x = rx[c], y = ry[c];
            asm volatile("" : "+r"(x), "+r"(y));  // consume after tcgen05.wait::ld
            d[c] = __uint_as_float(x) + __uint_as_float(y);
          }
          if (vterm) {  // the Vi accumulator
#pragma unroll
            for (int c = 0; c < 2 * NH; c += 4) {
              tc::tmem_ld4_raw(tl + 2 * NB + c, rx + c);
              tc::tmem_ld4_raw(tl + 3 * NB + c, ry + c);
            }
            tc::tmem_wait_ld();
#pragma unroll
            for (int jj = 0; jj < NH; ++jj) {
              uint32_t xr = rx[2 * jj], xi = rx[2 * jj + 1], yr = ry[2 * jj], yi = ry[2 * jj + 1];
              asm volatile("" : "+r"(xr), "+r"(xi), "+r"(yr), "+r"(yi));
              const float vr = __uint_as_float(xr) + __uint_as_float(yr), vi = __uint_as_float(xi) + __uint_as_float(yi);
              // V T = (Vr Tr - Vi Ti) + i (Vr Ti + Vi Tr)
              const float re = d[2 * jj] - vi, im = d[2 * jj + 1] + vr;
              d[2 * jj] = re;
              d[2 * jj + 1] = im;
            }
          }
        }
        const int b = b0 + wi;
        if (step == nsteps - 1) {  // w' = E O
#pragma unroll
          for (int jj = 0; jj < NH; ++jj) {
            const int j = jbase + jj;
            if (j < nc && prow) {
              const int s = j < sp.n[0] ? 0 : 1, n = s ? sp.n[1] : sp.n[0], col = s ? j - sp.off[1] : j;
              (s == 0 ? a.out_a : a.out_b)[((size_t)b * N + p) * n + col] =
                  make_double2(f2d_bits(d[2 * jj]), f2d_bits(d[2 * jj + 1]));
            }
          }
          continue;
        }
        unsigned char* B = Bbuf + (size_t)wi * kBBytes;
#pragma unroll
        for (int jj = 0; jj < NH; ++jj) {
          const int j = jbase + jj;
          if (j < nc) {
            float tr, ti;
            if (step == 0) { tr = d[2 * jj]; ti = d[2 * jj + 1]; }
            else { tr = -coef * d[2 * jj + 1]; ti = coef * d[2 * jj]; }
            orr[wi][jj] += tr;
            oi[wi][jj] += ti;
            put_b<NB>(B, 2 * j, p, next_is_v ? tr : orr[wi][jj]);
            put_b<NB>(B, 2 * j + 1, p, next_is_v ? ti : oi[wi][jj]);
          }
        }
        tc::fence_proxy_async();
        tc::fence_before_sync();
        tc::mbar_arrive(&b_ready[wi]);
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 16) tc::tmem_dealloc(taddr, X::TmemCols);
}

// [Vr | Vi] of every walker as the A image of trotter_tc_kernel: (W, 8 chunks, 3 slices, 128 rows, 32)
// from the VHS GEMM output (rows 2b / 2b+1 = Re / Im of walker b, n2pad columns pq, packed
// upper triangle when `packed`). One thread per (walker, chunk, row, 8 consecutive k): three
// 16-byte stores.
__global__ void vhs_image_kernel(int W, int N, int n2pad, int packed, const float* __restrict__ D,
                                 uint16_t* __restrict__ img) {
  const size_t total = (size_t)W * 8 * 128 * 4;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int kg = (int)(e & 3), p = (int)((e >> 2) & 127), kc = (int)((e >> 9) & 7);
    const size_t b = e >> 12;
    const int k0 = kc * kTcKC + kg * 8;              // 0..255
    const int im = k0 >= 128 ? 1 : 0, q0 = k0 & 127;
    const float* src = D + (2 * b + im) * (size_t)n2pad;
    uint32_t hw[4], mw[4], lw[4];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
      const float x0 = (p < N && q0 + i < N) ? src[vhs_col(p, q0 + i, N, packed)] : 0.f;
      const float x1 = (p < N && q0 + i + 1 < N) ? src[vhs_col(p, q0 + i + 1, N, packed)] : 0.f;
      uint16_t h0, m0, l0, h1, m1, l1;
      split3_bf16(x0, h0, m0, l0);
      split3_bf16(x1, h1, m1, l1);
      hw[i / 2] = (uint32_t)h0 | ((uint32_t)h1 << 16);
      mw[i / 2] = (uint32_t)m0 | ((uint32_t)m1 << 16);
      lw[i / 2] = (uint32_t)l0 | ((uint32_t)l1 << 16);
    }
    unsigned char* dst =
        reinterpret_cast<unsigned char*>(img) + (b * 8 + kc) * (size_t)kTcChunk + tc::tile_off32(p, kg * 8);
    *reinterpret_cast<uint4*>(dst) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(dst + kTcSlice) = make_uint4(mw[0], mw[1], mw[2], mw[3]);
    *reinterpret_cast<uint4*>(dst + 2 * kTcSlice) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

// phaseless weights from overlaps computed after the propagation
__global__ void tc_weight_kernel(TrotterArgs a, const double2* __restrict__ ov_new) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < a.W) phaseless_update(a, b, ov_new[b]);
}

// New overlaps of the propagated walkers and their phaseless weights:
// M_s = C_s^T w'_s in float-float (four independent accumulators per element),
// det by FP64 Gauss-Jordan; one CTA per (walker, spin) writes det(M_s)^mult_s, then
// overlap_weight_finish_kernel multiplies the spins and applies phaseless_update.
__global__ void __launch_bounds__(256) overlap_weight_ff_kernel(Spins sp, TrotterArgs a, double2* __restrict__ ovp) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int b = blockIdx.x, s = blockIdx.y, tid = threadIdx.x, nt = blockDim.x;
  const int N = a.N;
  const int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
  ffc* Wf = reinterpret_cast<ffc*>(smem_raw);                      // N x n
  ff* Cf = reinterpret_cast<ff*>(Wf + (size_t)N * nmax);            // N x n
  double2* Md = reinterpret_cast<double2*>(Cf + (size_t)N * nmax + ((N * nmax) & 1));  // n x n
  const int n = s ? sp.n[1] : sp.n[0];
  const double2* w = (s == 0 ? a.out_a : a.out_b) + (size_t)b * N * n;
  const double* C = s ? sp.mo[1] : sp.mo[0];
  for (int e = tid; e < N * n; e += nt) {
    const double2 x = w[e];
    Wf[e] = ffc{ff_from_d(x.x), ff_from_d(x.y)};
    Cf[e] = ff_from_d(C[e]);
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e / n, j = e % n;
    ff ar[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    ff ai[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    int p = 0;
    for (; p + 4 <= N; p += 4) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const ff c = Cf[(p + u) * n + i];
        const ffc x = Wf[(p + u) * n + j];
        ff_mad(ar[u], c, x.re);
        ff_mad(ai[u], c, x.im);
      }
    }
    for (; p < N; ++p) {
      const ff c = Cf[p * n + i];
      const ffc x = Wf[p * n + j];
      ff_mad(ar[0], c, x.re);
      ff_mad(ai[0], c, x.im);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      ar[u] = ff_fast(ar[u].hi, ar[u].lo);
      ai[u] = ff_fast(ai[u].hi, ai[u].lo);
    }
    const ff sr = ff_add(ff_add(ar[0], ar[1]), ff_add(ar[2], ar[3]));
    const ff si = ff_add(ff_add(ai[0], ai[1]), ff_add(ai[2], ai[3]));
    Md[e] = make_double2(ff_d(sr), ff_d(si));
  }
  __syncthreads();
  if (tid < 32) {  // LU determinant in FP64 by one warp
    const double2 det = warp_gauss_jordan(Md, n, false, nullptr);
    if (tid == 0) ovp[(size_t)s * a.W + b] = (s ? sp.mult[1] : sp.mult[0]) == 2 ? cmul(det, det) : det;
  }
}

// overlap = prod_s det(M_s)^mult_s, then the phaseless weight update
__global__ void overlap_weight_finish_kernel(int nspin, TrotterArgs a, const double2* __restrict__ ovp) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= a.W) return;
  double2 ov = cmul(cmk(1.0, 0.0), ovp[b]);
  if (nspin == 2) ov = cmul(ov, ovp[(size_t)a.W + b]);
  phaseless_update(a, b, ov);
}

// ------------------------------------------------------------------ host orchestration
static int check_mixed_shapes(const trot_system* s, const Spins& sp) {
  if (!s->mixed) { set_error("mixed precision needs a trot_mixed context"); return TROT_ERR_NULL_PTR; }
  if (s->norb > kKP) { set_error("mixed path: norb %d > %d", s->norb, kKP); return TROT_ERR_UNSUPPORTED; }
  for (int q = 0; q < sp.nspin; ++q)
    if (sp.n[q] > kMaxOcc) { set_error("mixed path: nocc %d > %d", sp.n[q], kMaxOcc); return TROT_ERR_UNSUPPORTED; }
  if (s->mixed->kpad != kKP || s->mixed->slices != kSlices || s->mixed->max_order != kGroups - 1 ||
      s->mixed->digit_format != kDigitFormat) {
    set_error("mixed context layout mismatch (kpad %d, digits %d, order %d, digit format %d)", s->mixed->kpad,
              s->mixed->slices, s->mixed->max_order, s->mixed->digit_format);
    return TROT_ERR_BAD_SHAPE;
  }
  return TROT_OK;
}

template <int NP>
static void exchange_exact_launch(dim3 grid, const ExArgs& a, cudaStream_t st) {
  constexpr size_t smem = ExShape<NP>::bytes;
  static_assert(smem <= 232448, "exchange kernel: shared memory above the 227 KB limit");
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(exchange_exact_kernel<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr_set = true;
  }
  exchange_exact_kernel<NP><<<grid, kExThreads, smem, st>>>(a);
}

static int launch_exchange_exact(int n_pad, dim3 grid, const ExArgs& a, cudaStream_t st) {
  switch (n_pad) {
    case 4: exchange_exact_launch<4>(grid, a, st); break;
    case 8: exchange_exact_launch<8>(grid, a, st); break;
    case 12: exchange_exact_launch<12>(grid, a, st); break;
    case 16: exchange_exact_launch<16>(grid, a, st); break;
    default: set_error("exchange: n_pad = %d unsupported", n_pad); return TROT_ERR_UNSUPPORTED;
  }
  TROT_CHECK_LAUNCH("exchange_exact_kernel");
  return TROT_OK;
}

static int run_slices_and_exchange(const trot_system* s, const Spins& sp, MixedBuffers& m, cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  for (int q = 0; q < sp.nspin; ++q) {
    SpinLayout L = spin_layout(s, sp, q);
    TROT_TIMED("green_slices", st, ([&]() -> int {
      green_slices_kernel<<<L.ntiles, 256, 0, st>>>(N, L.n, L.n_pad, L.P, L.WB, W, sp.ntot, sp.off[q], m.green, m.gq[q],
                                                    m.ge[q]);
      TROT_CHECK_LAUNCH("green_slices_kernel");
      return TROT_OK;
    })());
  }
  for (int q = 0; q < sp.nspin; ++q) {
    SpinLayout L = spin_layout(s, sp, q);
    const int mq = (s->kind == TROT_UHF_U) ? q : 0;
    ExArgs a{};
    a.L = L;
    a.G = G; a.W = W; a.mult = sp.mult[q];
    // persistent grid: one CTA per SM walks (Cholesky tile, run of 8 walker tiles) items
    const int tpi = tune_get(TROT_TUNE_EXCHANGE_TILES);
    a.tiles_per_item = std::min(tpi > 0 ? tpi : 8, L.ntiles);
    a.chunks = (L.ntiles + a.tiles_per_item - 1) / a.tiles_per_item;
    a.n_items = L.nblk * a.chunks;
    a.rot_img = s->mixed->rot_slices[mq];
    a.rot_e = s->mixed->rot_exp[mq];
    a.green_img = m.gq[q];
    a.green_e = m.ge[q];
    a.cs = m.cs[q];
    a.xpart = m.xpart;
    a.nblk_total = m.nblk_total;
    a.status = m.status;
    a.test_timeout_polls = tune_get(TROT_TUNE_TEST_TIMEOUT);
    const int gknob = tune_get(TROT_TUNE_EXCHANGE_GRID);
    dim3 grid(std::min(a.n_items, gknob > 0 ? gknob : 152));
    TROT_TIMED("exchange_exact_tc", st, launch_exchange_exact(L.n_pad, grid, a, st));
  }
  const int n = W * G;
  fb_combine_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, sp.nspin, sp.mult[0], sp.mult[1], m.cs[0],
                                                     sp.nspin == 2 ? m.cs[1] : nullptr, m.fb);
  TROT_CHECK_LAUNCH("fb_combine_kernel");
  return TROT_OK;
}

static void vhs_gemm_attr() {
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(vhs_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVhsSmem);
    attr_set = true;
  }
}

int launch_split3_gemm(int rows, int K, int kpad, int npad, const double2* x, const uint16_t* b_image,
                       uint16_t* xq, float* D, int* status, cudaStream_t st) {
  if (kpad % kVK || npad % 128 || K > kpad || rows <= 0) {
    set_error("split3 GEMM: bad layout rows=%d K=%d kpad=%d npad=%d", rows, K, kpad, npad);
    return TROT_ERR_BAD_SHAPE;
  }
  const int mpad = split3_mpad(rows);
  x_slices_kernel<<<152 * 8, 256, 0, st>>>(rows, K, kpad, mpad, x, xq);
  TROT_CHECK_LAUNCH("x_slices_kernel");
  vhs_gemm_attr();
  const int mtiles = mpad / 128, ntiles = npad / 128;
  const int grid = mtiles * ntiles > 152 ? 152 : mtiles * ntiles;
  vhs_gemm_kernel<<<grid, kVThreads, kVhsSmem, st>>>(mtiles, ntiles, kpad, npad, xq, b_image, D, status);
  TROT_CHECK_LAUNCH("vhs_gemm_kernel");
  return TROT_OK;
}

static int run_vhs(const trot_system* s, MixedBuffers& m, const double2* xs, cudaStream_t st) {
  const int W = s->n_walkers, G = s->nchol;
  const trot_mixed* mx = s->mixed;
  if (mx->vhs_slices != 3 || mx->vhs_order != 2 || mx->gpad % kVK || mx->n2pad % 128) {
    set_error("mixed context: VHS operand layout mismatch");
    return TROT_ERR_BAD_SHAPE;
  }
  TROT_TIMED("x_slices", st, ([&]() -> int {
    x_slices_kernel<<<152 * 8, 256, 0, st>>>(W, G, mx->gpad, m.mpad, xs, m.xq);
    TROT_CHECK_LAUNCH("x_slices_kernel");
    return TROT_OK;
  })());
  vhs_gemm_attr();
  const int mtiles = m.mpad / 128, ntiles = mx->n2pad / 128;
  int grid = mtiles * ntiles;
  if (grid > 152) grid = 152;
  TROT_TIMED("vhs_tc", st, ([&]() -> int {
    vhs_gemm_kernel<<<grid, kVThreads, kVhsSmem, st>>>(mtiles, ntiles, mx->gpad, mx->n2pad, m.xq,
                                                       mx->chol_t_slices, m.vhs, m.status);
    TROT_CHECK_LAUNCH("vhs_gemm_kernel");
    return TROT_OK;
  })());
  return TROT_OK;
}

static int run_trotter32(const trot_system* s, const Spins& sp, const TrotterArgs& t, const MixedBuffers& m,
                         cudaStream_t st) {
  const int N = s->norb;
  const size_t vbytes = ((size_t)N * N * sizeof(float2) + 15) & ~(size_t)15;
  const size_t tbytes = ((size_t)N * sp.ntot * sizeof(float2) + 15) & ~(size_t)15;
  size_t smem = vbytes + 3 * tbytes;
  const size_t need64 = (size_t)N * sp.ntot * sizeof(double2);
  if (need64 > vbytes) smem += need64;  // FP64 walker copy goes after the tiles when it does not fit the VHS region
  if (smem > 220 * 1024) {
    set_error("mixed trotter: %zu bytes of shared memory needed", smem);
    return TROT_ERR_UNSUPPORTED;
  }
  cudaFuncSetAttribute(trotter32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  Trot32Args a{};
  a.t = t;
  a.vhs = m.vhs;
  a.n2pad = s->mixed->n2pad;
  a.packed = s->mixed->vhs_packed;
  a.expH32 = s->mixed->exp_h1_half_f32;
  trotter32_kernel<<<s->n_walkers, 256, smem, st>>>(sp, a);
  TROT_CHECK_LAUNCH("trotter32_kernel");
  return TROT_OK;
}

template <int NB>
static void trotter_tc_launch(const Spins& sp, const TrotTcArgs& g, int W, cudaStream_t st) {
  constexpr size_t smem = TcShape<NB>::smem;
  cudaFuncSetAttribute(trotter_tc_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  trotter_tc_kernel<NB><<<(W + kTcWPC - 1) / kTcWPC, kTcThreads, smem, st>>>(sp, g);
}

static int run_trotter_tc(const trot_system* s, const Spins& sp, const TrotterArgs& t, const MixedBuffers& m,
                          cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, nc = sp.ntot;
  const int NB = (2 * nc + 15) / 16 * 16;
  if (N > 128 || NB > 64 || t.nterms < 1 || t.nterms > 16 || !m.vimg) {
    set_error("tensor-core Trotter: N=%d nc=%d nterms=%d unsupported", N, nc, t.nterms);
    return TROT_ERR_UNSUPPORTED;
  }
  static_assert(kTcImgBytes == 8 * (size_t)kTcChunk, "operand image size");
  TROT_TIMED("vhs_image", st, ([&]() -> int {
    const size_t threads = (size_t)W * 8 * 128 * 4;
    const int blocks = (int)std::min<size_t>((threads + 255) / 256, 152 * 32);
    vhs_image_kernel<<<blocks, 256, 0, st>>>(W, N, s->mixed->n2pad, s->mixed->vhs_packed, m.vhs, m.vimg);
    TROT_CHECK_LAUNCH("vhs_image_kernel");
    return TROT_OK;
  })());
  TrotTcArgs g{};
  g.t = t;
  g.vimg = m.vimg;
  g.eimg = s->mixed->exp_h1_half_img;
  g.status = m.status;
  TROT_TIMED("trotter_tc", st, ([&]() -> int {
    switch (NB) {
      case 16: trotter_tc_launch<16>(sp, g, W, st); break;
      case 32: trotter_tc_launch<32>(sp, g, W, st); break;
      case 48: trotter_tc_launch<48>(sp, g, W, st); break;
      default: trotter_tc_launch<64>(sp, g, W, st); break;
    }
    TROT_CHECK_LAUNCH("trotter_tc_kernel");
    return TROT_OK;
  })());
  if (t.overlaps) {  // step mode: overlaps of the new walkers (float-float C^T w', FP64 LU) and weights
    const int nmax = sp.n[0] > sp.n[1] ? sp.n[0] : sp.n[1];
    const size_t smem = (size_t)N * nmax * (sizeof(ffc) + sizeof(ff)) + 16 + (size_t)nmax * nmax * 16;
    if (smem > 40 * 1024)
      cudaFuncSetAttribute(overlap_weight_ff_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    TROT_TIMED("overlap_weight_ff", st, ([&]() -> int {
      overlap_weight_ff_kernel<<<dim3(W, sp.nspin), 256, smem, st>>>(sp, t, m.ovp);
      TROT_CHECK_LAUNCH("overlap_weight_ff_kernel");
      overlap_weight_finish_kernel<<<(W + 127) / 128, 128, 0, st>>>(sp.nspin, t, m.ovp);
      TROT_CHECK_LAUNCH("overlap_weight_finish_kernel");
      return TROT_OK;
    })());
  }
  return TROT_OK;
}

static int run_trotter(const trot_system* s, const Spins& sp, const TrotterArgs& t, const MixedBuffers& m,
                       cudaStream_t st) {
  if (s->mixed->exp_h1_half_img && m.vimg) return run_trotter_tc(s, sp, t, m, st);
  TROT_TIMED("trotter_fp32", st, run_trotter32(s, sp, t, m, st));
  return TROT_OK;
}

static int begin(const trot_system* s, const Spins& sp, Carver& c, MixedBuffers& m, int op, cudaStream_t st) {
  int rc = check_mixed_shapes(s, sp);
  if (rc != TROT_OK) return rc;
  carve_mixed(s, sp, c, m, op);
  if (!c.ok) {
    set_error("workspace too small: %zu < %zu", c.size, c.used);
    return TROT_ERR_WORKSPACE_TOO_SMALL;
  }
  cudaMemsetAsync(m.status, 0, sizeof(int), st);  // this call's status word (the sticky one persists)
  return TROT_OK;
}

int mixed_force_bias(const trot_system* s, const Spins& sp, const double2* wa, const double2* wb, double2* fb_out,
                     void* ws, size_t ws_bytes, cudaStream_t st) {
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  TROT_TRY(begin(s, sp, c, m, TROT_OP_FORCE_BIAS, st));
  TROT_TRY(launch_green_ff(sp, s->n_walkers, s->norb, wa, wb, m.green, nullptr, st));
  TROT_TRY(run_slices_and_exchange(s, sp, m, st));
  cudaMemcpyAsync(fb_out, m.fb, (size_t)s->n_walkers * s->nchol * sizeof(double2), cudaMemcpyDeviceToDevice, st);
  TROT_CHECK_LAUNCH("cudaMemcpyAsync");
  return TROT_OK;
}

int mixed_local_energy(const trot_system* s, const Spins& sp, const double2* wa, const double2* wb,
                       double2* energy, void* ws, size_t ws_bytes, cudaStream_t st) {
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  TROT_TRY(begin(s, sp, c, m, TROT_OP_LOCAL_ENERGY, st));
  TROT_TRY(launch_green_ff(sp, s->n_walkers, s->norb, wa, wb, m.green, m.e1, st));
  TROT_TRY(run_slices_and_exchange(s, sp, m, st));
  return launch_energy_combine(s->n_walkers, s->nchol, m.nblk_total, s->h0, m.fb, m.e1, sp.nspin, nullptr, energy,
                               st, m.status, m.xpart);
}

int mixed_apply_trotter(const trot_system* s, const Spins& sp, const double2* xs, const TrotterArgs& a, void* ws,
                        size_t ws_bytes, cudaStream_t st) {
  if (!s->mixed) { set_error("mixed precision needs a trot_mixed context"); return TROT_ERR_NULL_PTR; }
  if (s->norb > kKP) { set_error("mixed path: norb %d > %d", s->norb, kKP); return TROT_ERR_UNSUPPORTED; }
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  carve_mixed(s, sp, c, m, TROT_OP_APPLY_TROTTER);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaMemsetAsync(m.status, 0, sizeof(int), st);
  TROT_TRY(run_vhs(s, m, xs, st));
  return run_trotter(s, sp, a, m, st);
}

int mixed_prop_step(const trot_system* s, const Spins& sp, const trot_state* state, const double* fields,
                    double2* energy_out, void* ws, size_t ws_bytes, cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  TROT_TRY(begin(s, sp, c, m, TROT_OP_PROP_STEP, st));
  double2* wa = (double2*)state->walkers_a;
  double2* wb = (double2*)state->walkers_b;
  TROT_TIMED("green_ff", st, launch_green_ff(sp, W, N, wa, wb, m.green, energy_out ? m.e1 : nullptr, st));
  TROT_TRY(run_slices_and_exchange(s, sp, m, st));
  if (energy_out)
    TROT_TIMED("energy_combine", st,
               launch_energy_combine(W, G, m.nblk_total, s->h0, m.fb, m.e1, sp.nspin, nullptr, energy_out, st,
                                     m.status, m.xpart));
  TROT_TIMED("fields", st, launch_fields(W, G, s->sqrt_dt, m.fb, s->mf_shifts_im, fields, m.xs, m.shift_term,
                                         m.fb_term, st));
  TROT_TRY(run_vhs(s, m, m.xs, st));
  TrotterArgs a{};
  a.W = W; a.N = N; a.G = G; a.nterms = s->n_exp_terms; a.sqrt_dt = s->sqrt_dt; a.expH = s->exp_h1_half;
  a.in_a = wa; a.in_b = wb; a.out_a = wa; a.out_b = wb;
  a.overlaps = (double2*)state->overlaps; a.weights = state->weights; a.scalars = state->scalars;
  a.shift_term = m.shift_term; a.fb_term = m.fb_term; a.node_flag = m.node_flag;
  a.dt = s->dt; a.h0_prop = s->h0_prop; a.w_floor = s->weight_floor; a.w_cap = s->weight_cap;
  TROT_TRY(run_trotter(s, sp, a, m, st));
  TROT_TIMED("step_finalize", st, launch_step_finalize(W, state->weights, state->scalars,
                                                       (long long*)state->node_encounters, m.node_flag,
                                                       s->pop_control_damping, s->dt, st, m.status));
  return TROT_OK;
}

}  // namespace trot
