// Mixed-precision (tensor-core) path of the phaseless step and local energy.
//
//  * half Green's functions, LU / log-det, overlaps, weights, energy sums: FP64;
//  * f_g = rot_chol_g G^T for all g (exchange and, through its trace, the force
//    bias / Coulomb term): exact-slice BF16 products on tcgen05 tensor cores,
//    combined in float-float (FP32 pairs) arithmetic — near-FP64 accuracy;
//  * VHS = x_shifted . chol: 3-term BF16 split on tcgen05, FP32 accumulation;
//  * one-body half steps and the Taylor series: FP32 on the CUDA cores.
#include <cuda_bf16.h>

#include "mixed.h"
#include "profile.h"
#include "step_tail.cuh"
#include "tc.cuh"

namespace trot {

// ------------------------------------------------------------------ float-float
struct ff { float hi, lo; };
TROT_D ff ff_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return ff{s, (a - (s - bb)) + (b - bb)};
}
TROT_D ff ff_fast(float a, float b) {
  const float s = a + b;
  return ff{s, b - (s - a)};
}
TROT_D ff ff_add(ff x, ff y) {
  ff s = ff_two_sum(x.hi, y.hi);
  return ff_fast(s.hi, s.lo + x.lo + y.lo);
}
TROT_D ff ff_sub(ff x, ff y) { return ff_add(x, ff{-y.hi, -y.lo}); }
TROT_D ff ff_mul(ff x, ff y) {
  const float p = x.hi * y.hi;
  float e = fmaf(x.hi, y.hi, -p);
  e = fmaf(x.hi, y.lo, e);
  e = fmaf(x.lo, y.hi, e);
  return ff_fast(p, e);
}
TROT_D double ff_d(ff x) { return (double)x.hi + (double)x.lo; }
TROT_D ff ff_shfl_xor(ff x, int o) {
  return ff{__shfl_xor_sync(0xffffffffu, x.hi, o), __shfl_xor_sync(0xffffffffu, x.lo, o)};
}

// ------------------------------------------------------------------ layouts
static constexpr int kKP = 128;       // padded orbital dimension of the exact product
static constexpr int kBN = 96;        // MMA N of the exchange tile (columns = walker rows)
static constexpr int kGroups = 5;     // accumulators for t + u = 0..4
static constexpr int kSlices = 5;

struct SpinLayout {
  int n, n_pad, S, WB, nwb;  // rows per walker S = 2 n_pad, walkers per tile WB
  int gb, nblk, blk_off;     // Cholesky vectors per tile, tiles, offset in the partial array
};

static SpinLayout spin_layout(const trot_system* s, const Spins& sp, int q) {
  SpinLayout L{};
  L.n = sp.n[q];
  L.n_pad = L.n + (L.n & 1);
  L.S = 2 * L.n_pad;
  L.WB = kBN / L.S;
  L.nwb = (s->n_walkers + L.WB - 1) / L.WB;
  const int mq = (s->kind == TROT_UHF_U) ? q : 0;
  L.gb = s->mixed->gammas_per_block[mq];
  L.nblk = s->mixed->n_blocks[mq];
  L.blk_off = q == 0 ? 0 : s->mixed->n_blocks[0];
  if (s->kind != TROT_UHF_U && q == 1) L.blk_off = s->mixed->n_blocks[0];
  return L;
}

struct MixedBuffers {
  double2* green;
  double2* e1;
  uint16_t* gq[2];
  int32_t* ge[2];
  double2* cs[2];
  double2* xpart;
  double2* fb;
  double2* xs;
  double2 *shift_term, *fb_term;
  uint16_t* xq;
  float* vhs;
  int* node_flag;
  int* status;
  int nblk_total, mpad;
};

static size_t carve_mixed(const trot_system* s, const Spins& sp, Carver& c, MixedBuffers& m, int op) {
  const size_t W = s->n_walkers, N = s->norb, G = s->nchol;
  m = MixedBuffers{};
  if (op == TROT_OP_SR || op == TROT_OP_QR) return c.used;
  m.status = c.take<int>(4);
  const bool meas = op == TROT_OP_FORCE_BIAS || op == TROT_OP_LOCAL_ENERGY || op == TROT_OP_PROP_STEP;
  if (meas) {
    m.green = c.take<double2>(W * sp.ntot * N);
    m.e1 = c.take<double2>(W);
    m.nblk_total = 0;
    for (int q = 0; q < sp.nspin; ++q) {
      SpinLayout L = spin_layout(s, sp, q);
      m.gq[q] = c.take<uint16_t>((size_t)kSlices * W * L.S * kKP);
      m.ge[q] = c.take<int32_t>(W * L.S);
      m.cs[q] = c.take<double2>(W * G);
      m.nblk_total += L.nblk;
    }
    m.xpart = c.take<double2>(W * m.nblk_total);
    m.fb = c.take<double2>(W * G);
  }
  if (op == TROT_OP_APPLY_TROTTER || op == TROT_OP_PROP_STEP) {
    m.mpad = (int)((2 * W + 127) / 128 * 128);
    m.xs = c.take<double2>(W * G);
    m.xq = c.take<uint16_t>((size_t)s->mixed->vhs_slices * m.mpad * s->mixed->gpad);
    m.vhs = c.take<float>((size_t)m.mpad * s->mixed->n2pad);
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

// ------------------------------------------------------------------ Green's function slices
// Rows (b, spin, c in {re, im}, j) of the half Green's function over orbitals
// p, as exact fixed-point bf16 slices: v = round(x 2^(40 - e)) (|v| <= 2^40),
// balanced base-256 digits q_0..q_4 (|q| <= 255), x ~= sum_t q_t 2^(e - 8(t+1)).
// Output layout per spin: [slice][walker][row in 0..S)][kpad], rows j >= n zero.
__global__ void __launch_bounds__(256)
green_slices_kernel(int N, int n, int n_pad, int W, int ntot, int off, const double2* __restrict__ green,
                    uint16_t* __restrict__ gq, int32_t* __restrict__ ge) {
  const int b = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int S = 2 * n_pad;
  for (int row = warp; row < S; row += blockDim.x >> 5) {
    const int c = row / n_pad, j = row % n_pad;
    const bool valid = j < n;
    const double* src = reinterpret_cast<const double*>(green + (size_t)b * ntot * N + (size_t)(off + j) * N);
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
    int e = 0;
    if (mx != 0) {
      int ex;
      const double m = frexp(__longlong_as_double((long long)mx), &ex);  // mx = m 2^ex, m in [0.5, 1)
      e = (m == 0.5) ? ex - 1 : ex;                                       // mx <= 2^e
    }
    const size_t rowg = (size_t)b * S + row;
    if (lane == 0) ge[rowg] = e;
#pragma unroll
    for (int k = 0; k < kKP / 32; ++k) {
      const int p = lane + 32 * k;
      long long v = (long long)rint(ldexp(x[k], 8 * kSlices - e));
      int q[kSlices];
#pragma unroll
      for (int t = 0; t < kSlices; ++t) {
        const int sh = 8 * (kSlices - 1 - t);
        long long d = sh > 0 ? ((v + (1ll << (sh - 1))) >> sh) : v;
        d = d > 255 ? 255 : (d < -255 ? -255 : d);
        q[t] = (int)d;
        v -= d << sh;
      }
#pragma unroll
      for (int t = 0; t < kSlices; ++t) {
        const __nv_bfloat16 h = __int2bfloat16_rn(q[t]);
        gq[((size_t)t * W * S + rowg) * kKP + p] = *reinterpret_cast<const uint16_t*>(&h);
      }
    }
  }
}

// ------------------------------------------------------------------ exact exchange / trace kernel
// One CTA = one tile of gb Cholesky vectors (128 rows (g, i)) against a range of
// walker tiles (WB walkers x S rows).  The four rot_chol slices of the tile stay
// in shared memory; the Green's-function slices stream through two buffers.
// Products q_t (rot) x q_u (green) with t + u = d accumulate exactly in TMEM
// accumulator d (d = 0..4, 96 columns each).  The epilogue rebuilds
// f_g[i][j] = 2^(eA + eB - 16) sum_d 2^(-8 d) A_d as float-float and forms, per
// walker, sum_g sum_ij f_gij f_gji (exchange, trot/meas/rhf.py:33-60) and
// c_g = sum_i f_gii (Coulomb / force bias, trot/meas/rhf.py:119-125).
struct ExArgs {
  SpinLayout L;
  int G, W, mult, wb_per_cta;
  const uint16_t* rot_q;
  const int32_t* rot_e;
  const uint16_t* green_q;
  const int32_t* green_e;
  double2* cs;
  double2* xpart;
  int nblk_total;
  int* status;
};

static constexpr size_t kExSmemA = (size_t)kSlices * 128 * kKP * 2;   // 163840
static constexpr size_t kExSmemB = (size_t)2 * kBN * kKP * 2;         // 49152
static constexpr size_t kExSmemF = (size_t)128 * 32 * sizeof(ff);     // 32768, aliases the B buffers
static_assert(kExSmemF <= kExSmemB, "epilogue buffer must fit in the idle B buffers");
static constexpr size_t kExSmem = kExSmemA + kExSmemB + 128 * 4 + kBN * 4 + 128 * 2 * sizeof(ff) +
                                  8 * 2 * sizeof(ff) + 3 * 8 + 16 + 128;

TROT_D uint32_t off128(int r, int k) {  // core-matrix layout for a [rows x 128] K-major tile
  return (uint32_t)((r >> 3) * 2048 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v) {
  uint32_t r0, r1, r2, r3;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
  v[0] = __uint_as_float(r0); v[1] = __uint_as_float(r1); v[2] = __uint_as_float(r2); v[3] = __uint_as_float(r3);
}

__global__ void __launch_bounds__(128, 1) exchange_exact_kernel(ExArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  unsigned char* sA = base;
  unsigned char* sB = sA + kExSmemA;
  ff* sF = reinterpret_cast<ff*>(sB);  // [128][32]; used only after every MMA of the tile completed
  int* eA = reinterpret_cast<int*>(sB + kExSmemB);
  int* eB = eA + 128;
  ff* sC = reinterpret_cast<ff*>(eB + kBN);      // [128][2] traces (re, im)
  ff* sRed = sC + 128 * 2;                       // [4 warps][2]
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sRed + 16);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 3);

  const SpinLayout& L = a.L;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int blk = blockIdx.x;
  const int wb0 = blockIdx.y * a.wb_per_cta, wb1 = min(L.nwb, wb0 + a.wb_per_cta);
  if (wb0 >= wb1) return;

  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
  }
  // resident A: four rot_chol slices of this tile
  for (int c = tid; c < kSlices * 128 * (kKP / 8); c += 128) {
    const int t = c / (128 * (kKP / 8)), rem = c % (128 * (kKP / 8)), r = rem / (kKP / 8), g = rem % (kKP / 8);
    const uint4 v = *reinterpret_cast<const uint4*>(a.rot_q + (((size_t)t * L.nblk + blk) * 128 + r) * kKP + g * 8);
    *reinterpret_cast<uint4*>(sA + (size_t)t * 128 * kKP * 2 + off128(r, g * 8)) = v;
  }
  eA[tid] = a.rot_e[(size_t)blk * 128 + tid];
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t idesc = tc::idesc_bf16_f32(128, kBN);
  const uint32_t sA_u = tc::smem_u32(sA), sB_u = tc::smem_u32(sB);
  uint32_t phase[2] = {0u, 0u};
  bool ok = true;
  const size_t slice_stride = (size_t)a.W * L.S;  // rows per slice of the green operand
  const int rows_valid_tile = min(L.gb, a.G - blk * L.gb) * L.n;

  for (int wb = wb0; wb < wb1 && ok; ++wb) {
    const int row0 = wb * L.WB * L.S;
    const int nrows = min(L.WB * L.S, a.W * L.S - row0);
    for (int u = 0; u < kSlices && ok; ++u) {
      const int buf = u & 1;
      if (u >= kGroups) break;
      if (u >= 2) {
        ok = tc::mbar_wait(&mbar[buf], phase[buf]);
        phase[buf] ^= 1u;
        if (!ok) break;
      }
      unsigned char* dstB = sB + (size_t)buf * kBN * kKP * 2;
      for (int c = tid; c < kBN * (kKP / 8); c += 128) {
        const int r = c / (kKP / 8), g = c % (kKP / 8);
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < nrows) v = *reinterpret_cast<const uint4*>(a.green_q + ((size_t)u * slice_stride + row0 + r) * kKP + g * 8);
        *reinterpret_cast<uint4*>(dstB + off128(r, g * 8)) = v;
      }
      if (u == 0 && tid < kBN) eB[tid] = tid < nrows ? a.green_e[row0 + tid] : 0;
      tc::fence_proxy_async();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (tid == 0) {
        const int tmax = min(kSlices - 1, (kGroups - 1) - u);
        for (int t = 0; t <= tmax; ++t) {
          const int d = t + u;
          const int first_u = d > kSlices - 1 ? d - (kSlices - 1) : 0;  // first slice u that feeds group d
#pragma unroll
          for (int ks = 0; ks < kKP / 16; ++ks) {
            const uint64_t ad = tc::smem_desc(sA_u + (uint32_t)(t * 128 * kKP * 2 + ks * 256), 128, kKP * 16);
            const uint64_t bd = tc::smem_desc(sB_u + (uint32_t)(buf * kBN * kKP * 2 + ks * 256), 128, kKP * 16);
            tc::mma_bf16(taddr + (uint32_t)(d * kBN), ad, bd, idesc, (u == first_u && ks == 0) ? 0u : 1u);
          }
        }
        tc::mma_commit(&mbar[buf]);
      }
    }
    if (!ok) break;
    // all MMAs of this walker tile: the last commit on each buffer
    for (int bb = 0; bb < 2 && ok; ++bb) {
      ok = tc::mbar_wait(&mbar[bb], phase[bb]);
      phase[bb] ^= 1u;
    }
    if (!ok) break;
    tc::fence_after_sync();

    // ---------------- epilogue: one walker of the tile at a time
    const int r = tid;
    const bool rvalid = r < rows_valid_tile;
    const int i = r % L.n, gl = r / L.n;
    const uint32_t tlane = taddr + ((uint32_t)(warp * 32) << 16);
    for (int bl = 0; bl < L.WB; ++bl) {
      const int b = wb * L.WB + bl;
      if (b >= a.W) break;
      for (int c4 = 0; c4 < L.S / 4; ++c4) {
        float v[kGroups][4];
#pragma unroll
        for (int d = 0; d < kGroups; ++d) tmem_ld4(tlane + (uint32_t)(d * kBN + bl * L.S + c4 * 4), v[d]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int col = c4 * 4 + q;
          ff x = ff_two_sum(v[0][q], v[1][q] * 0.00390625f);
          float lo = x.lo + v[2][q] * 1.52587890625e-05f;
          lo += v[3][q] * 5.9604644775390625e-08f;
          lo += v[4][q] * 2.3283064365386963e-10f;
          x = ff_fast(x.hi, lo);
          const int e = eA[r] + eB[bl * L.S + col] - 16;
          sF[r * 32 + col] = ff{ldexpf(x.hi, e), ldexpf(x.lo, e)};
        }
      }
      __syncthreads();
      ff xr{0.f, 0.f}, xi{0.f, 0.f};
      if (rvalid) {
        const int base_row = gl * L.n;
        for (int j = 0; j < L.n; ++j) {
          const ff ar = sF[r * 32 + j], ai = sF[r * 32 + L.n_pad + j];
          const ff br = sF[(base_row + j) * 32 + i], bi = sF[(base_row + j) * 32 + L.n_pad + i];
          xr = ff_add(xr, ff_sub(ff_mul(ar, br), ff_mul(ai, bi)));
          xi = ff_add(xi, ff_add(ff_mul(ar, bi), ff_mul(ai, br)));
        }
        sC[2 * r] = sF[r * 32 + i];
        sC[2 * r + 1] = sF[r * 32 + L.n_pad + i];
      }
      // exchange: sum over the tile's rows
      for (int o = 16; o > 0; o >>= 1) {
        xr = ff_add(xr, ff_shfl_xor(xr, o));
        xi = ff_add(xi, ff_shfl_xor(xi, o));
      }
      if (lane == 0) {
        sRed[2 * warp] = xr;
        sRed[2 * warp + 1] = xi;
      }
      __syncthreads();
      if (tid == 0) {
        ff tr = sRed[0], ti = sRed[1];
        for (int w = 1; w < 4; ++w) {
          tr = ff_add(tr, sRed[2 * w]);
          ti = ff_add(ti, sRed[2 * w + 1]);
        }
        a.xpart[(size_t)b * a.nblk_total + L.blk_off + blk] =
            make_double2((double)a.mult * ff_d(tr), (double)a.mult * ff_d(ti));
      }
      // traces: c_g = sum_i f_gii for each Cholesky vector of the tile
      if (tid < L.gb) {
        const int g = blk * L.gb + tid;
        if (g < a.G) {
          ff tr{0.f, 0.f}, ti{0.f, 0.f};
          for (int ii = 0; ii < L.n; ++ii) {
            tr = ff_add(tr, sC[2 * (tid * L.n + ii)]);
            ti = ff_add(ti, sC[2 * (tid * L.n + ii) + 1]);
          }
          a.cs[(size_t)b * a.G + g] = make_double2(ff_d(tr), ff_d(ti));
        }
      }
      __syncthreads();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }
  if (!ok && tid == 0) atomicExch(a.status, (int)TROT_ERR_DEVICE_TIMEOUT);
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 512);
}

// fb = sum_s mult_s c_s   (complex, W x G)
__global__ void fb_combine_kernel(int n, int nspin, int m0, int m1, const double2* __restrict__ c0,
                                  const double2* __restrict__ c1, double2* __restrict__ fb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double2 v = cscale(c0[k], (double)m0);
  if (nspin == 2) v = cadd(v, cscale(c1[k], (double)m1));
  fb[k] = v;
}

// ------------------------------------------------------------------ VHS
// Shifted fields as a 3-term bf16 split, rows (walker, re/im), K = G padded.
__global__ void x_slices_kernel(int W, int G, int gpad, int mpad, const double2* __restrict__ xs,
                                uint16_t* __restrict__ xq) {
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
    xq[e] = *reinterpret_cast<const uint16_t*>(&h);
    xq[total + e] = *reinterpret_cast<const uint16_t*>(&m);
    xq[2 * total + e] = *reinterpret_cast<const uint16_t*>(&l);
  }
}

// D (mpad x n2pad, f32) = sum_{t + u <= 2} X_t (mpad x gpad) . Lt_u (n2pad x gpad)^T
// 128 x 128 tile per CTA, K in chunks of 64, operand chunks double-buffered.
static constexpr int kVK = 64;
static constexpr size_t kVhsStage = (size_t)3 * 128 * kVK * 2 * 2;  // X and L slices: 96 KB
static constexpr size_t kVhsSmem = 2 * kVhsStage + 64 + 1024;

__global__ void __launch_bounds__(128, 1)
vhs_gemm_kernel(int mpad, int n2pad, int gpad, const uint16_t* __restrict__ xq, const uint16_t* __restrict__ lq,
                float* __restrict__ D, int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(base + 2 * kVhsStage);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n0 = blockIdx.x * 128, m0 = blockIdx.y * 128;
  if (warp == 0) tc::tmem_alloc(tslot, 128);
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t taddr = *tslot;
  const uint32_t idesc = tc::idesc_bf16_f32(128, 128);
  const size_t xs_stride = (size_t)mpad * gpad, ls_stride = (size_t)n2pad * gpad;
  const int nk = gpad / kVK;
  uint32_t phase[2] = {0u, 0u};
  int pending[2] = {0, 0};
  bool ok = true;
  for (int kt = 0; kt < nk && ok; ++kt) {
    const int buf = kt & 1;
    if (pending[buf]) {
      ok = tc::mbar_wait(&mbar[buf], phase[buf]);
      phase[buf] ^= 1u;
      pending[buf] = 0;
      if (!ok) break;
    }
    unsigned char* st = base + (size_t)buf * kVhsStage;
    const int k0 = kt * kVK;
    // 3 X slices then 3 L slices, each 128 rows x 64 k
    for (int c = tid; c < 6 * 128 * 8; c += 128) {
      const int which = c / (128 * 8), rem = c % (128 * 8), r = rem >> 3, g = rem & 7;
      const uint16_t* src = which < 3 ? xq + which * xs_stride + (size_t)(m0 + r) * gpad
                                      : lq + (which - 3) * ls_stride + (size_t)(n0 + r) * gpad;
      *reinterpret_cast<uint4*>(st + (size_t)which * 128 * kVK * 2 + tc::tile_off(r, g * 8)) =
          *reinterpret_cast<const uint4*>(src + k0 + g * 8);
    }
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0) {
      const uint32_t su = tc::smem_u32(st);
      bool first = kt == 0;
      for (int t = 0; t < 3; ++t)
        for (int u = 0; t + u <= 2; ++u) {
#pragma unroll
          for (int ks = 0; ks < kVK / 16; ++ks) {
            const uint64_t ad = tc::smem_desc(su + (uint32_t)(t * 128 * kVK * 2 + ks * 256), 128, 1024);
            const uint64_t bd = tc::smem_desc(su + (uint32_t)((3 + u) * 128 * kVK * 2 + ks * 256), 128, 1024);
            tc::mma_bf16(taddr, ad, bd, idesc, first ? 0u : 1u);
            first = false;
          }
        }
      tc::mma_commit(&mbar[buf]);
    }
    pending[buf] = 1;
  }
  for (int bb = 0; bb < 2 && ok; ++bb)
    if (pending[bb]) {
      ok = tc::mbar_wait(&mbar[bb], phase[bb]);
      phase[bb] ^= 1u;
    }
  if (ok) {
    tc::fence_after_sync();
    const uint32_t trow = taddr + ((uint32_t)(warp * 32) << 16);
    float v[16];
    for (int c = 0; c < 8; ++c) {
      tc::tmem_ld16(trow + c * 16, v);
      float4* d = reinterpret_cast<float4*>(D + (size_t)(m0 + warp * 32 + lane) * n2pad + n0 + c * 16);
      d[0] = make_float4(v[0], v[1], v[2], v[3]);
      d[1] = make_float4(v[4], v[5], v[6], v[7]);
      d[2] = make_float4(v[8], v[9], v[10], v[11]);
      d[3] = make_float4(v[12], v[13], v[14], v[15]);
    }
  } else if (tid == 0) {
    atomicExch(status, (int)TROT_ERR_DEVICE_TIMEOUT);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(taddr, 128);
}

// ------------------------------------------------------------------ FP32 Trotter propagation
// Same algorithm as the FP64 trotter_kernel with float2 arithmetic: the walker's
// VHS (complex N x N, from rows (2b, 2b+1) of D) is staged in shared memory.
__device__ void real_mm32(int N, int nc, const float* __restrict__ E, const float2* in, float2* out) {
  for (int e = threadIdx.x; e < N * nc; e += blockDim.x) {
    const int p = e / nc, j = e % nc;
    const float* Er = E + (size_t)p * N;
    float2 acc = make_float2(0.f, 0.f);
    for (int q = 0; q < N; ++q) {
      const float w = Er[q];
      const float2 x = in[q * nc + j];
      acc.x = fmaf(w, x.x, acc.x);
      acc.y = fmaf(w, x.y, acc.y);
    }
    out[e] = acc;
  }
}

struct Trot32Args {
  TrotterArgs t;
  const float* vhs;
  int n2pad;
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
  for (int e = tid; e < N * N; e += nt) V[e] = make_float2(vre[e], vim[e]);
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
    const float c = (float)(a.sqrt_dt / (double)k);
    for (int e = tid; e < N * nc; e += nt) {
      const int p = e / nc, j = e % nc;
      const float2* Vr = V + (size_t)p * N;
      float2 acc = make_float2(0.f, 0.f);
      for (int q = 0; q < N; ++q) {
        const float2 v = Vr[q], x = T[q * nc + j];
        acc.x = fmaf(v.x, x.x, acc.x);
        acc.x = fmaf(-v.y, x.y, acc.x);
        acc.y = fmaf(v.x, x.y, acc.y);
        acc.y = fmaf(v.y, x.x, acc.y);
      }
      const float2 t = make_float2(-c * acc.y, c * acc.x);
      T2[e] = t;
      O[e] = make_float2(O[e].x + t.x, O[e].y + t.y);
    }
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

// ------------------------------------------------------------------ host orchestration
static int check_mixed_shapes(const trot_system* s, const Spins& sp) {
  if (!s->mixed) { set_error("mixed precision needs a trot_mixed context"); return TROT_ERR_NULL_PTR; }
  if (s->norb > kKP) { set_error("mixed path: norb %d > %d", s->norb, kKP); return TROT_ERR_UNSUPPORTED; }
  for (int q = 0; q < sp.nspin; ++q)
    if (2 * (sp.n[q] + (sp.n[q] & 1)) > 32) { set_error("mixed path: nocc %d > 16", sp.n[q]); return TROT_ERR_UNSUPPORTED; }
  if (s->mixed->kpad != kKP || s->mixed->slices != kSlices || s->mixed->max_order != kGroups - 1) {
    set_error("mixed context layout mismatch");
    return TROT_ERR_BAD_SHAPE;
  }
  return TROT_OK;
}

static int run_slices_and_exchange(const trot_system* s, const Spins& sp, MixedBuffers& m, cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  for (int q = 0; q < sp.nspin; ++q) {
    SpinLayout L = spin_layout(s, sp, q);
    TROT_TIMED("green_slices", st, ([&]() -> int {
      green_slices_kernel<<<W, 256, 0, st>>>(N, L.n, L.n_pad, W, sp.ntot, sp.off[q], m.green, m.gq[q], m.ge[q]);
      TROT_CHECK_LAUNCH("green_slices_kernel");
      return TROT_OK;
    })());
  }
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(exchange_exact_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kExSmem + 1024);
    attr_set = true;
  }
  for (int q = 0; q < sp.nspin; ++q) {
    SpinLayout L = spin_layout(s, sp, q);
    const int mq = (s->kind == TROT_UHF_U) ? q : 0;
    ExArgs a{};
    a.L = L;
    a.G = G; a.W = W; a.mult = sp.mult[q];
    // walker tiles per CTA: enough CTAs to fill the GPU a few times over
    const int target = 152 * 4;
    int chunks = (target + L.nblk - 1) / L.nblk;
    if (chunks > L.nwb) chunks = L.nwb;
    a.wb_per_cta = (L.nwb + chunks - 1) / chunks;
    chunks = (L.nwb + a.wb_per_cta - 1) / a.wb_per_cta;
    a.rot_q = s->mixed->rot_slices[mq];
    a.rot_e = s->mixed->rot_exp[mq];
    a.green_q = m.gq[q];
    a.green_e = m.ge[q];
    a.cs = m.cs[q];
    a.xpart = m.xpart;
    a.nblk_total = m.nblk_total;
    a.status = m.status;
    dim3 grid(L.nblk, chunks);
    TROT_TIMED("exchange_exact_tc", st, ([&]() -> int {
      exchange_exact_kernel<<<grid, 128, kExSmem + 1024, st>>>(a);
      TROT_CHECK_LAUNCH("exchange_exact_kernel");
      return TROT_OK;
    })());
  }
  const int n = W * G;
  fb_combine_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, sp.nspin, sp.mult[0], sp.mult[1], m.cs[0],
                                                     sp.nspin == 2 ? m.cs[1] : nullptr, m.fb);
  TROT_CHECK_LAUNCH("fb_combine_kernel");
  return TROT_OK;
}

static int run_vhs(const trot_system* s, MixedBuffers& m, const double2* xs, cudaStream_t st) {
  const int W = s->n_walkers, G = s->nchol;
  const trot_mixed* mx = s->mixed;
  TROT_TIMED("x_slices", st, ([&]() -> int {
    x_slices_kernel<<<152 * 8, 256, 0, st>>>(W, G, mx->gpad, m.mpad, xs, m.xq);
    TROT_CHECK_LAUNCH("x_slices_kernel");
    return TROT_OK;
  })());
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(vhs_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVhsSmem);
    attr_set = true;
  }
  dim3 grid(mx->n2pad / 128, m.mpad / 128);
  TROT_TIMED("vhs_tc", st, ([&]() -> int {
    vhs_gemm_kernel<<<grid, 128, kVhsSmem, st>>>(m.mpad, mx->n2pad, mx->gpad, m.xq, mx->chol_t_slices, m.vhs,
                                                m.status);
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
  a.expH32 = s->mixed->exp_h1_half_f32;
  trotter32_kernel<<<s->n_walkers, 256, smem, st>>>(sp, a);
  TROT_CHECK_LAUNCH("trotter32_kernel");
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
  cudaMemsetAsync(m.status, 0, 4 * sizeof(int), st);
  return TROT_OK;
}

int mixed_force_bias(const trot_system* s, const Spins& sp, const double2* wa, const double2* wb, double2* fb_out,
                     void* ws, size_t ws_bytes, cudaStream_t st) {
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  TROT_TRY(begin(s, sp, c, m, TROT_OP_FORCE_BIAS, st));
  TROT_TRY(launch_green(sp, s->n_walkers, s->norb, wa, wb, m.green, nullptr, nullptr, st));
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
  TROT_TRY(launch_green(sp, s->n_walkers, s->norb, wa, wb, m.green, nullptr, m.e1, st));
  TROT_TRY(run_slices_and_exchange(s, sp, m, st));
  return launch_energy_combine(s->n_walkers, s->nchol, m.nblk_total, s->h0, m.fb, m.e1, m.xpart, energy, st);
}

int mixed_apply_trotter(const trot_system* s, const Spins& sp, const double2* xs, const TrotterArgs& a, void* ws,
                        size_t ws_bytes, cudaStream_t st) {
  if (!s->mixed) { set_error("mixed precision needs a trot_mixed context"); return TROT_ERR_NULL_PTR; }
  if (s->norb > kKP) { set_error("mixed path: norb %d > %d", s->norb, kKP); return TROT_ERR_UNSUPPORTED; }
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  carve_mixed(s, sp, c, m, TROT_OP_APPLY_TROTTER);
  if (!c.ok) { set_error("workspace too small: %zu < %zu", ws_bytes, c.used); return TROT_ERR_WORKSPACE_TOO_SMALL; }
  cudaMemsetAsync(m.status, 0, 4 * sizeof(int), st);
  TROT_TRY(run_vhs(s, m, xs, st));
  return run_trotter32(s, sp, a, m, st);
}

int mixed_prop_step(const trot_system* s, const Spins& sp, const trot_state* state, const double* fields,
                    double2* energy_out, void* ws, size_t ws_bytes, cudaStream_t st) {
  const int W = s->n_walkers, N = s->norb, G = s->nchol;
  Carver c(ws, ws_bytes);
  MixedBuffers m;
  TROT_TRY(begin(s, sp, c, m, TROT_OP_PROP_STEP, st));
  double2* wa = (double2*)state->walkers_a;
  double2* wb = (double2*)state->walkers_b;
  TROT_TIMED("green", st, launch_green(sp, W, N, wa, wb, m.green, nullptr, energy_out ? m.e1 : nullptr, st));
  TROT_TRY(run_slices_and_exchange(s, sp, m, st));
  if (energy_out)
    TROT_TIMED("energy_combine", st,
               launch_energy_combine(W, G, m.nblk_total, s->h0, m.fb, m.e1, m.xpart, energy_out, st));
  TROT_TIMED("fields", st, launch_fields(W, G, s->sqrt_dt, m.fb, s->mf_shifts_im, fields, m.xs, m.shift_term,
                                         m.fb_term, st));
  TROT_TRY(run_vhs(s, m, m.xs, st));
  TrotterArgs a{};
  a.W = W; a.N = N; a.G = G; a.nterms = s->n_exp_terms; a.sqrt_dt = s->sqrt_dt; a.expH = s->exp_h1_half;
  a.in_a = wa; a.in_b = wb; a.out_a = wa; a.out_b = wb;
  a.overlaps = (double2*)state->overlaps; a.weights = state->weights; a.scalars = state->scalars;
  a.shift_term = m.shift_term; a.fb_term = m.fb_term; a.node_flag = m.node_flag;
  a.dt = s->dt; a.h0_prop = s->h0_prop; a.w_floor = s->weight_floor; a.w_cap = s->weight_cap;
  TROT_TIMED("trotter_fp32", st, run_trotter32(s, sp, a, m, st));
  TROT_TIMED("step_finalize", st, launch_step_finalize(W, state->weights, state->scalars,
                                                       (long long*)state->node_encounters, m.node_flag,
                                                       s->pop_control_damping, s->dt, st));
  return TROT_OK;
}

}  // namespace trot
