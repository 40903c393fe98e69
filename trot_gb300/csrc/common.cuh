// Shared device helpers for the trot_gb300 kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include "trot_gb300.h"

#define TROT_HD __host__ __device__ __forceinline__
#define TROT_D __device__ __forceinline__

// ---------------------------------------------------------------- device status words
// A mixed-precision workspace starts with int[4] status words: [0] the status of
// the current call (reset when the call begins), [3] a sticky copy that only
// trot_workspace_timeouts clears.  A tensor-core kernel whose bounded wait ran out
// records TROT_ERR_DEVICE_TIMEOUT in both, skips its outputs and returns; the
// kernels that combine its results then write NaN instead of numbers.
TROT_D void report_timeout(int* status) {
  atomicExch(status, (int)TROT_ERR_DEVICE_TIMEOUT);
  atomicExch(status + 3, (int)TROT_ERR_DEVICE_TIMEOUT);
}

// ---------------------------------------------------------------- complex (double2)
TROT_HD double2 cmk(double r, double i) { return make_double2(r, i); }
TROT_HD double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
TROT_HD double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
TROT_HD double2 cmul(double2 a, double2 b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
TROT_HD double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
// a += b * c (complex)
TROT_HD void cfma(double2& a, double2 b, double2 c) {
  a.x = fma(b.x, c.x, a.x);
  a.x = fma(-b.y, c.y, a.x);
  a.y = fma(b.x, c.y, a.y);
  a.y = fma(b.y, c.x, a.y);
}
// a += s * c (real times complex)
TROT_HD void crfma(double2& a, double s, double2 c) {
  a.x = fma(s, c.x, a.x);
  a.y = fma(s, c.y, a.y);
}
TROT_HD double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }
// complex division a / b, scaled to avoid overflow (Smith's method)
TROT_HD double2 cdiv(double2 a, double2 b) {
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  } else {
    double r = b.x / b.y, d = b.y + b.x * r;
    return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
  }
}
TROT_HD double2 cexp(double2 a) {
  double s, c;
  sincos(a.y, &s, &c);
  double e = exp(a.x);
  return cmk(e * c, e * s);
}

// ---------------------------------------------------------------- reductions
TROT_D double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
TROT_D double2 warp_sum2(double2 v) { return cmk(warp_sum(v.x), warp_sum(v.y)); }

// Block-wide sum in a fixed order (deterministic).  `red` holds >= 32 double2.
TROT_D double2 block_sum2(double2 v, double2* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum2(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double2 t = cmk(0.0, 0.0);
  if (wid == 0) {
    t = lane < nw ? red[lane] : cmk(0.0, 0.0);
    t = warp_sum2(t);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  t = red[0];
  __syncthreads();
  return t;
}

// ---------------------------------------------------------------- spin layout
// Per-system spin description used by every kernel: up to two spins; a
// restricted walker has one spin with multiplicity 2.
struct Spins {
  int nspin;        // 1 (restricted) or 2
  int n[2];         // columns per spin
  int mult[2];      // 2 for restricted, 1 otherwise
  int off[2];       // offset of spin s in the concatenated (n_a + n_b) column space
  int ntot;         // n[0] + n[1] (concatenated columns)
  const double* mo[2];
  const double* rot_h1[2];
  const double* rot_chol[2];
};

// Small-matrix LU with partial pivoting on an n x n complex matrix in shared
// memory (row-major, leading dimension ld), executed by the whole block.
// Returns det(A) to all threads; A is overwritten by its LU factors.
// If `inv` is non-null it receives A^{-1} (Gauss-Jordan on [A | I]).
// One warp, an n x n matrix A (row stride n) in shared memory, partial pivoting (the first
// largest |A[i][k]| wins, as in block_gauss_jordan).  Returns det(A).  With `inverse`, A is
// overwritten by its inverse (in-place Gauss-Jordan: each pivot step updates the n x n working
// array once, half the work of eliminating [A | I]; the row interchanges are undone as column
// interchanges in reverse order at the end, `perm` holds n ints of scratch); without it, A
// holds its LU factors.  Phases are separated by __syncwarp, so no CTA barrier is involved.
// The determinant is returned in lane 0.
TROT_D double2 warp_gauss_jordan(double2* A, int n, bool inverse, int* perm) {
  const int lane = threadIdx.x & 31;
  double2 det = cmk(1.0, 0.0);
  for (int k = 0; k < n; ++k) {
    double best = -1.0;
    int bi = k;
    for (int i = k + lane; i < n; i += 32) {
      const double a = cabs2(A[i * n + k]);
      if (a > best) { best = a; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (bi != k) {
      for (int j = lane; j < n; j += 32) {
        const double2 t = A[k * n + j];
        A[k * n + j] = A[bi * n + j];
        A[bi * n + j] = t;
      }
      det = cmk(-det.x, -det.y);
    }
    if (inverse && lane == 0) perm[k] = bi;
    __syncwarp();
    // the pivot's reciprocal and the running determinant by lane 0 only (the FP64 pipe is
    // narrow: an FP64 division issued by the whole warp costs as much as an elimination step)
    double2 rp = cmk(0.0, 0.0);
    if (lane == 0) {
      const double2 piv = A[k * n + k];
      det = cmul(det, piv);
      rp = cdiv(cmk(1.0, 0.0), piv);
    }
    rp.x = __shfl_sync(0xffffffffu, rp.x, 0);
    rp.y = __shfl_sync(0xffffffffu, rp.y, 0);
    if (inverse) {
      __syncwarp();
      for (int j = lane; j < n; j += 32) A[k * n + j] = j == k ? rp : cmul(A[k * n + j], rp);
      __syncwarp();
      // A[i][j] -= A[i][k] A[k][j] for i != k, j != k (the (n-1)^2 elements, row / column k
      // skipped by the index map); then column k: A[i][k] = -A[i][k] rp
      const int m = n - 1;
      for (int e = lane; e < m * m; e += 32) {
        int i = e / m, j = e - (e / m) * m;
        i += i >= k;
        j += j >= k;
        A[i * n + j] = csub(A[i * n + j], cmul(A[i * n + k], A[k * n + j]));
      }
      __syncwarp();
      for (int i = lane; i < n; i += 32)
        if (i != k) A[i * n + k] = cmul(cmk(-A[i * n + k].x, -A[i * n + k].y), rp);
    } else {
      for (int i = k + 1 + lane; i < n; i += 32) A[i * n + k] = cmul(A[i * n + k], rp);
      __syncwarp();
      const int m = n - k - 1;
      for (int e = lane; e < m * m; e += 32) {
        const int i = k + 1 + e / m, j = k + 1 + (e - (e / m) * m);
        A[i * n + j] = csub(A[i * n + j], cmul(A[i * n + k], A[k * n + j]));
      }
    }
    __syncwarp();
  }
  if (inverse) {
    for (int k = n - 1; k >= 0; --k) {
      const int p = perm[k];
      if (p != k)
        for (int i = lane; i < n; i += 32) {
          const double2 t = A[i * n + k];
          A[i * n + k] = A[i * n + p];
          A[i * n + p] = t;
        }
      __syncwarp();
    }
  }
  return det;
}

TROT_D double2 block_gauss_jordan(double2* A, int n, int ld, double2* inv, int* piv_s, double2* red) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (inv) {
    for (int e = tid; e < n * n; e += nt) {
      int i = e / n, j = e % n;
      inv[i * ld + j] = cmk(i == j ? 1.0 : 0.0, 0.0);
    }
  }
  __shared__ double2 det_s, rp_s;  // running determinant; reciprocal of the current pivot
  if (tid == 0) det_s = cmk(1.0, 0.0);
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    // pivot search: warp 0 finds argmax |A[i][k]|, i >= k (first max wins)
    if (tid < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + tid; i < n; i += 32) {
        double a = cabs2(A[i * ld + k]);
        if (a > best) { best = a; bi = i; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) *piv_s = bi;
    }
    __syncthreads();
    const int p = *piv_s;
    if (p != k) {
      for (int j = tid; j < n; j += nt) {
        double2 t = A[k * ld + j]; A[k * ld + j] = A[p * ld + j]; A[p * ld + j] = t;
        if (inv) { t = inv[k * ld + j]; inv[k * ld + j] = inv[p * ld + j]; inv[p * ld + j] = t; }
      }
    }
    __syncthreads();
    const double2 piv = A[k * ld + k];
    if (tid == 0) {
      det_s = cmul(p != k ? cmk(-det_s.x, -det_s.y) : det_s, piv);
      rp_s = cdiv(cmk(1.0, 0.0), piv);  // one division per pivot, shared by all threads
    }
    __syncthreads();
    const double2 rp = rp_s;
    if (inv) {
      // Gauss-Jordan: normalise row k, eliminate column k from every other row
      for (int j = tid; j < n; j += nt) {
        A[k * ld + j] = cmul(A[k * ld + j], rp);
        inv[k * ld + j] = cmul(inv[k * ld + j], rp);
      }
      __syncthreads();
      for (int e = tid; e < n * n; e += nt) {
        int i = e / n, j = e % n;
        if (i == k) continue;
        double2 f = A[i * ld + k];
        // column k of A itself is updated last (j == k) by the thread that owns it
        if (j != k) A[i * ld + j] = csub(A[i * ld + j], cmul(f, A[k * ld + j]));
        inv[i * ld + j] = csub(inv[i * ld + j], cmul(f, inv[k * ld + j]));
      }
      __syncthreads();
      for (int i = tid; i < n; i += nt)
        if (i != k) A[i * ld + k] = cmk(0.0, 0.0);
      __syncthreads();
    } else {
      // plain LU elimination below the pivot: multipliers once per row (stored in column k)
      for (int i = k + 1 + tid; i < n; i += nt) A[i * ld + k] = cmul(A[i * ld + k], rp);
      __syncthreads();
      const int m = n - k - 1;
      for (int e = tid; e < m * m; e += nt) {
        const int i = k + 1 + e / m, j = k + 1 + e % m;
        A[i * ld + j] = csub(A[i * ld + j], cmul(A[i * ld + k], A[k * ld + j]));
      }
      __syncthreads();
    }
  }
  __syncthreads();
  double2 d = det_s;
  __syncthreads();
  (void)red;
  return d;
}

// ---------------------------------------------------------------- errors
namespace trot {
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);
void prof_count_launch();  // profile.cu: counts launches while the timers are enabled
}  // namespace trot

#define TROT_CHECK_LAUNCH(where)                                      \
  do {                                                                \
    trot::prof_count_launch();                                        \
    cudaError_t _e = cudaGetLastError();                              \
    if (_e != cudaSuccess) return trot::cuda_status(_e, where);       \
  } while (0)
