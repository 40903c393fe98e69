// Shared tail of the Trotter kernels: overlap of the propagated walker with
// the trial (FP64 LU determinant) and the phaseless importance weight.
#pragma once
#include "kernels.h"

namespace trot {

// Phaseless importance weight of walker b given its new trial overlap
// (trot/prop/afqmc.py:111-130): weights, overlaps and node flag are updated in place.
__device__ __forceinline__ void phaseless_update(const TrotterArgs& a, int b, double2 ov_new) {
  const double2 ov_old = a.overlaps[b];
  const double2 ratio = cdiv(ov_new, ov_old);
  const double2 shift = a.shift_term[b];
  const double2 fbt = a.fb_term[b];
  const double e_shift = a.scalars[0];
  const double2 expo = cadd(cadd(cscale(shift, -a.sqrt_dt), fbt), cmk(a.dt * (e_shift + a.h0_prop), 0.0));
  const double2 imp = cmul(cexp(expo), ratio);
  const double2 ph = cmul(cexp(cscale(shift, -a.sqrt_dt)), ratio);
  const double theta = atan2(ph.y, ph.x);
  double imp_ph = hypot(imp.x, imp.y) * cos(theta);
  if (!isfinite(imp_ph) || imp_ph < a.w_floor) imp_ph = 0.0;
  a.node_flag[b] = imp_ph <= 0.0 ? 1 : 0;
  if (imp_ph > a.w_cap) imp_ph = 0.0;
  double wn = a.weights[b] * imp_ph;
  if (wn > a.w_cap) wn = 0.0;
  a.weights[b] = wn;
  a.overlaps[b] = ov_new;
}

// W2: propagated walker columns (N x nc, FP64, shared memory); Ms: n x n scratch.
__device__ __forceinline__ void overlap_and_weight(const Spins& sp, const TrotterArgs& a, int N, int nc,
                                                   const double2* W2, double2* Ms, int* piv, double2* red) {
  const int b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  // new overlap: prod_s det(C_s^T w'_s)^mult  (trot/trial/rhf.py:45-54, trot/trial/uhf.py:54-58)
  double2 det_all = cmk(1.0, 0.0);
  for (int s = 0; s < sp.nspin; ++s) {
    const int n = sp.n[s];
    const double* C = sp.mo[s];
    __syncthreads();
    for (int e = tid; e < n * n; e += nt) {
      const int i = e / n, j = e % n;
      double2 acc = cmk(0.0, 0.0);
      for (int p = 0; p < N; ++p) crfma(acc, C[p * n + i], W2[p * nc + sp.off[s] + j]);
      Ms[e] = acc;
    }
    __syncthreads();
    double2 det = block_gauss_jordan(Ms, n, n, nullptr, piv, red);
    det_all = cmul(det_all, sp.mult[s] == 2 ? cmul(det, det) : det);
  }
  if (tid == 0) phaseless_update(a, b, det_all);
}

}  // namespace trot
