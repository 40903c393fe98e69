// Host-side launchers shared between the kernel translation units and the C ABI.
#pragma once
#include "common.cuh"

#define TROT_TRY(x) do { int _r = (x); if (_r != TROT_OK) return _r; } while (0)

namespace trot {

// Bump allocator over the caller's workspace (256-byte aligned slices).  Every
// layout begins with a 256-byte status block at offset 0 (int[0]: the current
// call's status, int[3]: the sticky timeout word of report_timeout), so any
// workspace can be shared between ops without one op's buffers overwriting
// another's status words.
struct Carver {
  static constexpr size_t kStatusBytes = 256;
  char* base;
  size_t size, used = kStatusBytes;
  bool ok = true;
  Carver(void* b, size_t s) : base(static_cast<char*>(b)), size(s) {
    if (base && size < kStatusBytes) ok = false;
  }
  int* status() { return (base && size >= kStatusBytes) ? reinterpret_cast<int*>(base) : nullptr; }
  template <class T>
  T* take(size_t count) {
    size_t off = (used + 255) & ~size_t(255);
    used = off + count * sizeof(T);
    if (base == nullptr || used > size) { ok = false; return nullptr; }
    return reinterpret_cast<T*>(base + off);
  }
};

struct StepBuffers {
  double2 *green, *e1, *fb, *xs, *shift_term, *fb_term, *vhs, *exc;
  double2* vp;  // packed upper triangle of the VHS (W, N(N+1)/2) when chol_packed is set
  int* node_flag;
};

Spins make_spins(const trot_system* s);
int tune_get(int knob);  // tune.cu: 0 = default

// Green's function / overlap per walker (green.cu).
// green: complex (W, ntot*N) half Green's functions, spin blocks concatenated
// (may be null); det_out: complex (W) overlap = prod_s det(C_s^T w_s)^mult_s (may be null);
// e1_out: complex (W) sum_s mult_s sum(G_s o rot_h1_s) (may be null).
int launch_green(const Spins& sp, int W, int N, const double2* wa, const double2* wb,
                 double2* green, double2* ovlp_out, double2* e1_out, cudaStream_t st);

// C[m][n] (+)= alpha * sum_k A[m][k] * B(k, n), A complex (lda), C complex (ldc).
// b_is_nk: B stored (N, K) row-major (ldb) — otherwise (K, N) row-major.
int launch_zgemm_cr(int M, int Nn, int K, double alpha, const double2* A, int lda,
                    const double* B, int ldb, bool b_is_nk, double2* C, int ldc, bool accumulate,
                    cudaStream_t st);
// Same with K split into S slices computed by separate CTAs (for small M x Nn and long K):
// part holds S * M * Nn complex partials, reduced in slice order into C.
int launch_zgemm_cr_splitk(int M, int Nn, int K, double alpha, const double2* A, int lda, const double* B, int ldb,
                           bool b_is_nk, double2* C, int ldc, bool accumulate, double2* part, int S,
                           cudaStream_t st);
// FP64 VHS = xs . chol (W x N^2): over the packed upper triangle (then mirrored) when
// chol_packed and vp (W x N(N+1)/2 complex scratch) are given, else the full product.
int launch_vhs64(int W, int N, int G, const double2* xs, const double* chol_flat, const double* chol_packed,
                 double2* vp, double2* vhs, cudaStream_t st);
// Mp = the packed upper triangle of M + M^T (diagonal once), W matrices of N x N.
int launch_pack_sym(int N, int W, const double2* m, double2* mp, cudaStream_t st);

// step64.cu
int launch_fields(int W, int G, double sqrt_dt, const double2* fb, const double* mf_im,
                  const double* x, double2* xs, double2* shift_term, double2* fb_term, cudaStream_t st);

struct TrotterArgs {
  int W, N, G, nterms;
  double sqrt_dt;
  const double* expH;  // (N, N)
  const double2* vhs;  // (W, N, N)
  const double2* in_a; const double2* in_b;
  double2* out_a; double2* out_b;
  // step mode (all null otherwise)
  double2* overlaps;       // in: old, out: new
  double* weights;         // in/out
  const double* scalars;   // [E_shift, e_est]
  const double2* shift_term; const double2* fb_term;
  int* node_flag;
  double dt, h0_prop, w_floor, w_cap;
};
int launch_trotter(const Spins& sp, const TrotterArgs& a, cudaStream_t st);
// status (optional): the mixed-precision status words of the step (int[4], see
// report_timeout); when status[0] is set the step's weights and population shift
// become NaN instead of numbers computed from skipped tensor-core results
int launch_step_finalize(int W, double* weights, double* scalars, long long* nodes,
                         const int* node_flag, double damping, double dt, cudaStream_t st,
                         const int* status = nullptr);

int exchange_chunks(int G);
int launch_exchange(const Spins& sp, int W, int N, int G, const double2* green, double2* partial,
                    cudaStream_t st);
// Fixed-point partial sum of the tensor-core exchange kernel: value v[c] 2^-s[c] (c = re, im);
// s[c] = kExchangeNonFinite marks a non-finite contribution (the energy becomes NaN).
struct ExFixed {
  long long v[2];
  int s[2];
};
static constexpr int kExchangeNonFinite = -0x7fffffff;
// e1: e1_parts consecutive arrays of W values (one per spin for the mixed path), added in order
// status (optional): as for launch_step_finalize; the energies become NaN when status[0] is set
// partial: nchunks double2 per walker, or (xfixed != null) nchunks ExFixed per walker instead
int launch_energy_combine(int W, int G, int nchunks, double h0, const double2* fb, const double2* e1, int e1_parts,
                          const double2* partial, double2* energy, cudaStream_t st, const int* status = nullptr,
                          const ExFixed* xfixed = nullptr);
// dst[0] = dst[3] = src[0] when src[0] is set (status words of two workspace regions, see report_timeout)
int launch_status_merge(const int* src, int* dst, cudaStream_t st);

// walkers.cu
// write_q = false: only the norms prod_j |R_jj| (free-projection qr_norm); the walkers are left unchanged
int launch_qr(const Spins& sp, int W, int N, double2* wa, double2* wb, double2* norm_out, cudaStream_t st,
              bool write_q = true);
int launch_sr(const Spins& sp, int W, int N, const double* weights, const double* zeta_dev, double zeta,
              const double2* ina,
              const double2* inb, double2* outa, double2* outb, double* weights_out, long long* idx,
              double* cw, cudaStream_t st);

// ctx.cu: out = expm(A) (real n x n, device); status[0] guard, status[1] squarings; p0, p1 n x n scratch
int launch_expm(int n, const double* A, double* out, double* p0, double* p1, int* status, cudaStream_t st);

}  // namespace trot
