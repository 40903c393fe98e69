/*
 * trot_gb300 — C ABI of the GB300 (sm_103a) phaseless-AFQMC hot path.
 *
 * Every entry point takes caller-owned device buffers (plain pointers),
 * sizes, and a cudaStream_t passed as void*.  Nothing here allocates device
 * memory: scratch comes from a caller-provided workspace whose size is given
 * by trot_workspace_size().  Calls launch asynchronously on the given stream
 * and never synchronise with the host, so they can be issued inside a CUDA
 * graph capture.  Errors come back as a trot_status code; the message of the
 * last error on the calling thread is in trot_last_error().
 *
 * Array conventions (all row-major, C order, as numpy/jax/torch lay them out):
 *   complex128 arrays are interleaved (re, im) doubles;
 *   walkers            (W, N, n)   complex128   W walkers, N orbitals, n columns
 *   trial coefficients (N, n)      float64
 *   Cholesky vectors   (G, N, N)   float64      (chol_flat = (G, N*N))
 *   rot_chol           (G, n, N)   float64      half-rotated C^T L_g
 *   rot_h1             (n, N)      float64      C^T h1
 *
 * Walker/trial kinds (the reference's make_*_meas_ops(sys) dispatch):
 *   TROT_RHF_R  RHF trial, restricted walkers     trot/meas/rhf.py:119-138
 *   TROT_RHF_U  RHF trial, unrestricted walkers   trot/meas/rhf.py:141-172
 *   TROT_UHF_U  UHF trial, unrestricted walkers   trot/meas/uhf.py:43-57,205-231
 */
#ifndef TROT_GB300_H
#define TROT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TROT_ABI_VERSION 4

typedef enum {
  TROT_OK = 0,
  TROT_ERR_BAD_SHAPE = 1,
  TROT_ERR_BAD_DTYPE = 2,
  TROT_ERR_NULL_PTR = 3,
  TROT_ERR_WORKSPACE_TOO_SMALL = 4,
  TROT_ERR_CUDA = 5,
  TROT_ERR_DEVICE_TIMEOUT = 6,
  TROT_ERR_NUMERIC_GUARD = 7,
  TROT_ERR_UNSUPPORTED = 8
} trot_status;

typedef enum { TROT_RHF_R = 0, TROT_RHF_U = 1, TROT_UHF_U = 2 } trot_kind;

/* Arithmetic of the dense contractions.  TROT_FP64 computes everything in
 * float64.  TROT_MIXED runs the force-bias / VHS / Taylor / exchange
 * contractions on tensor cores and keeps LU, log-det, QR, weights and energy
 * accumulation in float64. */
typedef enum { TROT_FP64 = 0, TROT_MIXED = 1 } trot_precision;

typedef enum {
  TROT_OP_FORCE_BIAS = 0,
  TROT_OP_LOCAL_ENERGY = 1,
  TROT_OP_APPLY_TROTTER = 2,
  TROT_OP_PROP_STEP = 3,
  TROT_OP_QR = 4,
  TROT_OP_SR = 5,
  TROT_OP_OVERLAP = 6,
  TROT_OP_RDM1 = 7
} trot_op;

/* Operands of the mixed-precision path, prepared once per (trial,
 * Hamiltonian, dt) by trot_gb300.mixed (host) and pointed to by
 * trot_system.mixed (this struct lives in host memory; its pointers are
 * device pointers).
 *
 * Local energy / force bias use an exact-digit FP16 product on tensor cores:
 * every row x of rot_chol (rows (g, i) over orbitals p) and of the half
 * Green's function is written as x = 2^e sum_t q_t 2^-(T + 9 t) with integer
 * digits (exact in FP16), one exponent e per row, a leading digit of T bits
 * (T = 9, |q_0| <= 512, for rot_chol; T = 8, |q_0| <= 256, for the Green's
 * function) and balanced 9-bit lower digits |q_t| <= 256; a rot_chol row whose
 * sum of |q_0| exceeds 2^15 has its exponent raised by one.  Digit products
 * with equal t + u share one FP32 accumulator, and the two leading groups
 * (t + u <= 1) stay below 2^24 in magnitude, so they accumulate exactly.  The
 * VHS uses a plain 3-term bf16 split (x = hi + mid + lo) with FP32
 * accumulation. */
typedef struct {
  int slices;            /* digits per operand of the exact product (5) */
  int max_order;         /* products with t + u <= max_order (4) */
  int kpad;              /* padded orbital dimension of the exact product (128) */
  int gammas_per_block[2];   /* Cholesky vectors per 128-row tile, per spin */
  int n_blocks[2];           /* tiles per spin: ceil(G / gammas_per_block) */
  const uint16_t* rot_slices[2]; /* fp16 digits (slices, n_blocks, 128, kpad) per spin */
  const int32_t* rot_exp[2];     /* int32 (n_blocks, 128) row exponents per spin */
  int vhs_slices;        /* 3 */
  int vhs_order;         /* products with t + u <= vhs_order (2) */
  int n2pad;             /* N*N rounded up to 128 */
  int gpad;              /* G rounded up to 64 */
  const uint16_t* chol_t_slices; /* bf16 (vhs_slices, n2pad, gpad): row pq holds L[:, pq] */
  const float* exp_h1_half_f32;  /* (N, N) */
  /* exp(-dt/2 h1_eff), zero-padded to 128 x 128, as 3 BF16 slices in the
   * tensor-core operand image (4 chunks x 3 slices x 128 rows x 32); when set,
   * the Trotter action runs on the tensor cores (N <= 128, nocc_a + nocc_b <=
   * 32), else in FP32. */
  const uint16_t* exp_h1_half_img;
  /* 1 when every Cholesky matrix is symmetric to working precision: the rows of
   * chol_t_slices are then the packed upper triangle k(p, q) = p N - p (p - 1) / 2
   * + q - p (p <= q) of (L + L^T) / 2, n2pad = N (N + 1) / 2 rounded up to 128,
   * and the VHS (symmetric) is produced in that packed column order. */
  int vhs_packed;
  /* digit format of rot_slices: 1 = the FP16 digits described above (the only
   * format this library accepts) */
  int digit_format;
} trot_mixed;

/* Static description of one Hamiltonian + trial + propagation context.
 * Mirrors HamChol (trot/ham/chol.py:14-58), RhfMeasCtx / UhfMeasCtx
 * (trot/meas/rhf.py:282-319, trot/meas/uhf.py:277-336), CholAfqmcCtx
 * (trot/prop/chol_afqmc_ops.py:16-50) and the QmcParams fields the step reads
 * (trot/prop/types.py:30-47).  All pointers are device pointers.  For TROT_RHF_*
 * the *_b trial/rot pointers may be NULL (the alpha ones are used for both
 * spins). */
typedef struct {
  int kind;          /* trot_kind */
  int precision;     /* trot_precision */
  int n_walkers;     /* W */
  int norb;          /* N */
  int nchol;         /* G */
  int nocc_a;        /* columns of alpha (or restricted) walkers */
  int nocc_b;        /* columns of beta walkers (ignored for TROT_RHF_R) */
  int n_exp_terms;   /* Taylor terms, reference default 6 */
  double h0;
  double h0_prop;    /* -h0 - 1/2 sum_g mf_g^2 (real) */
  double dt;
  double sqrt_dt;
  double weight_floor;         /* 1e-3 */
  double weight_cap;           /* 100 */
  double pop_control_damping;  /* 0.1 */
  const double* mo_a;          /* (N, na) */
  const double* mo_b;          /* (N, nb) */
  const double* rot_h1_a;      /* (na, N) */
  const double* rot_h1_b;      /* (nb, N) */
  const double* rot_chol_a;    /* (G, na, N) */
  const double* rot_chol_b;    /* (G, nb, N) */
  const double* exp_h1_half;   /* (N, N) */
  const double* chol_flat;     /* (G, N*N) */
  const double* mf_shifts_im;  /* (G) imaginary parts of mf_shifts (real parts are 0) */
  const trot_mixed* mixed;     /* host struct of mixed-precision operands, or NULL */
  /* (G, N(N+1)/2): the upper triangle of every chol[g], row-major packed (k(p, q) = p N -
   * p (p - 1) / 2 + q - p, q >= p), when every chol[g] is exactly symmetric; else NULL.  The
   * FP64 VHS (and its transpose contraction in the step VJP) then runs over the packed
   * columns and is mirrored: half the FP64 products, the same values.  The FP64 step's and
   * apply-Trotter's workspace grows by W N(N+1)/2 complex values. */
  const double* chol_packed;
} trot_system;

/* Walker population.  Walkers are updated in place by the step. */
typedef struct {
  double* walkers_a;           /* complex128 (W, N, na) */
  double* walkers_b;           /* complex128 (W, N, nb); NULL for TROT_RHF_R */
  double* weights;             /* float64 (W) */
  double* overlaps;            /* complex128 (W) */
  double* scalars;             /* float64 [pop_control_ene_shift, e_estimate] */
  int64_t* node_encounters;    /* int64 [1] */
} trot_state;

const char* trot_last_error(void);
int trot_abi_version(void);

/* Bytes of workspace the given op needs for this system. */
size_t trot_workspace_size(const trot_system* sys, int op);

/* Trial overlaps of all walkers (complex128 out (W)).
 * Replaces overlap_r / overlap_u: trot/trial/rhf.py:45-54, trot/trial/uhf.py:48-58. */
int trot_overlap(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                 double* overlaps_out, void* stream);

/* Half-rotated Green's functions of all walkers, G_s = (w_s (C_s^H w_s)^{-1})^T
 * (_half_green_from_overlap_matrix, trot/meas/rhf.py:21-25, per spin for
 * unrestricted walkers): green_out complex128 (W, nocc_a + nocc_b, norb), rows
 * [0, nocc_a) alpha and [nocc_a, nocc_a + nocc_b) beta (restricted walkers:
 * (W, nocc_a, norb)); overlaps_out (optional) as trot_overlap. FP64. */
int trot_half_green(const trot_system* sys, const double* walkers_a, const double* walkers_b, double* green_out,
                    double* overlaps_out, void* stream);

/* Force bias of all walkers (complex128 out (W, G)).
 * Replaces force_bias_kernel_rw_rh / _uw_rh: trot/meas/rhf.py:119-125,141-153;
 * trot/meas/uhf.py:43-57. */
int trot_force_bias(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                    double* force_bias_out, void* workspace, size_t workspace_bytes, void* stream);

/* Local energy of all walkers (complex128 out (W)).
 * Replaces energy_kernel_rw_rh / _uw_rh: trot/meas/rhf.py:128-138,156-172;
 * trot/meas/uhf.py:205-231. */
int trot_local_energy(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                      double* energy_out, void* workspace, size_t workspace_bytes, void* stream);

/* exp(-dt/2 h1) exp(sqrt(dt) i VHS(x)) exp(-dt/2 h1) applied to every walker,
 * with complex128 shifted fields x (W, G); the Taylor series has
 * sys->n_exp_terms terms.  In-place allowed (out == in).
 * Replaces apply_trotter (trot/prop/chol_afqmc_ops.py:198-222,
 * trot/prop/utils.py:20-30). */
int trot_apply_trotter(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                       const double* shifted_fields, double* out_a, double* out_b,
                       void* workspace, size_t workspace_bytes, void* stream);

/* One phaseless step with injected float64 fields (W, G): force bias, field
 * shifts, Trotter propagation, overlaps, importance weights, population
 * control shift.  Updates *state in place.  If energy_out is not NULL it also
 * writes the local energy of the walkers at the START of the step
 * (complex128 (W)), reusing the step's Green's functions.
 * Replaces afqmc_step (trot/prop/afqmc.py:79-144). */
int trot_prop_step(const trot_system* sys, const trot_state* state, const double* fields,
                   double* energy_out, void* workspace, size_t workspace_bytes, void* stream);

/* Device status of the last mixed-precision op that used this workspace
 * (its first bytes): TROT_OK, or TROT_ERR_DEVICE_TIMEOUT when a tensor-core
 * kernel's completion wait ran out (the kernel then skipped its output, freed
 * its tensor memory and returned, and the op wrote NaN results: the local
 * energies, or the step's weights and population shift).  Synchronous
 * (cudaMemcpy). */
int trot_workspace_status(const void* workspace, int* status_out);

/* Sticky device status of every mixed-precision op that used this workspace
 * since the sticky word (the fourth int of the workspace) was last cleared:
 * TROT_ERR_DEVICE_TIMEOUT if any of them timed out as above, else TROT_OK.
 * A workspace whose first 16 bytes were zero-filled starts clear; clear != 0
 * resets the word after reading it.  Lets a caller that issues many
 * asynchronous calls (steps, graph replays) check once per block.
 * Synchronous.  No counterpart in the reference (it has no device waits). */
int trot_workspace_timeouts(void* workspace, int clear, int* status_out);

/* Reduced QR of every walker with diag(R) real non-negative; Q replaces the
 * walkers in place; norm_out (complex128 (W), may be NULL) receives
 * det(R)^2 (restricted) or det(R_a) det(R_b).
 * Replaces orthogonalize / orthonormalize (trot/walkers.py:137-179). */
int trot_orthonormalize(const trot_system* sys, double* walkers_a, double* walkers_b,
                        double* norm_out, void* stream);

/* Stochastic reconfiguration (comb resampling) with zeta in [0, 1) read from
 * the device (zeta_dev, float64 [1]) or, when zeta_dev is NULL, the value zeta:
 * idx_out (int64 (W)) = searchsorted(cumsum|w|, tot (k + zeta) / W, 'left');
 * walkers_out[k] = walkers_in[idx_out[k]]; weights_out[:] = tot / W.
 * Input and output walker buffers must not overlap.
 * Replaces stochastic_reconfiguration / _sr_indices (trot/walkers.py:249-293). */
int trot_sr_resample(const trot_system* sys, const double* weights_in, const double* zeta_dev, double zeta,
                     const double* walkers_a_in, const double* walkers_b_in,
                     double* walkers_a_out, double* walkers_b_out, double* weights_out,
                     int64_t* idx_out, void* workspace, size_t workspace_bytes, void* stream);

/* Block energy on the device (trot/prop/blocks.py:236-257): clamps Re(E_L)
 * to e_estimate when non-finite or further than sqrt(2/dt) from it, zeroes the
 * weights of non-finite walkers (in place), forms the weighted block energy
 * and updates e_estimate (scalars[1]) with the shift_ema moving average.
 * obs_out (float64 [2], device) receives [e_block, sum of weights]. */
int trot_block_energy(int n_walkers, const double* energy, double* weights, double* scalars, double dt,
                      double shift_ema, double* obs_out, void* stream);

/* The block's rdm1 observable (trot/prop/blocks.py:259-268 with
 * rdm1_kernel_rw / _uw, trot/meas/rhf.py:191-216, trot/meas/uhf.py:97-110):
 * rdm1_s = sum_w wt_w G_ws^T C_s^H / sum_w wt_w, complex128 (2, norb, norb)
 * (restricted walkers: the same matrix for both spins), zero when the weights
 * sum to 0.  green: trot_half_green's output for the block's walkers (after the
 * block's orthonormalisation); weights / obs: the guarded weights and the
 * [e_block, sum of weights] that trot_block_energy wrote (as in the reference,
 * a walker of weight 0 with a non-finite Green's function makes the sum NaN).
 * Workspace: trot_workspace_size(sys, TROT_OP_RDM1).  FP64. */
int trot_block_rdm1(const trot_system* sys, const double* green, const double* weights, const double* obs,
                    double* rdm1_out, void* workspace, size_t workspace_bytes, void* stream);

/* Auxiliary fields N(0, 1), float64 (W, G), drawn on the device from the
 * sub-key of `key` (int64 [2] device array holding two uint32 words,
 * Philox-4x32-10).  Replaces jax.random.normal in afqmc_step
 * (trot/prop/afqmc.py:91-93); call trot_split_key afterwards to advance. */
int trot_sample_normal_fields(const int64_t* key, int n_walkers, int nchol, double* fields, void* stream);

/* n uniforms in [0, 1) from the sub-key of `key` (the SR zeta,
 * trot/prop/blocks.py:270-271). */
int trot_sample_uniform(const int64_t* key, int n, double* out, void* stream);

/* key <- split(key)[0] in place on the device (jax.random.split pattern). */
int trot_split_key(int64_t* key, void* stream);

/* Local energy with no caller workspace and no allocation: same inputs,
 * output and numbers as trot_local_energy, with the scratch taken from a
 * fixed 32 MiB device array built into the library (held on every GPU that
 * loads it, until the process exits).  For callers that cannot allocate
 * device memory, e.g. a JAX custom call inside a process whose GPU memory
 * XLA has pre-allocated.  Systems needing more scratch than 32 MiB
 * (trot_workspace_size(sys, TROT_OP_LOCAL_ENERGY)) are rejected with
 * TROT_ERR_WORKSPACE_TOO_SMALL.  A call outside stream capture resolves the
 * array's address on the current device (cudaGetSymbolAddress) and caches it;
 * calls under capture use the cache, so the first call on a device must come
 * before any stream capture.  With CUDA's lazy module loading that first call
 * also reserves the 32 MiB: make it before a framework pre-allocates the GPU,
 * or set CUDA_MODULE_LOADING=EAGER.  All calls share the array, so calls that
 * overlap on the GPU race.  A mixed-precision call whose tensor-core kernel
 * timed out writes NaN energies; mixed-precision callers check
 * trot_local_energy_noalloc_status.  No counterpart in the reference. */
int trot_local_energy_noalloc(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                              double* energy_out, void* stream);

/* Sticky timeout status of trot_local_energy_noalloc on the current device
 * (trot_workspace_timeouts on the built-in array): TROT_ERR_DEVICE_TIMEOUT if
 * a call since the last clear had a tensor-core wait run out, else TROT_OK;
 * clear != 0 resets it.  Synchronous.  No counterpart in the reference. */
int trot_local_energy_noalloc_status(int clear, int* status_out);

/* ---------------------------------------------------------------- CISD trial
 * Configuration-interaction singles+doubles trial with restricted walkers in
 * the trial's MO basis (reference determinant = orbitals [0, nocc)), the
 * whole space active: nocc + nvir == norb (no frozen core, no outer
 * virtuals).  All arrays are device float64, row-major:
 *   ci1      (nocc, nvir)                      c_ia
 *   ci2m     (nocc*nvir, nocc*nvir)            2 c_iajb - c_ibja, row (i,a), column (j,b)
 *            (every doubles contraction of the overlap, force bias and energy
 *            uses c_iajb only in this combination)
 *   h1       (norb, norb), chol (nchol, norb, norb)
 *   lci1     (nchol, norb, nocc)               lci1[g][i][p] = sum_a chol[g][i][nocc+a] c_pa
 *   mo       (norb, nocc)                      the first nocc columns of I
 * Replaces CisdTrial / the CISD meas context (trot/trial/cisd.py:14-88,
 * trot/meas/cisd.py:772-836 build_meas_ctx). */
typedef struct {
  int norb, nocc, nvir, nchol;
  double h0;
  const double* ci1;
  const double* ci2m;
  const double* h1;
  const double* chol;
  const double* lci1;
  const double* mo;
  /* TROT_FP64, or TROT_MIXED: the l2ci2 quadratic forms on the tensor cores
   * (3-term BF16 split, FP32 accumulation), as the reference computes them in
   * float32 unless testing=True (trot/meas/cisd.py:838-839). */
  int l2ci2_precision;
  /* TROT_FP64, or TROT_MIXED: gl = G L_g and lci2_green in FP32 (the
   * reference's mixed_precision=True float32 contractions). */
  int gl_precision;
  /* for l2ci2_precision == TROT_MIXED: ci2m (nocc nvir columns padded to
   * ncpad, a multiple of 128; nocc nvir rows padded to nvpad, a multiple of
   * 64) as 3 BF16 slices in the tensor-core operand image
   * (trot_gb300.mixed.split3_image). */
  int nvpad, ncpad;
  const uint16_t* ci2_image;
  /* nonzero when every chol[g] is symmetric to working precision (checked by
   * the caller): the contraction chol . (ci1_green + ci2_green) then runs over
   * the packed upper triangle of (chol[g] + chol[g]^T) / 2 (norb (norb + 1) / 2
   * terms instead of norb^2). */
  int chol_symmetric;
} trot_cisd;

/* Device workspace for trot_cisd_overlap (TROT_OP_OVERLAP), trot_cisd_force_bias
 * (TROT_OP_FORCE_BIAS) or trot_cisd_local_energy (TROT_OP_LOCAL_ENERGY); 0 on bad
 * sizes.  The local energy needs 2 W nchol nocc nvir complex values for the
 * l2ci2 quadratic forms. */
size_t trot_cisd_workspace_size(const trot_cisd* cisd, int n_walkers, int op);
/* walkers: complex128 (W, norb, nocc); out complex128 (W).
 * overlap_r_high (trot/trial/cisd.py:148-186). */
int trot_cisd_overlap(const trot_cisd* cisd, int n_walkers, const double* walkers, double* overlap_out,
                      void* workspace, size_t workspace_bytes, void* stream);
/* out complex128 (W, nchol).  force_bias_kernel_rw_rh_high (trot/meas/cisd.py:548-572). */
int trot_cisd_force_bias(const trot_cisd* cisd, int n_walkers, const double* walkers, double* fb_out,
                         void* workspace, size_t workspace_bytes, void* stream);
/* out complex128 (W).  energy_kernel_rw_rh, "high" memory mode, float64
 * contractions (trot/meas/cisd.py:608-769). */
int trot_cisd_local_energy(const trot_cisd* cisd, int n_walkers, const double* walkers, double* energy_out,
                           void* workspace, size_t workspace_bytes, void* stream);

/* out complex128 (W, norb, norb): the mixed-estimator 1-RDM of one spin,
 * G0 - (ci1_green + ci2_green) / ov (rdm1_kernel_rw, trot/meas/cisd.py:772-820;
 * both spins are equal for restricted walkers).  Workspace as for
 * TROT_OP_FORCE_BIAS. */
int trot_cisd_rdm1(const trot_cisd* cisd, int n_walkers, const double* walkers, double* rdm1_out, void* workspace,
                   size_t workspace_bytes, void* stream);

/* One phaseless step with the CISD trial (trot/prop/afqmc.py:79-144 with
 * make_cisd_meas_ops): force bias (and, if energy_out is not null, the local
 * energy of the incoming walkers), shifted fields, VHS, Taylor propagation
 * with one-body half steps, CISD overlaps of the new walkers, phaseless
 * weights and population shift.  `prop` carries the propagation context (kind
 * TROT_RHF_R, n_walkers, n_exp_terms, dt, sqrt_dt, h0_prop,
 * weight_floor/cap, pop_control_damping, exp_h1_half, chol_flat,
 * mf_shifts_im; precision TROT_FP64, or TROT_MIXED with prop->mixed for the
 * tensor-core VHS / Taylor action); state->walkers_a (W, norb, nocc) is
 * updated in place.  Workspace: trot_cisd_workspace_size(cisd, W,
 * TROT_OP_PROP_STEP), plus trot_workspace_size(prop, TROT_OP_APPLY_TROTTER)
 * bytes (at the next 256-byte boundary) for the mixed propagation. */
int trot_cisd_prop_step(const trot_cisd* cisd, const trot_system* prop, const trot_state* state,
                        const double* fields, double* energy_out, void* workspace, size_t workspace_bytes,
                        void* stream);

/* ---------------------------------------------------------------- free projection
 * One free-projection step (trot/prop/afqmc_fp.py:18-72): unshifted fields
 * (W, nchol) float64, the Trotter action with sys->n_exp_terms terms (10 in
 * the reference) at sys->precision, walker columns times
 * exp(-sqrt(dt) sum_g x_g mf_g + dt h0_prop)^(1/n_total), QR norms
 * prod_j |R_jj| (qr_norm, trot/walkers.py:182-207), weights times the norms,
 * comb resampling with the device scalar *zeta_dev, and the resampled weights
 * divided by the selected walkers' norms.  sys->h0_prop includes ene0
 * (_build_prop_ctx_fp, trot/prop/chol_afqmc_ops_fp.py:49-72).  Walkers and
 * weights are updated in place; overlaps, scalars and node count are not read.
 * Workspace: trot_fp_workspace_size(sys) bytes. */
size_t trot_fp_workspace_size(const trot_system* sys);
int trot_fp_step(const trot_system* sys, const trot_state* state, const double* fields, const double* zeta_dev,
                 void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------- one-time constants on the device
 * Propagation context (replaces the host precompute _build_restricted_prop_ctx_from_host,
 * trot/runtime_layout.py:125-197, and _build_prop_ctx, trot/prop/chol_afqmc_ops.py:103-127):
 * from h1 (norb, norb), chol (nchol, norb, norb) and the spin-summed trial 1-RDM rdm1
 * (norb, norb), all float64 on the device, writes
 *   mf_im[g]    = tr(L_g rdm1)           (mf_shifts = i mf_im, nchol doubles)
 *   *h0_prop    = -h0 + 1/2 sum_g mf_im[g]^2
 *   exp_h1_half = expm(-dt/2 (h1 - 1/2 sum_g L_g L_g + sum_g mf_im[g] L_g))   (norb, norb)
 * Workspace: trot_prop_ctx_workspace_size(norb, nchol) bytes; after the stream
 * reaches the end of the call, trot_workspace_status(workspace) is
 * TROT_ERR_NUMERIC_GUARD when h1_eff had a non-finite entry or
 * dt/2 ||h1_eff||_1 > 2^39 (outputs undefined then), else TROT_OK. */
size_t trot_prop_ctx_workspace_size(int norb, int nchol);
int trot_build_prop_ctx(int norb, int nchol, double h0, double dt, const double* h1, const double* chol,
                        const double* rdm1, double* mf_im, double* h0_prop, double* exp_h1_half,
                        void* workspace, size_t workspace_bytes, void* stream);

/* Half rotation with a real trial (replaces _build_rhf_meas_ctx_from_host,
 * trot/runtime_layout.py:200-245, and build_meas_ctx, trot/meas/rhf.py:308-319,
 * trot/meas/uhf.py:318-336): rot_h1 = mo^T h1 (nocc, norb) and rot_chol[g] =
 * mo^T L_g (nchol, nocc, norb) for mo (norb, nocc) row-major.  Either h1 or chol
 * may be null (its output is then not written). */
int trot_half_rotate(int norb, int nchol, int nocc, const double* mo, const double* h1, const double* chol,
                     double* rot_h1, double* rot_chol, void* stream);

/* CISD lci1 (replaces the loop of _build_cisd_meas_ctx_from_host,
 * trot/runtime_layout.py:248-292; trot/meas/cisd.py:92-110):
 * lci1[g][i][p] = sum_t chol[g][i][nocc + t] ci1[p][t], ci1 (nocc, norb - nocc),
 * lci1 (nchol, norb, nocc). */
int trot_cisd_lci1(int norb, int nchol, int nocc, const double* ci1, const double* chol, double* lci1,
                   void* stream);

/* ---------------------------------------------------------------- adjoint (reverse mode)
 * Hand-written vector-Jacobian products in FP64 for TROT_RHF_R, TROT_RHF_U and
 * TROT_UHF_U (precision TROT_MIXED returns TROT_ERR_UNSUPPORTED).  The reference
 * has no adjoint: these differentiate its forward formulas
 * (trot/prop/afqmc.py:91-144, trot/meas/rhf.py:21-60,128-172,
 * trot/meas/uhf.py:205-231, trot/trial/rhf.py:45-54, trot/trial/uhf.py:54-58,
 * trot/walkers.py:137-179) so that gradients of an energy estimator with
 * respect to h1 come out of one run.  Cotangents of a real objective J:
 * g_z = dJ/dRe z + i dJ/dIm z for complex z (complex128 arrays laid out like
 * z), dJ/dz for real z; *_b arguments are ignored for TROT_RHF_R.  Workspace:
 * trot_vjp_workspace_size(sys, op) with op TROT_OP_PROP_STEP,
 * TROT_OP_LOCAL_ENERGY or TROT_OP_OVERLAP.
 *
 * trot_prop_step_vjp: given the state BEFORE the step (state_in), the step's
 * fields and the cotangents of the state after it (walkers, weights (may be
 * NULL), overlaps (may be NULL), scalars [E_shift, e_estimate]), writes the
 * cotangents of the state before it and adds dJ/d exp_h1_half (N x N) into
 * g_exp_h1_half.  The forward step is recomputed inside; walkers that the
 * step's floor / cap / non-finite guards (or a zero weight) remove from the
 * objective get exactly zero cotangents.
 * trot_local_energy_vjp: adds g_energy[b] * d Re E_L[b] / d walkers into
 * g_walkers and sum_b g_energy[b] d Re E_L[b] / d h1 (through rot_h1 = C^T h1)
 * into g_h1 (N x N).
 * trot_overlap_vjp: adds the cotangent of prod_s det(C_s^T w_s)^mult_s into g_walkers.
 * trot_orthonormalize_vjp: g_w = g_q (w^H q)^-1 per spin for q the orthonormalised
 * walkers (everything downstream is invariant under q -> q M). */
size_t trot_vjp_workspace_size(const trot_system* sys, int op);
int trot_prop_step_vjp(const trot_system* sys, const trot_state* state_in, const double* fields,
                       const double* g_walkers_out_a, const double* g_walkers_out_b, const double* g_weights_out,
                       const double* g_overlaps_out, const double* g_scalars_out, double* g_walkers_in_a,
                       double* g_walkers_in_b, double* g_weights_in, double* g_overlaps_in, double* g_scalars_in,
                       double* g_exp_h1_half, void* workspace, size_t workspace_bytes, void* stream);
int trot_local_energy_vjp(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                          const double* g_energy, double* g_walkers_a, double* g_walkers_b, double* g_h1,
                          void* workspace, size_t workspace_bytes, void* stream);
int trot_overlap_vjp(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                     const double* g_overlaps, double* g_walkers_a, double* g_walkers_b, void* workspace,
                     size_t workspace_bytes, void* stream);
int trot_orthonormalize_vjp(const trot_system* sys, const double* walkers_a, const double* walkers_b,
                            const double* q_a, const double* q_b, const double* g_q_a, const double* g_q_b,
                            double* g_walkers_a, double* g_walkers_b, void* stream);

/* Adjoint of the propagation context's exp(-dt/2 h1_eff) with respect to h1:
 * adds the Frechet-derivative adjoint of expm applied to g_exp_h1_half, times
 * -dt/2, into g_h1 (N x N); same inputs as trot_build_prop_ctx.  Workspace:
 * trot_prop_ctx_vjp_workspace_size(norb, nchol). */
size_t trot_prop_ctx_vjp_workspace_size(int norb, int nchol);
int trot_prop_ctx_vjp(int norb, int nchol, double dt, const double* h1, const double* chol, const double* rdm1,
                      const double* g_exp_h1_half, double* g_h1, void* workspace, size_t workspace_bytes,
                      void* stream);

/* Plain BF16 tensor-core GEMM (tcgen05, accumulator in tensor memory):
 * D (M x N, float32) = A (M x K, bf16) * B (N x K, bf16)^T, all row-major,
 * M and N multiples of 128, K a multiple of 64, A and B 16-byte aligned.
 * *status (device int) is set to TROT_ERR_DEVICE_TIMEOUT if a completion
 * wait ran out (the kernel then frees its tensor memory and returns).  The
 * building block of the mixed-precision kernels; no counterpart in the
 * reference (it has no hand-written GEMM). */
int trot_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, int* status,
                      void* stream);

/* Tuning knobs (process-wide; 0 restores the built-in default).  Chosen by
 * timing candidates on the caller's workload (trot_gb300.autotune); every
 * setting computes bit-identical results.  No counterpart in the reference.
 *   TROT_TUNE_EXCHANGE_TILES: walker tiles per work item of the exact-digit
 *     exchange kernel (default 8);
 *   TROT_TUNE_EXCHANGE_GRID: persistent CTAs of that kernel (default 152);
 *   TROT_TUNE_TEST_TIMEOUT: test switch of the device-timeout path, not a
 *     tuning knob: when v > 0 the exchange kernel's first wait is on a barrier
 *     nothing arrives on, limited to v polls, so it takes its timeout path
 *     (status TROT_ERR_DEVICE_TIMEOUT, no copies or MMAs issued, NaN energies)
 *     on every call until the knob is set back to 0. */
typedef enum {
  TROT_TUNE_EXCHANGE_TILES = 0,
  TROT_TUNE_EXCHANGE_GRID = 1,
  TROT_TUNE_TEST_TIMEOUT = 2,
  TROT_TUNE_COUNT = 3
} trot_tune_knob;
int trot_set_tuning(int knob, int value);
int trot_get_tuning(int knob);

/* Per-kernel timers for measurement: trot_profile_enable(n) creates a pool
 * for n launches (0 disables); while enabled every kernel launch of the C ABI
 * is bracketed by CUDA events on its stream.  trot_profile_collect
 * synchronises, writes up to max_names kernel names (48-byte slots), total
 * milliseconds and launch counts, clears the records and returns the number
 * of names.  Keep disabled during CUDA graph capture.  No counterpart in the
 * reference (it has no profiling hooks). */
int trot_profile_enable(int max_launches);
int trot_profile_collect(int max_names, char* names, double* total_ms, int* launches);
/* Kernel launches the library issued since the last trot_profile_enable,
 * timed or not (counted only while enabled). */
long long trot_profile_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* TROT_GB300_H */
