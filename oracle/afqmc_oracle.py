"""CPU oracle for the phaseless-AFQMC hot path.

TEST INFRASTRUCTURE ONLY. This module is the checker: only the test suite,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it. The product path (``trot_gb300``) never
calls it and has no CPU fallback.

It is a numpy complex128 restatement of trot's per-walker JAX functions,
written batched over walkers (leading axis W) instead of per-walker + vmap.
Each function cites the reference function it restates (paths are relative to
the trot repository root).

Parity pin: ``tests/golden/make_golden.py`` runs the reference's own modules
(with a numpy stand-in for the jax API) and stores their outputs under
``tests/golden/``; ``tests/test_oracle_golden.py`` checks this module against
those vectors, and ``tests/test_oracle_invariants.py`` against the reference
tests' known-answer cases (``tests/test_prop_afqmc_step.py``,
``tests/test_trial_rhf.py``).

Conventions
-----------
* walkers: restricted (W, N, n) complex128; unrestricted a pair
  ((W, N, na), (W, N, nb)).
* trial coefficients: real float64 (N, n) (RHF) or a pair (UHF).
* Cholesky vectors ``chol``: (G, N, N) real float64, symmetric.
* fields: (W, G) real float64, N(0, 1), injected by the caller.
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace

import numpy as np
import scipy.linalg

__all__ = [
    "PropCtx", "RhfMeasCtx", "UhfMeasCtx", "State", "Params",
    "build_prop_ctx", "build_rhf_meas_ctx", "build_uhf_meas_ctx",
    "half_green", "overlap_rhf_r", "overlap_rhf_u", "overlap_uhf_u",
    "force_bias_rhf_r", "force_bias_rhf_u", "force_bias_uhf_u",
    "energy_rhf_r", "energy_rhf_u", "energy_uhf_u",
    "make_vhs", "taylor_expm_action", "apply_trotter_r", "apply_trotter_u",
    "afqmc_step", "qr_phase_fixed", "orthogonalize", "orthonormalize",
    "sr_indices", "stochastic_reconfiguration", "block", "init_walkers",
]


# ----------------------------------------------------------------------------
# parameters and state


@dataclass(frozen=True)
class Params:
    """Mirror of ``QmcParams`` (trot/prop/types.py:30-47)."""

    dt: float = 0.005
    n_exp_terms: int = 6
    n_prop_steps: int = 50
    n_walkers: int = 200
    pop_control_damping: float = 0.1
    weight_floor: float = 1.0e-3
    weight_cap: float = 100.0
    shift_ema: float = 0.1


@dataclass
class State:
    """Mirror of ``PropState`` (trot/prop/types.py:20-27) without the rng key."""

    walkers: object
    weights: np.ndarray
    overlaps: np.ndarray
    pop_control_ene_shift: float
    e_estimate: float
    node_encounters: int = 0


# ----------------------------------------------------------------------------
# one-time contexts


@dataclass(frozen=True)
class PropCtx:
    """``CholAfqmcCtx`` (trot/prop/chol_afqmc_ops.py:16-50)."""

    dt: float
    sqrt_dt: float
    exp_h1_half: np.ndarray  # (N, N) real
    mf_shifts: np.ndarray  # (G,) complex, purely imaginary
    h0_prop: float
    chol_flat: np.ndarray  # (G, N*N) real
    norb: int


def build_prop_ctx(h0, h1, chol, rdm1, dt) -> PropCtx:
    """``_build_prop_ctx`` (trot/prop/chol_afqmc_ops.py:103-127).

    mf_shifts = i tr(L_g rho)            (:74-76, rho = rdm1[0] + rdm1[1])
    h0_prop   = -h0 - 1/2 sum_g mf_g^2   (:113)
    h1_eff    = h1 - 1/2 sum_g L_g L_g - sum_g Re(i mf_g) L_g   (:90-100)
    exp_h1_half = expm(-dt/2 h1_eff)     (:79-80)
    """
    rdm1 = np.asarray(rdm1)
    dm = rdm1[0] + rdm1[1] if (rdm1.ndim == 3 and rdm1.shape[0] == 2) else rdm1
    chol = np.asarray(chol, dtype=np.float64)
    G, N, _ = chol.shape
    mf = 1.0j * np.einsum("gij,ji->g", chol, dm)
    h0_prop = float(np.real(-h0 - 0.5 * np.sum(mf * mf)))
    v0 = 0.5 * np.einsum("gik,gkj->ij", chol, chol)
    v1 = np.einsum("g,gik->ik", np.real(1.0j * mf), chol)
    h1_eff = np.asarray(h1, dtype=np.float64) - v0 - v1
    exp_h1_half = scipy.linalg.expm(-0.5 * dt * h1_eff)
    return PropCtx(
        dt=float(dt),
        sqrt_dt=float(np.sqrt(dt)),
        exp_h1_half=np.real(exp_h1_half) if np.isrealobj(h1_eff) else exp_h1_half,
        mf_shifts=mf,
        h0_prop=h0_prop,
        chol_flat=chol.reshape(G, N * N),
        norb=N,
    )


@dataclass(frozen=True)
class RhfMeasCtx:
    """``RhfMeasCtx`` / ``build_meas_ctx`` (trot/meas/rhf.py:282-319)."""

    rot_h1: np.ndarray  # (n, N)
    rot_chol: np.ndarray  # (G, n, N)
    rot_chol_flat: np.ndarray  # (G, n*N)


def build_rhf_meas_ctx(h1, chol, mo) -> RhfMeasCtx:
    cH = np.conj(np.asarray(mo)).T
    rot_h1 = cH @ h1
    rot_chol = np.einsum("pi,gij->gpj", cH, chol)
    return RhfMeasCtx(rot_h1, rot_chol, rot_chol.reshape(rot_chol.shape[0], -1))


@dataclass(frozen=True)
class UhfMeasCtx:
    """``UhfMeasCtx`` / ``build_meas_ctx`` (trot/meas/uhf.py:277-336)."""

    rot_h1_a: np.ndarray
    rot_h1_b: np.ndarray
    rot_chol_a: np.ndarray
    rot_chol_b: np.ndarray


def build_uhf_meas_ctx(h1, chol, mo_a, mo_b) -> UhfMeasCtx:
    a = build_rhf_meas_ctx(h1, chol, mo_a)
    b = build_rhf_meas_ctx(h1, chol, mo_b)
    return UhfMeasCtx(a.rot_h1, b.rot_h1, a.rot_chol, b.rot_chol)


# ----------------------------------------------------------------------------
# trial overlaps and Green's functions


def _ovlp_mat(mo, w):
    """m = C^H w, batched: (W, n, n)."""
    return np.einsum("pi,bpj->bij", np.conj(mo), w)


def half_green(w, mo):
    """``_half_green_from_overlap_matrix`` (trot/meas/rhf.py:21-25):
    green_half = solve(m^T, w^T) = (w m^{-1})^T, shape (W, n, N)."""
    m = _ovlp_mat(mo, w)
    return np.linalg.solve(np.swapaxes(m, -1, -2), np.swapaxes(w, -1, -2))


def overlap_rhf_r(w, mo):
    """``overlap_r`` (trot/trial/rhf.py:45-47): det(C^H w)^2."""
    d = np.linalg.det(_ovlp_mat(mo, w))
    return d * d


def overlap_rhf_u(wu, wd, mo):
    """``overlap_u`` (trot/trial/rhf.py:50-54)."""
    return np.linalg.det(_ovlp_mat(mo, wu)) * np.linalg.det(_ovlp_mat(mo, wd))


def overlap_uhf_u(wu, wd, mo_a, mo_b):
    """``overlap_u`` (trot/trial/uhf.py:54-58)."""
    return np.linalg.det(_ovlp_mat(mo_a, wu)) * np.linalg.det(_ovlp_mat(mo_b, wd))


# ----------------------------------------------------------------------------
# force bias


def force_bias_rhf_r(w, mo, ctx: RhfMeasCtx):
    """``force_bias_kernel_rw_rh`` (trot/meas/rhf.py:119-125)."""
    g = half_green(w, mo)
    return 2.0 * (g.reshape(g.shape[0], -1) @ ctx.rot_chol_flat.T)


def force_bias_rhf_u(wu, wd, mo, ctx: RhfMeasCtx):
    """``force_bias_kernel_uw_rh`` (trot/meas/rhf.py:141-153)."""
    g = half_green(wu, mo) + half_green(wd, mo)
    return g.reshape(g.shape[0], -1) @ ctx.rot_chol_flat.T


def force_bias_uhf_u(wu, wd, mo_a, mo_b, ctx: UhfMeasCtx):
    """``force_bias_kernel_uw_rh`` (trot/meas/uhf.py:43-57)."""
    gu = half_green(wu, mo_a)
    gd = half_green(wd, mo_b)
    G = ctx.rot_chol_a.shape[0]
    fa = gu.reshape(gu.shape[0], -1) @ ctx.rot_chol_a.reshape(G, -1).T
    fb = gd.reshape(gd.shape[0], -1) @ ctx.rot_chol_b.reshape(G, -1).T
    return fa + fb


# ----------------------------------------------------------------------------
# local energy


def _coul_exch(g, rot_chol):
    """f_g = rot_chol_g @ g^T per walker; returns (c (W,G), exchange (W,)).

    (trot/meas/rhf.py:41-60 "high" mode; trot/meas/uhf.py:220-225)."""
    f = np.matmul(rot_chol[None], np.swapaxes(g, -1, -2)[:, None])  # (W, G, n, n), BLAS batched
    c = np.einsum("bgii->bg", f)
    exc = np.sum(f * np.swapaxes(f, -1, -2), axis=(1, 2, 3))
    return c, exc


def energy_rhf_r(w, mo, h0, ctx: RhfMeasCtx):
    """``energy_kernel_rw_rh`` (trot/meas/rhf.py:128-138):
    E = h0 + 2 sum(G o rot_h1) + 2 sum_g c_g^2 - sum_g sum_ij f_gij f_gji."""
    g = half_green(w, mo)
    e1 = 2.0 * np.einsum("bij,ij->b", g, ctx.rot_h1)
    c, exc = _coul_exch(g, ctx.rot_chol)
    return h0 + e1 + 2.0 * np.sum(c * c, axis=1) - exc


def energy_rhf_u(wu, wd, mo, h0, ctx: RhfMeasCtx):
    """``energy_kernel_uw_rh`` (trot/meas/rhf.py:156-172)."""
    gu = half_green(wu, mo)
    gd = half_green(wd, mo)
    e1 = np.einsum("bij,ij->b", gu + gd, ctx.rot_h1)
    cu, xu = _coul_exch(gu, ctx.rot_chol)
    cd, xd = _coul_exch(gd, ctx.rot_chol)
    e2 = (np.sum(cu * cu, 1) + np.sum(cd * cd, 1) + 2.0 * np.sum(cu * cd, 1) - xu - xd) / 2.0
    return h0 + e1 + e2


def energy_uhf_u(wu, wd, mo_a, mo_b, h0, ctx: UhfMeasCtx):
    """``energy_kernel_uw_rh`` (trot/meas/uhf.py:205-231)."""
    gu = half_green(wu, mo_a)
    gd = half_green(wd, mo_b)
    e1 = np.einsum("bij,ij->b", gu, ctx.rot_h1_a) + np.einsum("bij,ij->b", gd, ctx.rot_h1_b)
    cu, xu = _coul_exch(gu, ctx.rot_chol_a)
    cd, xd = _coul_exch(gd, ctx.rot_chol_b)
    e2 = (np.sum(cu * cu, 1) + np.sum(cd * cd, 1) + 2.0 * np.sum(cu * cd, 1) - xu - xd) / 2.0
    return h0 + e1 + e2


# ----------------------------------------------------------------------------
# propagation


def make_vhs(x, ctx: PropCtx):
    """``_make_vhs_split_flat`` (trot/prop/chol_afqmc_ops.py:83-87), batched:
    VHS_b = Re(x_b) @ chol_flat + i Im(x_b) @ chol_flat, reshaped (W, N, N)."""
    x = np.asarray(x)
    N = ctx.norb
    v = np.real(x) @ ctx.chol_flat + 1.0j * (np.imag(x) @ ctx.chol_flat)
    return v.reshape(x.shape[0], N, N)


def taylor_expm_action(a, mat, vecs, n_terms):
    """``taylor_expm_action`` (trot/prop/utils.py:20-30), batched over W."""
    out = vecs
    term = vecs
    for k in range(1, n_terms + 1):
        term = (a / k) * (mat @ term)
        out = out + term
    return out


def apply_trotter_r(w, x, ctx: PropCtx, n_terms):
    """``_apply_trotter_r`` (trot/prop/chol_afqmc_ops.py:198-208)."""
    e = ctx.exp_h1_half
    v = make_vhs(x, ctx)
    w1 = e @ w
    w2 = taylor_expm_action(1.0j * ctx.sqrt_dt, v, w1, n_terms)
    return e @ w2


def apply_trotter_u(wu, wd, x, ctx: PropCtx, n_terms):
    """``_apply_trotter_u`` (trot/prop/chol_afqmc_ops.py:211-222): one VHS
    shared by both spins."""
    e = ctx.exp_h1_half
    v = make_vhs(x, ctx)
    a = 1.0j * ctx.sqrt_dt
    ou = e @ taylor_expm_action(a, v, e @ wu, n_terms)
    od = e @ taylor_expm_action(a, v, e @ wd, n_terms)
    return ou, od


def phaseless_weights(state: State, overlaps_new, shift_term, fb_term, ctx: PropCtx, params: Params):
    """Importance-function block of ``afqmc_step`` (trot/prop/afqmc.py:111-134).

    Returns (weights_new, node_encounters_new, pop_control_ene_shift_new)."""
    ratio = overlaps_new / state.overlaps
    exponent = -ctx.sqrt_dt * shift_term + fb_term + ctx.dt * (state.pop_control_ene_shift + ctx.h0_prop)
    with np.errstate(all="ignore"):
        imp = np.exp(exponent) * ratio
        theta = np.angle(np.exp(-ctx.sqrt_dt * shift_term) * ratio)
        imp_ph = np.abs(imp) * np.cos(theta)
        imp_ph = np.where(~np.isfinite(imp_ph) | (imp_ph < params.weight_floor), 0.0, imp_ph)
        nodes = state.node_encounters + int(np.sum(imp_ph <= 0.0))
        imp_ph = np.where(imp_ph > params.weight_cap, 0.0, imp_ph)
        wn = state.weights * imp_ph
        wn = np.where(wn > params.weight_cap, 0.0, wn)
        avg_w = max(float(np.mean(wn)), 1.0e-300)
        shift = state.e_estimate - params.pop_control_damping * (np.log(avg_w) / ctx.dt)
    return wn, nodes, float(shift)


def field_shifts(force_bias, ctx: PropCtx, x):
    """Shifted fields (trot/prop/afqmc.py:99-103): returns (x - s, shift_term, fb_term)."""
    s = -ctx.sqrt_dt * (1.0j * force_bias - ctx.mf_shifts[None, :])
    xs = x - s
    shift_term = np.sum(xs * ctx.mf_shifts[None, :], axis=1)
    fb_term = np.sum(x * s - 0.5 * s * s, axis=1)
    return xs, shift_term, fb_term


@dataclass(frozen=True)
class Model:
    """Everything one phaseless step needs for one (trial, walker) kind.

    kind: "rhf_r" (RHF trial, restricted walkers), "rhf_u" (RHF trial,
    unrestricted walkers) or "uhf_u" (UHF trial, unrestricted walkers)."""

    kind: str
    h0: float
    mo: object  # (N, n) or (mo_a, mo_b)
    meas: object  # RhfMeasCtx | UhfMeasCtx
    prop: PropCtx

    def overlap(self, w):
        if self.kind == "rhf_r":
            return overlap_rhf_r(w, self.mo)
        if self.kind == "rhf_u":
            return overlap_rhf_u(w[0], w[1], self.mo)
        return overlap_uhf_u(w[0], w[1], self.mo[0], self.mo[1])

    def force_bias(self, w):
        if self.kind == "rhf_r":
            return force_bias_rhf_r(w, self.mo, self.meas)
        if self.kind == "rhf_u":
            return force_bias_rhf_u(w[0], w[1], self.mo, self.meas)
        return force_bias_uhf_u(w[0], w[1], self.mo[0], self.mo[1], self.meas)

    def energy(self, w):
        if self.kind == "rhf_r":
            return energy_rhf_r(w, self.mo, self.h0, self.meas)
        if self.kind == "rhf_u":
            return energy_rhf_u(w[0], w[1], self.mo, self.h0, self.meas)
        return energy_uhf_u(w[0], w[1], self.mo[0], self.mo[1], self.h0, self.meas)

    def trotter(self, w, xs, n_terms):
        if self.kind == "rhf_r":
            return apply_trotter_r(w, xs, self.prop, n_terms)
        return apply_trotter_u(w[0], w[1], xs, self.prop, n_terms)

    @property
    def walker_kind(self):
        return "restricted" if self.kind == "rhf_r" else "unrestricted"

    def rdm1(self, w):
        """Per-walker one-body RDMs (W, 2, N, N): ``rdm1_kernel_rw`` / ``_uw``
        (trot/meas/rhf.py:191-216, trot/meas/uhf.py:97-110): G_s^T C_s^H per spin,
        the same matrix twice for restricted walkers."""
        if self.kind == "rhf_r":
            g = np.swapaxes(half_green(w, self.mo), -1, -2) @ np.conj(self.mo).T
            return np.stack([g, g], axis=1)
        ma, mb = (self.mo, self.mo) if self.kind == "rhf_u" else self.mo
        da = np.swapaxes(half_green(w[0], ma), -1, -2) @ np.conj(ma).T
        db = np.swapaxes(half_green(w[1], mb), -1, -2) @ np.conj(mb).T
        return np.stack([da, db], axis=1)


def afqmc_step(state: State, model: Model, params: Params, fields) -> State:
    """``afqmc_step`` (trot/prop/afqmc.py:79-144) with injected fields (W, G)."""
    ctx = model.prop
    fb = model.force_bias(state.walkers)
    xs, shift_term, fb_term = field_shifts(fb, ctx, fields)
    wn = model.trotter(state.walkers, xs, params.n_exp_terms)
    ov = model.overlap(wn)
    weights, nodes, shift = phaseless_weights(state, ov, shift_term, fb_term, ctx, params)
    return State(wn, weights, ov, shift, state.e_estimate, nodes)


# ----------------------------------------------------------------------------
# walkers


def qr_phase_fixed(mat):
    """``_qr`` (trot/walkers.py:137-148), batched: reduced QR with diag(R)
    made real non-negative; returns (q, det_r)."""
    q, r = np.linalg.qr(mat, mode="reduced")
    d = np.diagonal(r, axis1=-2, axis2=-1)
    ad = np.abs(d)
    phase = d / np.where(ad == 0, 1.0, ad)
    q = q * np.conj(phase)[:, None, :]
    r = phase[:, :, None] * r
    det_r = np.prod(np.diagonal(r, axis1=-2, axis2=-1), axis=-1)
    return q, det_r


def orthogonalize(w, walker_kind):
    """``orthogonalize`` (trot/walkers.py:151-171)."""
    if walker_kind == "unrestricted":
        qu, du = qr_phase_fixed(w[0])
        qd, dd = qr_phase_fixed(w[1])
        return (qu, qd), du * dd
    q, d = qr_phase_fixed(w)
    return q, (d * d if walker_kind == "restricted" else d)


def orthonormalize(w, walker_kind):
    """``orthonormalize`` (trot/walkers.py:174-179)."""
    return orthogonalize(w, walker_kind)[0]


def sr_indices(weights, zeta, n):
    """``_sr_indices`` (trot/walkers.py:249-254)."""
    cw = np.cumsum(np.abs(weights))
    z = cw[-1] * (np.arange(n) + zeta) / n
    return np.searchsorted(cw, z, side="left")


def stochastic_reconfiguration(w, weights, zeta, walker_kind):
    """``stochastic_reconfiguration`` (trot/walkers.py:257-293)."""
    n = weights.shape[0]
    cw = np.cumsum(np.abs(weights))
    avg = cw[-1] / n
    idx = sr_indices(weights, zeta, n)
    if walker_kind == "unrestricted":
        wn = (w[0][idx], w[1][idx])
    else:
        wn = w[idx]
    return wn, np.full((n,), avg, dtype=weights.dtype), idx


def block(state: State, model: Model, params: Params, fields_seq, zeta, rdm1=False):
    """``block`` (trot/prop/blocks.py:195-287): n_prop_steps steps with injected
    fields, orthonormalise, energy with outlier clamp, EMA of e_estimate, SR with
    injected zeta. Returns (state, e_block, w_sum), and with ``rdm1`` also the
    block's rdm1 observable (blocks.py:259-268): sum_w wt_w rdm1_w / sum_w wt_w
    over the guarded weights (zeros when they sum to 0; 0 x NaN stays NaN, as there)."""
    for x in fields_seq:
        state = afqmc_step(state, model, params, x)
    w = orthonormalize(state.walkers, model.walker_kind)
    ov = model.overlap(w)
    e = np.real(model.energy(w))
    thresh = np.sqrt(2.0 / params.dt)
    e_ref = state.e_estimate
    with np.errstate(invalid="ignore"):
        is_nan = ~np.isfinite(e)
        e = np.where(is_nan | (np.abs(e - e_ref) > thresh), e_ref, e)
    weights = np.where(is_nan, 0.0, state.weights)
    w_sum = float(np.sum(weights))
    w_safe = 1.0 if w_sum == 0 else w_sum
    e_block = float(np.sum(weights * e) / w_safe)
    if w_sum == 0:
        e_block = e_ref
    alpha = params.shift_ema
    e_est = (1.0 - alpha) * state.e_estimate + alpha * e_block
    if rdm1:
        samples = model.rdm1(w)
        num = np.einsum("b,bsij->sij", weights, samples)
        obs_rdm1 = np.zeros_like(num) if w_sum == 0 else num / w_safe
    w_sr, weights_sr, _ = stochastic_reconfiguration(w, weights, zeta, model.walker_kind)
    ov_sr = model.overlap(w_sr)
    st = State(w_sr, weights_sr, ov_sr, state.pop_control_ene_shift, e_est, state.node_encounters)
    if rdm1:
        return st, e_block, w_sum, obs_rdm1
    return st, e_block, w_sum


def qr_norm(w, walker_kind):
    """``qr_norm`` (trot/walkers.py:182-207): det of the phase-fixed R only
    (R = phase * R, det = prod diag), squared for restricted walkers."""

    def det_r(mat):
        r = np.linalg.qr(mat, mode="r")
        d = np.diagonal(r, axis1=-2, axis2=-1)
        ad = np.abs(d)
        phase = d / np.where(ad == 0, 1.0, ad)
        return np.prod(phase * d, axis=-1)

    if walker_kind == "unrestricted":
        return det_r(w[0]) * det_r(w[1])
    d = det_r(w)
    return d * d if walker_kind == "restricted" else d


def multiply_constants(w, constants, walker_kind):
    """``multiply_constants`` (trot/walkers.py:210-227): c^(1/n_total) on every column."""
    constants = np.asarray(constants)
    if walker_kind == "unrestricted":
        n_total = w[0].shape[-1] + w[1].shape[-1]
        c = (constants ** (1.0 / n_total))[:, None, None]
        return (w[0] * c, w[1] * c)
    n_total = 2 * w.shape[-1]
    c = (constants ** (1.0 / n_total))[:, None, None]
    return w * c


def afqmc_step_fp(state: State, model: Model, fields, zeta, n_terms=10):
    """``afqmc_step_fp`` (trot/prop/afqmc_fp.py:18-72) with injected fields (W, G) and zeta;
    ``model.prop`` is the free-projection context (h0_prop includes ene0)."""
    ctx = model.prop
    shift_term = fields @ ctx.mf_shifts
    constants = np.exp(-ctx.sqrt_dt * shift_term + ctx.dt * ctx.h0_prop)
    wn = model.trotter(state.walkers, fields.astype(np.complex128), n_terms)
    wn = multiply_constants(wn, constants, model.walker_kind)
    norms = qr_norm(wn, model.walker_kind)
    weights = state.weights * norms.real
    n = weights.shape[0]
    idx = sr_indices(weights, zeta, n)
    w_sr, weights_sr, _ = stochastic_reconfiguration(wn, weights, zeta, model.walker_kind)
    weights_sr = weights_sr / norms[idx].real
    return State(w_sr, weights_sr, state.overlaps, state.pop_control_ene_shift, state.e_estimate,
                 state.node_encounters)


def natorbs(dm, n_occ):
    """``_natorbs`` (trot/walkers.py:14-17)."""
    dm = 0.5 * (dm + np.conj(dm.T))
    vecs = np.linalg.eigh(dm)[1][:, ::-1]
    return vecs[:, :n_occ]


def init_walkers(walker_kind, rdm1, nup, ndn, n_walkers):
    """``init_walkers`` (trot/walkers.py:20-78) for restricted / unrestricted."""
    if walker_kind == "restricted":
        w0 = natorbs(rdm1[0] + rdm1[1], nup) + 0.0j
        return np.broadcast_to(w0, (n_walkers,) + w0.shape).copy()
    wu = natorbs(rdm1[0], nup) + 0.0j
    wd = natorbs(rdm1[1], ndn) + 0.0j
    return (np.broadcast_to(wu, (n_walkers,) + wu.shape).copy(),
            np.broadcast_to(wd, (n_walkers,) + wd.shape).copy())
