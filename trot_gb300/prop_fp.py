"""Free-projection AFQMC step (trot/prop/afqmc_fp.py), one call into the C ABI
(``trot_fp_step``): unshifted fields, the Trotter action with 10 Taylor terms,
the per-walker constants, QR norms, comb resampling and the norm-corrected
weights, all on the device.  ``make_prop_ops_fp`` returns the reference's
``PropOps(init_prop_state, build_prop_ctx, step)`` triple."""
from __future__ import annotations

import ctypes

import torch

from . import _lib, native, rng
from .core import PropOps, PropState, QmcParamsFp, System
from .prop import CholAfqmcCtx, _build_prop_ctx, _h0, init_prop_state

FP_EXP_TERMS = 10  # trot/prop/afqmc_fp.py:41


def build_prop_ctx_fp(ham_data, rdm1, dt: float, ene0: float, mixed_precision: bool = False) -> CholAfqmcCtx:
    """``_build_prop_ctx_fp`` (trot/prop/chol_afqmc_ops_fp.py:49-72): the phaseless
    context with h0_prop shifted by ene0."""
    ctx = _build_prop_ctx(ham_data, rdm1, dt, mixed_precision=mixed_precision)
    return CholAfqmcCtx(dt=ctx.dt, sqrt_dt=ctx.sqrt_dt, exp_h1_half=ctx.exp_h1_half, mf_shifts_im=ctx.mf_shifts_im,
                        h0_prop=ctx.h0_prop + float(ene0), chol_flat=ctx.chol_flat, norb=ctx.norb,
                        chol_packed=ctx.chol_packed)


def afqmc_step_fp(state: PropState, sys: System, *, params, ham_data, trial_data, prop_ctx: CholAfqmcCtx,
                  precision: int = _lib.FP64, fields=None, zeta=None) -> PropState:
    """trot/prop/afqmc_fp.py:18-72.  ``fields`` (W, G) float64 and ``zeta`` (1,)
    float64 CUDA tensors; drawn from ``state.rng_key`` when None."""
    kind = native.kind_of(trial_data, sys.walker_kind)
    wa, wb = native.split_walkers(state.walkers, kind)
    W = wa.shape[0]
    s = native.system(kind, W, trial_data, None, prop_ctx, h0=_h0(ham_data), params=params, precision=precision)
    s.n_exp_terms = FP_EXP_TERMS
    if fields is None:
        fields = rng.normal_fields(state.rng_key, W, s.nchol)
    elif fields.dtype != torch.float64 or not fields.is_cuda or tuple(fields.shape) != (W, s.nchol):
        raise ValueError("fields must be a (W, G) float64 CUDA tensor")
    if zeta is None:
        zeta = rng.uniform(state.rng_key, 1)
    fields, zeta = fields.contiguous(), zeta.to(torch.float64).contiguous()
    st = _lib.TrotState()
    st.walkers_a, st.walkers_b = native.ptr(wa), native.ptr(wb)
    st.weights, st.overlaps = state.weights.data_ptr(), state.overlaps.data_ptr()
    st.scalars, st.node_encounters = state.scalars.data_ptr(), state.node_encounters.data_ptr()
    n = _lib.load().trot_fp_workspace_size(ctypes.byref(s))
    if n == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    buf = native.workspace(n)
    _lib.call("trot_fp_step", ctypes.byref(s), ctypes.byref(st), fields.data_ptr(), zeta.data_ptr(),
              buf.data_ptr(), buf.numel(), native.stream_ptr())
    return state


def make_prop_ops_fp(ham_basis: str, walker_kind: str, sys: System, mixed_precision: bool = False) -> PropOps:
    """trot/prop/afqmc_fp.py:75-118."""
    if ham_basis != "restricted":
        raise NotImplementedError(f"CUDA path: ham_basis {ham_basis}")
    if walker_kind.lower() not in ("restricted", "unrestricted"):
        raise NotImplementedError(f"CUDA path: walker_kind {walker_kind}")
    precision = _lib.MIXED if mixed_precision else _lib.FP64

    def step_fp(state: PropState, *, params, ham_data, trial_data, trial_ops, meas_ops, meas_ctx, prop_ctx,
                fields=None, zeta=None) -> PropState:
        return afqmc_step_fp(state, sys, params=params, ham_data=ham_data, trial_data=trial_data,
                             prop_ctx=prop_ctx, precision=precision, fields=fields, zeta=zeta)

    def build_prop_ctx(ham_data, rdm1, params) -> CholAfqmcCtx:
        if not isinstance(params, QmcParamsFp):
            raise TypeError("free projection needs QmcParamsFp")
        if params.ene0 is None:
            raise ValueError("ene0 must be set for FP propagation")
        return build_prop_ctx_fp(ham_data, rdm1, params.dt, params.ene0, mixed_precision=mixed_precision)

    return PropOps(init_prop_state=init_prop_state, build_prop_ctx=build_prop_ctx, step=step_fp)
