"""Phaseless Cholesky AFQMC propagation (trot/prop/afqmc.py,
trot/prop/chol_afqmc_ops.py), driving the CUDA step.

``make_prop_ops(ham_basis, walker_kind, mixed_precision)`` returns the same
``PropOps(init_prop_state, build_prop_ctx, step)`` triple as the reference.
``step`` is one call into the C ABI (``trot_prop_step``): force bias, field
shifts, VHS, Taylor propagation, overlaps, phaseless weights and the
population-control shift, all on the device, with no host synchronisation.
The state's buffers are updated in place and the same state is returned.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Any, NamedTuple

import numpy as np
import torch

from . import _lib, native, rng
from . import ctx as ctx_dev
from .core import HamChol, MeasOps, PropOps, PropState, QmcParamsBase, System, TrialOps, k_energy


@dataclass(frozen=True)
class CholAfqmcCtx:
    """trot/prop/chol_afqmc_ops.py:16-50.  ``mf_shifts`` are purely imaginary;
    the device keeps their imaginary parts (``mf_shifts_im``)."""

    dt: float
    sqrt_dt: float
    exp_h1_half: torch.Tensor  # (N, N) float64
    mf_shifts_im: torch.Tensor  # (G,) float64
    h0_prop: float
    chol_flat: torch.Tensor  # (G, N*N) float64
    norb: int
    # (G, N(N+1)/2) upper triangles when every chol[g] is exactly symmetric (the FP64 VHS is then
    # built over the packed columns: half the products, identical values), else None
    chol_packed: torch.Tensor | None = None

    @property
    def mf_shifts(self) -> torch.Tensor:
        return torch.complex(torch.zeros_like(self.mf_shifts_im), self.mf_shifts_im)


def _build_prop_ctx(ham_data: HamChol, rdm1, dt: float, mixed_precision: bool = False) -> CholAfqmcCtx:
    """One-time propagation constants (trot/prop/chol_afqmc_ops.py:74-127; host
    twin trot/runtime_layout.py:125-197), built on the device by
    ``trot_build_prop_ctx``: mf = i tr(L_g rho), h0_prop = -h0 - 1/2 sum mf^2,
    exp(-dt/2 h1_eff) with h1_eff = h1 - 1/2 sum_g L_g L_g - sum_g Re(i mf_g) L_g."""
    h0 = float(np.real(np.asarray(ham_data.h0.item() if isinstance(ham_data.h0, torch.Tensor) else ham_data.h0)))
    mf_im, h0_prop, eh, chol = ctx_dev.prop_ctx(h0, ham_data.h1, ham_data.chol, rdm1, dt)
    G, N = int(chol.shape[0]), int(chol.shape[1])
    return CholAfqmcCtx(dt=float(dt), sqrt_dt=float(np.sqrt(dt)), exp_h1_half=eh, mf_shifts_im=mf_im,
                        h0_prop=h0_prop, chol_flat=chol.reshape(G, N * N), norb=N, chol_packed=pack_symmetric(chol))


def pack_symmetric(chol: torch.Tensor) -> torch.Tensor | None:
    """Row-major packed upper triangles (G, N(N+1)/2) of the Cholesky vectors when every
    chol[g] is exactly symmetric, else None."""
    N = int(chol.shape[1])
    if N == 0 or not bool(torch.equal(chol, chol.transpose(1, 2))):
        return None
    iu = torch.triu_indices(N, N, device=chol.device)
    return chol[:, iu[0], iu[1]].contiguous()


class TrotterOps(NamedTuple):
    apply_trotter: Any


def make_trotter_ops(ham_basis: str, walker_kind: str, mixed_precision: bool = False) -> TrotterOps:
    """trot/prop/chol_afqmc_ops.py:240-289, batched: apply_trotter(walkers (W,...),
    shifted_fields (W, G) complex, ctx, n_terms)."""
    if ham_basis != "restricted":
        raise NotImplementedError(f"CUDA path: ham_basis {ham_basis}")
    wk = walker_kind.lower()
    if wk not in ("restricted", "unrestricted"):
        raise NotImplementedError(f"CUDA path: walker_kind {walker_kind}")
    prec = _lib.MIXED if mixed_precision else _lib.FP64

    def apply_trotter(walkers, fields, ctx: CholAfqmcCtx, n_terms: int):
        unres = wk == "unrestricted"
        wa, wb = (walkers if unres else (walkers, None))
        W, N, na = wa.shape
        nb = wb.shape[2] if unres else 0
        native.check_walker_tensor(wa, N, na)
        if unres:
            native.check_walker_tensor(wb, N, nb, W)
        xs = fields.to(torch.complex128).contiguous()
        if tuple(xs.shape) != (W, ctx.chol_flat.shape[0]):
            raise ValueError(f"fields shape {tuple(xs.shape)} != (W, G)")
        s = _lib.TrotSystem()
        s.kind = _lib.UHF_U if unres else _lib.RHF_R
        s.precision = prec
        s.n_walkers, s.norb, s.nchol = W, N, int(ctx.chol_flat.shape[0])
        s.nocc_a, s.nocc_b = na, nb
        s.n_exp_terms = int(n_terms)
        s.sqrt_dt, s.dt = ctx.sqrt_dt, ctx.dt
        s.exp_h1_half, s.chol_flat = native.ptr(ctx.exp_h1_half), native.ptr(ctx.chol_flat)
        s.chol_packed = native.ptr(ctx.chol_packed)
        s.mf_shifts_im = native.ptr(ctx.mf_shifts_im)
        if prec == _lib.MIXED:
            from . import mixed

            s.mixed = mixed.context(None, ctx).data_ptr()
        s.mo_a = s.mo_b = s.exp_h1_half  # not read by the Trotter op; keeps the struct check satisfied
        oa = torch.empty_like(wa)
        ob = torch.empty_like(wb) if unres else None
        ws, nws = native.ws_for(s, _lib.OP_APPLY_TROTTER)
        _lib.call("trot_apply_trotter", ctypes.byref(s), native.ptr(wa), native.ptr(wb), xs.data_ptr(),
                  native.ptr(oa), native.ptr(ob), ws, nws, native.stream_ptr())
        return (oa, ob) if unres else oa

    return TrotterOps(apply_trotter)


def _h0(ham_data) -> float:
    h0 = ham_data.h0
    if isinstance(h0, torch.Tensor):
        h0 = h0.item()
    return float(np.real(np.asarray(h0)))


def afqmc_step(state: PropState, *, params, ham_data, trial_data, meas_ops: MeasOps, prop_ctx: CholAfqmcCtx,
               meas_ctx, walker_kind: str, precision: int = _lib.FP64, fields=None, energy_out=None) -> PropState:
    """trot/prop/afqmc.py:79-144.  ``fields`` (W, G) float64 device tensor; when
    None they are drawn on the device from ``state.rng_key`` (which is advanced).
    If ``energy_out`` (W,) complex128 is given it receives the local energy of
    the walkers entering the step."""
    from .cisd import CisdTrial

    if isinstance(trial_data, CisdTrial):
        from . import cisd

        return cisd.afqmc_step(state, params=params, ham_data=ham_data, trial_data=trial_data, meas_ctx=meas_ctx,
                               prop_ctx=prop_ctx, fields=fields, energy_out=energy_out, precision=precision)
    kind = native.kind_of(trial_data, walker_kind)
    wa, wb = native.split_walkers(state.walkers, kind)
    W = wa.shape[0]
    s = native.system(kind, W, trial_data, meas_ctx, prop_ctx, h0=_h0(ham_data), params=params,
                      precision=precision)
    if fields is None:
        fields = rng.normal_fields(state.rng_key, W, s.nchol)
    elif fields.dtype != torch.float64 or not fields.is_cuda or tuple(fields.shape) != (W, s.nchol):
        raise ValueError("fields must be a (W, G) float64 CUDA tensor")
    fields = fields.contiguous()
    st = _lib.TrotState()
    st.walkers_a, st.walkers_b = native.ptr(wa), native.ptr(wb)
    st.weights, st.overlaps = state.weights.data_ptr(), state.overlaps.data_ptr()
    st.scalars, st.node_encounters = state.scalars.data_ptr(), state.node_encounters.data_ptr()
    ws, nws = native.ws_for(s, _lib.OP_PROP_STEP)
    _lib.call("trot_prop_step", ctypes.byref(s), ctypes.byref(st), fields.data_ptr(), native.ptr(energy_out),
              ws, nws, native.stream_ptr())
    return state


def init_prop_state(*, sys: System, ham_data, trial_ops: TrialOps, trial_data, meas_ops: MeasOps, params,
                    initial_walkers=None, initial_e_estimate=None, rdm1=None, mesh=None) -> PropState:
    """trot/prop/afqmc.py:19-76 (``mesh`` is accepted and ignored: one GPU)."""
    from . import walkers as wk

    n_walkers = params.n_walkers
    dev = native_device()
    if initial_walkers is None:
        if rdm1 is None:
            rdm1 = trial_ops.get_rdm1(trial_data)
        initial_walkers = wk.init_walkers(sys=sys, rdm1=rdm1, n_walkers=n_walkers)
    overlaps = wk.vmap_chunked(meas_ops.overlap, n_chunks=params.n_chunks, in_axes=(0, None))(
        initial_walkers, trial_data)
    if initial_e_estimate is not None:
        e_est = float(np.real(np.asarray(initial_e_estimate.item() if isinstance(initial_e_estimate, torch.Tensor)
                                         else initial_e_estimate)))
    else:
        meas_ctx = meas_ops.build_meas_ctx(ham_data, trial_data)
        e_kernel = meas_ops.require_kernel(k_energy)
        w0 = wk.take_walkers(initial_walkers, slice(0, 1))
        e_est = float(torch.real(e_kernel(w0, ham_data, meas_ctx, trial_data)).mean().item())
    scalars = torch.tensor([e_est, e_est], dtype=torch.float64, device=dev)
    return PropState(
        walkers=initial_walkers,
        weights=torch.ones(n_walkers, dtype=torch.float64, device=dev),
        overlaps=overlaps,
        rng_key=rng.key(params.seed),
        scalars=scalars,
        node_encounters=torch.zeros(1, dtype=torch.int64, device=dev),
    )


def native_device():
    from .core import device

    return device()


def make_prop_ops(ham_basis: str, walker_kind: str, mixed_precision: bool = False) -> PropOps:
    """trot/prop/afqmc.py:147-180."""
    if ham_basis != "restricted":
        raise NotImplementedError(f"CUDA path: ham_basis {ham_basis}")
    wk = walker_kind.lower()
    if wk not in ("restricted", "unrestricted"):
        raise NotImplementedError(f"CUDA path: walker_kind {walker_kind}")
    precision = _lib.MIXED if mixed_precision else _lib.FP64

    def step(state: PropState, *, params, ham_data, trial_data, trial_ops, meas_ops, meas_ctx, prop_ctx,
             fields=None, energy_out=None) -> PropState:
        return afqmc_step(state, params=params, ham_data=ham_data, trial_data=trial_data, meas_ops=meas_ops,
                          prop_ctx=prop_ctx, meas_ctx=meas_ctx, walker_kind=wk, precision=precision,
                          fields=fields, energy_out=energy_out)

    def build_prop_ctx(ham_data, rdm1, params) -> CholAfqmcCtx:
        return _build_prop_ctx(ham_data, rdm1, params.dt, mixed_precision=mixed_precision)

    return PropOps(init_prop_state=init_prop_state, build_prop_ctx=build_prop_ctx, step=step)
