"""One AFQMC block (trot/prop/blocks.py:195-287): n_prop_steps phaseless
steps, QR, overlaps, local energy with the outlier clamp, EMA of e_estimate,
stochastic reconfiguration.  Every stage is a call into the CUDA library; the
block returns device scalars and synchronises with the host only if the
caller reads them."""
from __future__ import annotations

import ctypes
from typing import Any, Callable, NamedTuple

import torch

from . import _lib, native, rng
from . import walkers as wk
from .core import MeasOps, PropOps, PropState, System, TrialOps, k_energy


class BlockObs(NamedTuple):
    scalars: dict
    observables: dict


def block(state: PropState, *, sys: System, params, ham_data, trial_data, trial_ops: TrialOps,
          meas_ops: MeasOps, meas_ctx, prop_ops: PropOps, prop_ctx, sr_fn: Callable = wk.stochastic_reconfiguration,
          observable_names: tuple = (), fields_seq=None, zeta=None):
    """``fields_seq`` (n_prop_steps, W, G) and ``zeta`` inject the random numbers
    (tests); by default both are drawn on the device from ``state.rng_key``.
    ``observable_names``: "rdm1" (the weighted block average of the one-body
    RDM, complex128 (2, N, N); trot/prop/blocks.py:259-268)."""
    unknown = [o for o in observable_names if o != "rdm1"]
    if unknown:
        raise NotImplementedError(f"CUDA path: block observables {unknown} (supported: 'rdm1')")
    for k in range(params.n_prop_steps):
        state = prop_ops.step(state, params=params, ham_data=ham_data, trial_data=trial_data, trial_ops=trial_ops,
                              meas_ops=meas_ops, meas_ctx=meas_ctx, prop_ctx=prop_ctx,
                              fields=None if fields_seq is None else fields_seq[k])
    walkers = wk.orthonormalize_(state.walkers, sys.walker_kind)
    overlaps = wk.vmap_chunked(meas_ops.overlap, n_chunks=params.n_chunks, in_axes=(0, None))(walkers, trial_data)
    e_kernel = meas_ops.require_kernel(k_energy)
    e = wk.vmap_chunked(e_kernel, n_chunks=params.n_chunks, in_axes=(0, None, None, None))(
        walkers, ham_data, meas_ctx, trial_data)
    obs = torch.empty(2, dtype=torch.float64, device=state.weights.device)
    _lib.call("trot_block_energy", wk.n_walkers(walkers), e.data_ptr(), state.weights.data_ptr(),
              state.scalars.data_ptr(), float(params.dt), float(getattr(params, "shift_ema", 0.1)),
              obs.data_ptr(), native.stream_ptr())
    observables = {}
    if "rdm1" in observable_names:
        from .trial import half_green_batched

        green = half_green_batched(walkers, trial_data, sys.walker_kind)
        s = native.system(native.kind_of(trial_data, sys.walker_kind), wk.n_walkers(walkers), trial_data)
        N = green.shape[2]
        rdm1 = torch.empty((2, N, N), dtype=torch.complex128, device=green.device)
        nbytes = _lib.load().trot_workspace_size(ctypes.byref(s), _lib.OP_RDM1)
        ws = native.workspace(nbytes)
        _lib.call("trot_block_rdm1", ctypes.byref(s), green.data_ptr(), state.weights.data_ptr(), obs.data_ptr(),
                  rdm1.data_ptr(), ws.data_ptr(), ws.numel(), native.stream_ptr())
        observables["rdm1"] = rdm1
    if zeta is None:
        zeta = rng.uniform(state.rng_key, 1)
    w_sr, weights_sr = sr_fn(walkers, state.weights, zeta, sys.walker_kind)[:2]
    overlaps_sr = wk.vmap_chunked(meas_ops.overlap, n_chunks=params.n_chunks, in_axes=(0, None))(w_sr, trial_data)
    state = state._replace(walkers=w_sr, weights=weights_sr, overlaps=overlaps_sr)
    return state, BlockObs(scalars={"energy": obs[0], "weight": obs[1]}, observables=observables)
