"""RHF / UHF measurement ops: force bias and local energy (trot/meas/rhf.py,
trot/meas/uhf.py), batched over walkers and computed by the CUDA library."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, native
from . import ctx as ctx_dev
from .core import HamChol, MeasOps, System, batched, k_energy, k_force_bias
from .trial import RhfTrial, UhfTrial, _make_overlap


@dataclass(frozen=True)
class RhfMeasCtx:
    """Half-rotated integrals (trot/meas/rhf.py:282-305): rot_h1 (n, N),
    rot_chol (G, n, N); rot_chol_flat is the (G, n*N) view."""

    rot_h1: torch.Tensor
    rot_chol: torch.Tensor
    memory_mode: str = "high"

    @property
    def rot_chol_flat(self) -> torch.Tensor:
        return self.rot_chol.reshape(self.rot_chol.shape[0], -1)

    def spin_arrays(self):
        return self.rot_h1, None, self.rot_chol, None


@dataclass(frozen=True)
class UhfMeasCtx:
    """trot/meas/uhf.py:277-316."""

    rot_h1_a: torch.Tensor
    rot_h1_b: torch.Tensor
    rot_chol_a: torch.Tensor
    rot_chol_b: torch.Tensor

    def spin_arrays(self):
        return self.rot_h1_a, self.rot_h1_b, self.rot_chol_a, self.rot_chol_b


def build_rhf_meas_ctx(ham_data: HamChol, trial_data: RhfTrial, memory_mode: str = "high") -> RhfMeasCtx:
    """One-time half rotation (trot/meas/rhf.py:308-319; host twin
    trot/runtime_layout.py:200-245), on the device (``trot_half_rotate``)."""
    if ham_data.basis != "restricted":
        raise ValueError("RHF MeasOps currently assumes HamChol.basis == 'restricted'.")
    rot_h1, rot_chol = ctx_dev.half_rotate(trial_data.mo_coeff, ham_data.h1, ham_data.chol)
    return RhfMeasCtx(rot_h1, rot_chol, memory_mode)


def build_uhf_meas_ctx(ham_data: HamChol, trial_data: UhfTrial) -> UhfMeasCtx:
    """trot/meas/uhf.py:318-336, on the device."""
    if ham_data.basis != "restricted":
        raise ValueError("UHF MeasOps currently assumes HamChol.basis == 'restricted'.")
    h1 = ctx_dev.real_dev(ham_data.h1, "h1")
    chol = ctx_dev.real_dev(ham_data.chol, "chol")
    ha, ra = ctx_dev.half_rotate(trial_data.mo_coeff_a, h1, chol)
    hb, rb = ctx_dev.half_rotate(trial_data.mo_coeff_b, h1, chol)
    return UhfMeasCtx(ha, hb, ra, rb)


def _h0(ham_data) -> float:
    h0 = ham_data.h0
    if isinstance(h0, torch.Tensor):
        h0 = h0.item()
    return float(np.real(np.asarray(h0)))


def force_bias_batched(walkers, ham_data, meas_ctx, trial_data, walker_kind, precision=_lib.FP64,
                       prop_ctx=None):
    kind = native.kind_of(trial_data, walker_kind)
    wa, wb = native.split_walkers(walkers, kind)
    W = wa.shape[0]
    ca, cb = trial_data.coeffs()
    native.check_walker_tensor(wa, ca.shape[0], ca.shape[1])
    if wb is not None:
        native.check_walker_tensor(wb, cb.shape[0], cb.shape[1], W)
    s = native.system(kind, W, trial_data, meas_ctx, None, precision=precision)
    G = s.nchol
    out = torch.empty((W, G), dtype=torch.complex128, device=wa.device)
    ws, nws = native.ws_for(s, _lib.OP_FORCE_BIAS)
    _lib.call("trot_force_bias", ctypes.byref(s), native.ptr(wa), native.ptr(wb), out.data_ptr(), ws, nws,
              native.stream_ptr())
    if precision == _lib.MIXED:
        native.raise_on_timeout(ws, "force bias")
    return out


def local_energy_batched(walkers, ham_data, meas_ctx, trial_data, walker_kind, precision=_lib.FP64,
                         prop_ctx=None):
    kind = native.kind_of(trial_data, walker_kind)
    wa, wb = native.split_walkers(walkers, kind)
    W = wa.shape[0]
    ca, cb = trial_data.coeffs()
    native.check_walker_tensor(wa, ca.shape[0], ca.shape[1])
    if wb is not None:
        native.check_walker_tensor(wb, cb.shape[0], cb.shape[1], W)
    s = native.system(kind, W, trial_data, meas_ctx, None, h0=_h0(ham_data), precision=precision)
    out = torch.empty(W, dtype=torch.complex128, device=wa.device)
    ws, nws = native.ws_for(s, _lib.OP_LOCAL_ENERGY)
    _lib.call("trot_local_energy", ctypes.byref(s), native.ptr(wa), native.ptr(wb), out.data_ptr(), ws, nws,
              native.stream_ptr())
    if precision == _lib.MIXED:
        # the sticky word also covers the asynchronous mixed steps issued before this call
        native.raise_on_timeout(ws, "local energy")
    return out


def _kernels(walker_kind, precision=_lib.FP64):
    @batched
    def force_bias(walkers, ham_data, meas_ctx, trial_data):
        return force_bias_batched(walkers, ham_data, meas_ctx, trial_data, walker_kind, precision)

    @batched
    def energy(walkers, ham_data, meas_ctx, trial_data):
        return local_energy_batched(walkers, ham_data, meas_ctx, trial_data, walker_kind, precision)

    return {k_force_bias: force_bias, k_energy: energy}


def make_rhf_meas_ops(sys: System, memory_mode: str = "high", mixed_precision: bool = False) -> MeasOps:
    """trot/meas/rhf.py:322-367.  ``memory_mode`` is accepted for signature
    compatibility: the CUDA exchange kernel always streams over Cholesky
    vectors, so "high" and "low" compute the same numbers.  With
    ``mixed_precision`` the force bias and local energy run on the tensor
    cores (exact-slice BF16 products, float-float epilogue)."""
    if memory_mode not in ("high", "low"):
        raise ValueError(f"Unsupported RHF measurement memory_mode: {memory_mode!r}")
    if sys.walker_kind not in ("restricted", "unrestricted"):
        raise NotImplementedError(f"CUDA path: walker_kind {sys.walker_kind}")
    ops = MeasOps(
        overlap=_make_overlap(sys.walker_kind),
        build_meas_ctx=lambda ham_data, trial_data: build_rhf_meas_ctx(ham_data, trial_data, memory_mode),
        kernels=_kernels(sys.walker_kind, _lib.MIXED if mixed_precision else _lib.FP64),
    )
    object.__setattr__(ops, "walker_kind", sys.walker_kind)
    return ops


def make_uhf_meas_ops(sys: System, mixed_precision: bool = False) -> MeasOps:
    """trot/meas/uhf.py:339-379 (``mixed_precision`` as in make_rhf_meas_ops)."""
    if sys.walker_kind != "unrestricted":
        raise NotImplementedError(f"CUDA path: UHF measurements with {sys.walker_kind} walkers")
    ops = MeasOps(
        overlap=_make_overlap(sys.walker_kind),
        build_meas_ctx=build_uhf_meas_ctx,
        kernels=_kernels(sys.walker_kind, _lib.MIXED if mixed_precision else _lib.FP64),
    )
    object.__setattr__(ops, "walker_kind", sys.walker_kind)
    return ops
