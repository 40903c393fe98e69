"""RHF / UHF trial wave functions (trot/trial/rhf.py, trot/trial/uhf.py).

``overlap`` takes the whole walker batch and returns (W,) complex128 overlaps
computed by the CUDA library (LU determinant of C^T w per walker)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _lib, native
from .core import System, TrialOps, as_dev, batched, real_part


@dataclass(frozen=True)
class RhfTrial:
    """trot/trial/rhf.py:13-36; mo_coeff (N, n) real float64 on the device."""

    mo_coeff: torch.Tensor

    def __post_init__(self):
        object.__setattr__(self, "mo_coeff", as_dev(real_part(self.mo_coeff, "mo_coeff")))

    @property
    def norb(self) -> int:
        return int(self.mo_coeff.shape[0])

    @property
    def nocc(self) -> int:
        return int(self.mo_coeff.shape[1])

    def coeffs(self):
        return self.mo_coeff, self.mo_coeff


@dataclass(frozen=True)
class UhfTrial:
    """trot/trial/uhf.py:15-37."""

    mo_coeff_a: torch.Tensor
    mo_coeff_b: torch.Tensor

    def __post_init__(self):
        object.__setattr__(self, "mo_coeff_a", as_dev(real_part(self.mo_coeff_a, "mo_coeff_a")))
        object.__setattr__(self, "mo_coeff_b", as_dev(real_part(self.mo_coeff_b, "mo_coeff_b")))

    @property
    def norb(self) -> int:
        return int(self.mo_coeff_a.shape[0])

    @property
    def nocc(self) -> tuple[int, int]:
        return int(self.mo_coeff_a.shape[1]), int(self.mo_coeff_b.shape[1])

    def coeffs(self):
        return self.mo_coeff_a, self.mo_coeff_b


def get_rdm1(trial_data) -> torch.Tensor:
    """Trial 1-RDM spin blocks (2, N, N) (trot/trial/rhf.py:39-42, trot/trial/uhf.py:40-45)."""
    ca, cb = trial_data.coeffs()
    return torch.stack([ca @ ca.T, cb @ cb.T])


def overlap_batched(walkers, trial_data, walker_kind: str) -> torch.Tensor:
    kind = native.kind_of(trial_data, walker_kind)
    wa, wb = native.split_walkers(walkers, kind)
    ca, cb = trial_data.coeffs()
    W = wa.shape[0]
    native.check_walker_tensor(wa, ca.shape[0], ca.shape[1])
    if wb is not None:
        native.check_walker_tensor(wb, cb.shape[0], cb.shape[1], W)
    out = torch.empty(W, dtype=torch.complex128, device=wa.device)
    s = native.system(kind, W, trial_data)
    _lib.call("trot_overlap", ctypes.byref(s), native.ptr(wa), native.ptr(wb), out.data_ptr(),
              native.stream_ptr())
    return out


def half_green_batched(walkers, trial_data, walker_kind: str, with_overlaps: bool = False):
    """Half-rotated Green's functions (W, nocc_a [+ nocc_b], N) of a walker batch,
    ``_half_green_from_overlap_matrix`` (trot/meas/rhf.py:21-25) per spin; with
    ``with_overlaps`` also the trial overlaps (W)."""
    kind = native.kind_of(trial_data, walker_kind)
    wa, wb = native.split_walkers(walkers, kind)
    ca, cb = trial_data.coeffs()
    W, N = wa.shape[0], ca.shape[0]
    native.check_walker_tensor(wa, ca.shape[0], ca.shape[1])
    rows = ca.shape[1]
    if wb is not None:
        native.check_walker_tensor(wb, cb.shape[0], cb.shape[1], W)
        rows += cb.shape[1]
    green = torch.empty((W, rows, N), dtype=torch.complex128, device=wa.device)
    ov = torch.empty(W, dtype=torch.complex128, device=wa.device) if with_overlaps else None
    s = native.system(kind, W, trial_data)
    _lib.call("trot_half_green", ctypes.byref(s), native.ptr(wa), native.ptr(wb), green.data_ptr(),
              native.ptr(ov), native.stream_ptr())
    return (green, ov) if with_overlaps else green


def _make_overlap(walker_kind: str):
    @batched
    def overlap(walkers, trial_data):
        return overlap_batched(walkers, trial_data, walker_kind)

    return overlap


def make_rhf_trial_ops(sys: System) -> TrialOps:
    """trot/trial/rhf.py:66-87."""
    if sys.nup != sys.ndn:
        raise ValueError("RHF requires nelec[0] == nelec[1].")
    if sys.walker_kind not in ("restricted", "unrestricted"):
        raise NotImplementedError(f"CUDA path: walker_kind {sys.walker_kind}")
    return TrialOps(overlap=_make_overlap(sys.walker_kind), get_rdm1=get_rdm1)


def make_uhf_trial_ops(sys: System) -> TrialOps:
    """trot/trial/uhf.py:61-80."""
    if sys.walker_kind != "unrestricted":
        raise NotImplementedError(f"CUDA path: UHF trial with {sys.walker_kind} walkers")
    return TrialOps(overlap=_make_overlap(sys.walker_kind), get_rdm1=get_rdm1)


def make_rhf_trial_data(data: dict, sys: System) -> RhfTrial:
    return RhfTrial(real_part(data["mo"], "mo")[:, : sys.nup])


def make_uhf_trial_data(data: dict, sys: System) -> UhfTrial:
    if "mo_a" in data and "mo_b" in data:
        a, b = data["mo_a"], data["mo_b"]
    elif "mo" in data:
        a = b = data["mo"]
    else:
        raise KeyError("Failed to find the trial coeff.")
    return UhfTrial(real_part(a, "mo_a")[:, : sys.nup], real_part(b, "mo_b")[:, : sys.ndn])
