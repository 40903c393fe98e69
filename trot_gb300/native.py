"""Assemble ``trot_system`` / ``trot_state`` structs from the Python objects and
call the C ABI on torch's current CUDA stream."""
from __future__ import annotations

import ctypes

import torch

from . import _lib

_workspaces: dict = {}


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t) -> int:
    return 0 if t is None else t.data_ptr()


def workspace(nbytes: int) -> torch.Tensor:
    """A cached uint8 device buffer of at least ``nbytes``, one per (device,
    stream): calls on one stream are ordered and may share it, calls running
    concurrently on different streams (fragment batches) get their own.  The
    256-byte status block at the start of a new buffer is zero-filled, so its
    sticky timeout word starts clear (a buffer replaced by a larger one starts
    a new record)."""
    dev = torch.cuda.current_device()
    key = (dev, torch.cuda.current_stream().cuda_stream)
    buf = _workspaces.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=f"cuda:{dev}")
        buf[:256].zero_()
        _workspaces[key] = buf
    return buf


def capturing() -> bool:
    return torch.cuda.is_current_stream_capturing()


def raise_on_timeout(ws_ptr: int, what: str) -> None:
    """Read (and clear) the sticky timeout word of the workspace at ``ws_ptr``
    after the work queued on the current stream; raise TrotError(DEVICE_TIMEOUT)
    if a tensor-core kernel of any call that used it since the last check had
    a bounded wait run out (those calls wrote NaN results).  Synchronises the
    stream; a no-op under CUDA graph capture."""
    if capturing():
        return
    torch.cuda.current_stream().synchronize()
    st = ctypes.c_int(0)
    _lib.call("trot_workspace_timeouts", ws_ptr, 1, ctypes.addressof(st))
    if st.value != _lib.OK:
        raise _lib.TrotError(st.value, f"{what}: a tensor-core kernel's bounded wait ran out; its results are NaN")


def check_device_timeouts(what: str = "trot_gb300") -> None:
    """raise_on_timeout for every cached workspace of the current device (one
    check per block or per graph replay covers all the asynchronous steps
    before it)."""
    dev = torch.cuda.current_device()
    for (d, _), buf in list(_workspaces.items()):
        if d == dev:
            raise_on_timeout(buf.data_ptr(), what)


def kind_of(trial, walker_kind: str) -> int:
    from .trial import RhfTrial, UhfTrial

    wk = walker_kind.lower()
    if isinstance(trial, RhfTrial):
        if wk == "restricted":
            return _lib.RHF_R
        if wk == "unrestricted":
            return _lib.RHF_U
    elif isinstance(trial, UhfTrial):
        if wk == "unrestricted":
            return _lib.UHF_U
    raise NotImplementedError(f"CUDA path: trial {type(trial).__name__} with {walker_kind} walkers")


def split_walkers(walkers, kind):
    if kind == _lib.RHF_R:
        if isinstance(walkers, tuple):
            raise TypeError("restricted walkers must be one (W, N, n) tensor")
        return walkers, None
    if not isinstance(walkers, tuple) or len(walkers) != 2:
        raise TypeError("unrestricted walkers must be a (wu, wd) tuple")
    return walkers[0], walkers[1]


def check_walker_tensor(w, N, n, W=None):
    if w.dtype != torch.complex128:
        raise TypeError(f"walkers must be complex128, got {w.dtype}")
    if not w.is_cuda:
        raise TypeError("walkers must be CUDA tensors (no CPU fallback)")
    if not w.is_contiguous():
        raise ValueError("walkers must be contiguous")
    if w.dim() != 3 or w.shape[1] != N or w.shape[2] != n or (W is not None and w.shape[0] != W):
        raise ValueError(f"walker shape {tuple(w.shape)} != (W, {N}, {n})")


def system(kind, n_walkers, trial, meas_ctx=None, prop_ctx=None, h0=0.0, params=None,
           precision=_lib.FP64, mixed=None) -> _lib.TrotSystem:
    """Fill a trot_system for one call. Keeps no references: the caller's
    objects own the device buffers for the duration of the (stream-ordered) call."""
    s = _lib.TrotSystem()
    s.kind = kind
    s.precision = precision
    s.n_walkers = int(n_walkers)
    mo_a, mo_b = trial.coeffs()
    s.norb = int(mo_a.shape[0])
    s.nocc_a = int(mo_a.shape[1])
    s.nocc_b = int(mo_b.shape[1]) if kind != _lib.RHF_R else 0
    s.mo_a, s.mo_b = ptr(mo_a), ptr(mo_b if kind == _lib.UHF_U else None)
    s.h0 = float(h0)
    if meas_ctx is not None:
        ha, hb, ra, rb = meas_ctx.spin_arrays()
        s.rot_h1_a, s.rot_h1_b, s.rot_chol_a, s.rot_chol_b = ptr(ha), ptr(hb), ptr(ra), ptr(rb)
        s.nchol = int(ra.shape[0])
    if prop_ctx is not None:
        s.nchol = int(prop_ctx.chol_flat.shape[0])
        s.exp_h1_half = ptr(prop_ctx.exp_h1_half)
        s.chol_flat = ptr(prop_ctx.chol_flat)
        s.chol_packed = ptr(getattr(prop_ctx, "chol_packed", None))
        s.mf_shifts_im = ptr(prop_ctx.mf_shifts_im)
        s.h0_prop = float(prop_ctx.h0_prop)
        s.dt = float(prop_ctx.dt)
        s.sqrt_dt = float(prop_ctx.sqrt_dt)
    if precision == _lib.MIXED:
        if mixed is None:
            from . import mixed as _mixed

            mixed = _mixed.context(meas_ctx, prop_ctx)
        s.mixed = mixed.data_ptr()
    if params is not None:
        s.n_exp_terms = int(params.n_exp_terms)
        s.weight_floor = float(getattr(params, "weight_floor", 1.0e-3))
        s.weight_cap = float(getattr(params, "weight_cap", 100.0))
        s.pop_control_damping = float(getattr(params, "pop_control_damping", 0.1))
    else:
        s.n_exp_terms = 6
    return s


def ws_for(s: _lib.TrotSystem, op: int) -> tuple[int, int]:
    n = _lib.load().trot_workspace_size(ctypes.byref(s), op)
    if n == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    buf = workspace(n)
    return buf.data_ptr(), buf.numel()
