"""Walker batch functions (trot/walkers.py) on the CUDA library.

Walkers are complex128 CUDA tensors: restricted (W, N, n), unrestricted a
(wu, wd) tuple."""
from __future__ import annotations

import ctypes
from typing import Any, Callable

import numpy as np
import torch

from . import _lib, native
from .core import System, as_dev


def is_unrestricted(w) -> bool:
    return isinstance(w, tuple) and len(w) == 2


def n_walkers(w) -> int:
    return int((w[0] if is_unrestricted(w) else w).shape[0])


def take_walkers(w, idx):
    if is_unrestricted(w):
        return (w[0][idx].contiguous(), w[1][idx].contiguous())
    return w[idx].contiguous()


def _natorbs(dm: np.ndarray, n_occ: int) -> np.ndarray:
    dm = 0.5 * (dm + np.conj(dm.T))
    return np.linalg.eigh(dm)[1][:, ::-1][:, :n_occ]


def init_walkers(sys: System, rdm1, n_walkers: int):
    """Natural orbitals of the trial density, broadcast to all walkers
    (trot/walkers.py:20-78; one-time host setup, eigenvector signs as LAPACK
    returns them)."""
    rd = rdm1.detach().cpu().numpy() if isinstance(rdm1, torch.Tensor) else np.asarray(rdm1)
    if rd.ndim != 3 or rd.shape[0] != 2:
        raise ValueError("Expected rdm1 with shape (2, norb, norb).")
    wk = sys.walker_kind
    if wk == "restricted":
        w0 = as_dev(_natorbs(rd[0] + rd[1], sys.nup) + 0.0j, torch.complex128)
        return w0.unsqueeze(0).expand(n_walkers, *w0.shape).contiguous()
    if wk == "unrestricted":
        wu = as_dev(_natorbs(rd[0], sys.nup) + 0.0j, torch.complex128)
        wd = as_dev(_natorbs(rd[1], sys.ndn) + 0.0j, torch.complex128)
        return (wu.unsqueeze(0).expand(n_walkers, *wu.shape).contiguous(),
                wd.unsqueeze(0).expand(n_walkers, *wd.shape).contiguous())
    raise NotImplementedError(f"CUDA path: walker_kind {wk}")


def vmap_chunked(fn: Callable, n_chunks: int, *, in_axes=0):
    """trot/walkers.py:94-134.  Batched kernels (``fn.batched``) are called on
    the whole batch, or on ``n_chunks`` contiguous slices whose results are
    concatenated (same numbers either way); other functions are mapped per
    walker."""

    def wrapped(*args, **kwargs):
        axes = in_axes if isinstance(in_axes, tuple) else (in_axes,) * len(args)
        mapped = [i for i, a in enumerate(axes) if a == 0]
        if not mapped:
            return fn(*args, **kwargs)
        nw = n_walkers(args[mapped[0]])
        if getattr(fn, "batched", False):
            if n_chunks <= 1:
                return fn(*args, **kwargs)
            bs = (nw + n_chunks - 1) // n_chunks
            outs = []
            for s in range(0, nw, bs):
                call = [take_walkers(a, slice(s, s + bs)) if i in mapped else a for i, a in enumerate(args)]
                outs.append(fn(*call, **kwargs))
            if isinstance(outs[0], tuple):
                return tuple(torch.cat([o[k] for o in outs]) for k in range(len(outs[0])))
            return torch.cat(outs)
        outs = []
        for b in range(nw):
            call = [take_walkers(a, b) if i in mapped else a for i, a in enumerate(args)]
            outs.append(fn(*call, **kwargs))
        if isinstance(outs[0], tuple):
            return tuple(torch.stack([o[k] for o in outs]) for k in range(len(outs[0])))
        return torch.stack(outs)

    return wrapped


def _qr_system(w, walker_kind):
    wk = walker_kind.lower()
    s = _lib.TrotSystem()
    if wk == "unrestricted":
        wa, wb = w
        s.kind, s.nocc_b = _lib.RHF_U if wa.shape[2] == wb.shape[2] else _lib.UHF_U, int(wb.shape[2])
    elif wk == "restricted":
        wa, wb = w, None
        s.kind = _lib.RHF_R
    else:
        raise NotImplementedError(f"CUDA path: walker_kind {walker_kind}")
    s.n_walkers, s.norb, s.nocc_a = int(wa.shape[0]), int(wa.shape[1]), int(wa.shape[2])
    native.check_walker_tensor(wa, s.norb, s.nocc_a)
    if wb is not None:
        native.check_walker_tensor(wb, s.norb, s.nocc_b, s.n_walkers)
    s.mo_a = s.mo_b = wa.data_ptr()  # not read by QR / SR; satisfies the struct check
    return s, wa, wb


def orthogonalize(w, walker_kind: str):
    """trot/walkers.py:151-171: returns (Q walkers, norm); the input is not modified."""
    w = tuple(x.clone() for x in w) if is_unrestricted(w) else w.clone()
    s, wa, wb = _qr_system(w, walker_kind)
    norm = torch.empty(s.n_walkers, dtype=torch.complex128, device=wa.device)
    _lib.call("trot_orthonormalize", ctypes.byref(s), wa.data_ptr(), native.ptr(wb), norm.data_ptr(),
              native.stream_ptr())
    return (wa, wb) if wb is not None else wa, norm


def orthonormalize(w, walker_kind: str):
    """trot/walkers.py:174-179."""
    return orthogonalize(w, walker_kind)[0]


def orthonormalize_(w, walker_kind: str):
    """In-place variant (no copy, no norm)."""
    s, wa, wb = _qr_system(w, walker_kind)
    _lib.call("trot_orthonormalize", ctypes.byref(s), wa.data_ptr(), native.ptr(wb), 0, native.stream_ptr())
    return w


def stochastic_reconfiguration(w, weights: torch.Tensor, zeta, walker_kind: str, *, data_sharding=None,
                               return_indices: bool = False):
    """trot/walkers.py:257-293 with a given zeta: a float, or a float64 CUDA
    tensor whose first element the kernel reads on the device (no host sync)."""
    zeta_dev = 0
    if isinstance(zeta, torch.Tensor):
        if not zeta.is_cuda or zeta.dtype != torch.float64:
            zeta = float(zeta.reshape(-1)[0].item())
        else:
            zeta_dev = zeta.data_ptr()
            zeta = 0.0
    s, wa, wb = _qr_system(w, walker_kind)
    if weights.dtype != torch.float64 or not weights.is_cuda or weights.shape[0] != s.n_walkers:
        raise ValueError("weights must be a (W,) float64 CUDA tensor")
    oa = torch.empty_like(wa)
    ob = torch.empty_like(wb) if wb is not None else None
    wout = torch.empty_like(weights)
    idx = torch.empty(s.n_walkers, dtype=torch.int64, device=wa.device)
    nbytes = _lib.load().trot_workspace_size(ctypes.byref(s), _lib.OP_SR)
    ws = native.workspace(nbytes)
    _lib.call("trot_sr_resample", ctypes.byref(s), weights.contiguous().data_ptr(), zeta_dev, float(zeta), wa.data_ptr(),
              native.ptr(wb), oa.data_ptr(), native.ptr(ob), wout.data_ptr(), idx.data_ptr(), ws.data_ptr(),
              ws.numel(), native.stream_ptr())
    out = ((oa, ob) if wb is not None else oa, wout)
    return out + (idx,) if return_indices else out


def no_sr(w, weights, zeta, walker_kind):
    return w, weights


def _sr_indices(weights, zeta, n_walkers):
    w = torch.zeros((n_walkers, 1, 1), dtype=torch.complex128, device=weights.device)
    return stochastic_reconfiguration(w, weights, zeta, "restricted", return_indices=True)[2]
