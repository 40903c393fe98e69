"""One-time constants built on the device by the CUDA library.

* ``prop_ctx``  — mf_shifts, h0_prop and exp(-dt/2 h1_eff) of the propagation
  context (trot/runtime_layout.py:125-197; trot/prop/chol_afqmc_ops.py:103-127),
  ``trot_build_prop_ctx``;
* ``half_rotate`` — rot_h1 = C^T h1 and rot_chol[g] = C^T L_g
  (trot/runtime_layout.py:200-245; trot/meas/rhf.py:308-319), ``trot_half_rotate``;
* ``cisd_lci1`` — lci1 of the CISD measurement context
  (trot/runtime_layout.py:248-292; trot/meas/cisd.py:92-110), ``trot_cisd_lci1``.

Inputs may be numpy arrays or torch tensors (host or device); they are moved to
the current CUDA device once, and every contraction runs in the library.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, native
from .core import device


def real_dev(x, name: str) -> torch.Tensor:
    """``x`` as a contiguous float64 tensor on the current device; complex input
    must have a zero imaginary part (checked on the device)."""
    t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.ascontiguousarray(x))
    t = t.to(device=device())
    if t.is_complex():
        if bool((t.imag != 0).any()):
            raise NotImplementedError(f"{name}: complex-valued input is not supported by the CUDA path")
        t = t.real
    return t.to(dtype=torch.float64).contiguous()


def _spin_summed(rdm1) -> torch.Tensor:
    rd = real_dev(rdm1, "rdm1")
    if rd.dim() == 3 and rd.shape[0] == 2:
        rd = (rd[0] + rd[1]).contiguous()
    if rd.dim() != 2 or rd.shape[0] != rd.shape[1]:
        raise ValueError(f"rdm1 shape {tuple(rd.shape)} is neither (N, N) nor (2, N, N)")
    return rd


def prop_ctx(h0: float, h1, chol, rdm1, dt: float):
    """Returns (mf_im (G,), h0_prop float, exp_h1_half (N, N), chol (G, N, N)),
    all but h0_prop device tensors; mf_shifts = i * mf_im."""
    h1 = real_dev(h1, "h1")
    chol = real_dev(chol, "chol")
    dm = _spin_summed(rdm1)
    G, N = int(chol.shape[0]), int(chol.shape[1])
    if tuple(chol.shape) != (G, N, N) or tuple(h1.shape) != (N, N) or tuple(dm.shape) != (N, N):
        raise ValueError(f"shapes h1 {tuple(h1.shape)}, chol {tuple(chol.shape)}, rdm1 {tuple(dm.shape)}")
    lib = _lib.load()
    nbytes = lib.trot_prop_ctx_workspace_size(N, G)
    if nbytes == 0:
        _lib.check(1)  # TROT_ERR_BAD_SHAPE, message from the library
    ws = torch.empty(nbytes, dtype=torch.uint8, device=chol.device)
    mf_im = torch.empty(G, dtype=torch.float64, device=chol.device)
    h0p = torch.empty(1, dtype=torch.float64, device=chol.device)
    eh = torch.empty((N, N), dtype=torch.float64, device=chol.device)
    _lib.call("trot_build_prop_ctx", N, G, float(h0), float(dt), h1.data_ptr(), chol.data_ptr(), dm.data_ptr(),
              mf_im.data_ptr(), h0p.data_ptr(), eh.data_ptr(), ws.data_ptr(), nbytes, native.stream_ptr())
    torch.cuda.current_stream().synchronize()
    st = ctypes.c_int(0)
    _lib.call("trot_workspace_status", ws.data_ptr(), ctypes.addressof(st))
    if st.value != _lib.OK:
        raise _lib.TrotError(st.value, "propagation context: h1_eff has a non-finite entry or "
                                       "dt/2 ||h1_eff||_1 > 2^39")
    return mf_im, float(h0p.item()), eh, chol


def half_rotate(mo, h1, chol):
    """rot_h1 (n, N) and rot_chol (G, n, N) for a real trial ``mo`` (N, n)."""
    mo = real_dev(mo, "mo_coeff")
    h1 = real_dev(h1, "h1")
    chol = real_dev(chol, "chol")
    N, n = int(mo.shape[0]), int(mo.shape[1])
    G = int(chol.shape[0])
    if tuple(h1.shape) != (N, N) or tuple(chol.shape) != (G, N, N):
        raise ValueError(f"shapes mo {tuple(mo.shape)}, h1 {tuple(h1.shape)}, chol {tuple(chol.shape)}")
    rot_h1 = torch.empty((n, N), dtype=torch.float64, device=mo.device)
    rot_chol = torch.empty((G, n, N), dtype=torch.float64, device=mo.device)
    _lib.call("trot_half_rotate", N, G, n, mo.data_ptr(), h1.data_ptr(), chol.data_ptr(), rot_h1.data_ptr(),
              rot_chol.data_ptr(), native.stream_ptr())
    return rot_h1, rot_chol


def cisd_lci1(ci1, chol) -> torch.Tensor:
    """lci1 (G, N, nocc) from ci1 (nocc, N - nocc) and chol (G, N, N)."""
    ci1 = real_dev(ci1, "ci1")
    chol = real_dev(chol, "chol")
    n, v = int(ci1.shape[0]), int(ci1.shape[1])
    G, N = int(chol.shape[0]), int(chol.shape[1])
    if n + v != N or tuple(chol.shape) != (G, N, N):
        raise ValueError(f"shapes ci1 {tuple(ci1.shape)}, chol {tuple(chol.shape)}")
    lci1 = torch.empty((G, N, n), dtype=torch.float64, device=chol.device)
    _lib.call("trot_cisd_lci1", N, G, n, ci1.data_ptr(), chol.data_ptr(), lci1.data_ptr(), native.stream_ptr())
    return lci1
