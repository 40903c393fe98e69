"""Operands of the mixed-precision (tensor-core) path.

Built once per (trial, Hamiltonian, dt) on the host and kept on the device:

* exact-digit FP16 copies of the half-rotated Cholesky vectors for the local
  energy / force bias: each row (g, i) over orbitals p is written as
  2^e (q_0 2^-9 + sum_{t=1..4} q_t 2^-(9 + 9 t)) with integer digits
  |q_0| <= 512, |q_t| <= 256 (exact in FP16) and one exponent per row, laid
  out as 128-row tiles of whole Cholesky vectors; a row whose top digits sum
  (in absolute value) past 2^15 gets its exponent raised by one, which keeps
  every partial sum of the two leading digit-product groups below 2^24 (exact
  in the tensor core's FP32 accumulator) against Green's-function digits with
  |q_0| <= 256, |q_t| <= 256;
* a 3-term BF16 split (hi + mid + lo) of the Cholesky vectors, transposed to
  (N*N, G) and stored as the VHS kernel's shared-memory image (128 x 64
  tiles in core-matrix order);
* exp(-dt/2 h1_eff) in FP32 for the one-body half steps.

``context(meas_ctx, prop_ctx, kind)`` returns the cached ``MixedCtx`` whose
``data_ptr()`` is the address of the ``trot_mixed`` struct the C ABI reads.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .core import device

SLICES = 5
MAX_ORDER = 4
KPAD = 128
VHS_SLICES = 3
VHS_ORDER = 2
# digit format of the exact product (trot_mixed.digit_format): FP16 digits, Cholesky
# rows with a 9-bit leading digit, Green's-function rows (made on the device) with an
# 8-bit leading digit, 9-bit lower digits for both
DIGIT_FORMAT = 2
ROT_TOP_BITS = 9
GREEN_TOP_BITS = 8
LOW_BITS = 9
ROT_L1_CAP = 2 ** 15


def digit_slices(x: np.ndarray, slices: int = SLICES, top: int = ROT_TOP_BITS, low: int = LOW_BITS,
                 l1_cap: float | None = ROT_L1_CAP):
    """Exact integer digits of the rows (last axis) of ``x``: returns (q (slices,
    ...) float32 integers, e int32 row exponents) with
    x ~= 2^e sum_t q_t 2^-(top + low t), |q_0| <= 2^top and balanced lower digits
    |q_t| <= 2^(low - 1); the representation error is at most 2^(e - top - low
    (slices - 1) - 1) per element.  e is the smallest integer with max |x| <= 2^e,
    raised by one for rows whose sum of |q_0| would exceed ``l1_cap``."""
    x = np.asarray(x, dtype=np.float64)
    mx = np.max(np.abs(x), axis=-1)
    e = np.where(mx > 0, np.ceil(np.log2(np.where(mx > 0, mx, 1.0))), 0.0).astype(np.int32)
    if l1_cap is not None:
        q0 = np.rint(x / np.ldexp(1.0, e - top)[..., None])
        e = e + (np.sum(np.abs(q0), axis=-1) > l1_cap).astype(np.int32)
    r = x.copy()
    out = []
    for t in range(slices):
        sc = np.ldexp(1.0, e - top - low * t)[..., None]
        q = np.rint(r / sc)
        out.append(q.astype(np.float32))
        r = r - q * sc
    return np.stack(out), e


def plain_split(x: np.ndarray, slices: int = VHS_SLICES) -> list[torch.Tensor]:
    """x ~= sum of bf16 terms, each the round-to-nearest bf16 of the remainder."""
    r = torch.as_tensor(np.asarray(x, dtype=np.float64))
    out = []
    for _ in range(slices):
        h = r.to(torch.float32).to(torch.bfloat16)
        out.append(h)
        r = r - h.to(torch.float64)
    return out


def split3_image(bt: np.ndarray, kchunk: int = 64):
    """Operand image of a real matrix B (K, ncols) for the split-BF16 tensor-core
    kernels, given its transpose bt (ncols, K): rows padded to a multiple of
    128, K to a multiple of kchunk, split into 3 BF16 terms and laid out as
    [ncols/128][K/kchunk][3][128][kchunk] tiles in core-matrix order (8 x 8
    blocks).  Returns (image (bf16, host), ncols_pad, k_pad)."""
    bt = np.asarray(bt, dtype=np.float64)
    nc, K = bt.shape
    npad, kpad = (nc + 127) // 128 * 128, (K + kchunk - 1) // kchunk * kchunk
    lt = np.zeros((npad, kpad), dtype=np.float64)
    lt[:nc, :K] = bt
    sl = torch.stack(plain_split(lt))  # (3, npad, kpad)
    nt, nk = npad // 128, kpad // kchunk
    sl = sl.reshape(3, nt, 16, 8, nk, kchunk // 8, 8).permute(1, 4, 0, 2, 5, 3, 6).contiguous()
    return sl.reshape(nt, nk, 3, 128, kchunk).contiguous(), npad, kpad


def vhs_operand(chol_flat):
    """B^T of the VHS product VHS = x chol_flat: (N^2, G) rows pq, or, when every Cholesky
    matrix is symmetric to working precision (Cholesky vectors of real integrals are), the
    packed upper triangle (N (N + 1) / 2, G) of (L + L^T) / 2 in row-major p <= q order, so
    that only the upper triangle of the symmetric VHS is computed.  Returns (bt, packed)."""
    cf = np.asarray(chol_flat, dtype=np.float64)
    G, N = cf.shape[0], int(round(np.sqrt(cf.shape[1])))
    L = cf.reshape(G, N, N)
    amax = float(np.abs(L).max()) if L.size else 0.0
    packed = L.size > 0 and float(np.abs(L - L.transpose(0, 2, 1)).max()) <= 1e-12 * amax
    if not packed:
        return cf.T, False
    iu, ju = np.triu_indices(N)
    return (0.5 * (L[:, iu, ju] + L[:, ju, iu])).T, True


def packed_index(p: int, q: int, N: int) -> int:
    """Column of V[p][q] in the packed upper triangle (the kernels' vhs_col)."""
    if p > q:
        p, q = q, p
    return p * N - p * (p - 1) // 2 + (q - p)


def gammas_per_block(n: int) -> int:
    return max(1, 128 // n)


def rot_tiles(rot_chol: np.ndarray):
    """(G, n, N) -> FP16 digits in the exchange kernel's shared-memory image
    layout (nblk, KSTEPS, SLICES, 128, 16): per 128-row tile of whole Cholesky
    vectors, per K16 step, per digit plane a 128 x 16 block in 8 x 8 core-matrix
    order (K fastest; core matrices 128 B apart along K, 256 B apart along rows),
    so one K16 step of all planes is one contiguous 20 KB chunk; and the row
    exponents (nblk, 128)."""
    G, n, N = rot_chol.shape
    if n > 16 or N > KPAD:
        raise NotImplementedError(f"mixed path: n={n}, N={N} outside the tensor-core tile limits (n<=16, N<={KPAD})")
    gb = gammas_per_block(n)
    nblk = (G + gb - 1) // gb
    rows = np.zeros((nblk, 128, KPAD), dtype=np.float64)
    for blk in range(nblk):
        g0, g1 = blk * gb, min(G, (blk + 1) * gb)
        r = rot_chol[g0:g1].reshape(-1, N)
        rows[blk, : r.shape[0], :N] = r
    q, e = digit_slices(rows)  # (SLICES, nblk, 128, KPAD)
    ks = KPAD // 16
    # (plane, blk, row group, row, kstep, k group, k) -> (blk, kstep, plane, row group, k group, row, k)
    img = q.reshape(SLICES, nblk, 16, 8, ks, 2, 8).transpose(1, 4, 0, 2, 5, 3, 6)
    img = np.ascontiguousarray(img).reshape(nblk, ks, SLICES, 128, 16)
    return torch.from_numpy(img.astype(np.float16)), torch.from_numpy(e.astype(np.int32)), gb, nblk


class MixedCtx:
    """Device operands + the host ``trot_mixed`` struct pointing at them."""

    def __init__(self, rot_a, rot_b, chol_flat=None, exp_h1_half=None):
        dev = device()
        s = _lib.TrotMixed()
        s.slices, s.max_order, s.kpad = SLICES, MAX_ORDER, KPAD
        s.digit_format = DIGIT_FORMAT
        self._keep = []
        for k, rc in enumerate((rot_a, rot_b)):
            if rc is None:
                continue
            q, e, gb, nblk = rot_tiles(rc)
            q, e = q.to(dev), e.to(dev)
            self._keep += [q, e]
            s.gammas_per_block[k], s.n_blocks[k] = gb, nblk
            s.rot_slices[k], s.rot_exp[k] = q.data_ptr(), e.data_ptr()
        self.struct = s
        if chol_flat is None:
            return
        bt, packed = vhs_operand(chol_flat)
        sl, n2pad, gpad = split3_image(bt)
        sl = sl.to(dev)
        self._keep.append(sl)
        s.vhs_slices, s.vhs_order, s.n2pad, s.gpad = VHS_SLICES, VHS_ORDER, n2pad, gpad
        s.vhs_packed = 1 if packed else 0
        s.chol_t_slices = sl.data_ptr()
        eh = torch.as_tensor(np.asarray(exp_h1_half, dtype=np.float32)).to(dev).contiguous()
        self._keep.append(eh)
        s.exp_h1_half_f32 = eh.data_ptr()
        E = np.asarray(exp_h1_half, dtype=np.float64)
        if E.shape[0] <= 128:
            E128 = np.zeros((128, 128))  # the kernel reads K = 128 (two 64-wide chunks) for every N
            E128[: E.shape[0], : E.shape[1]] = E
            ei, _, kp = split3_image(E128, kchunk=32)  # A operand rows p, K = q: (1, 4, 3, 128, 32)
            assert tuple(ei.shape) == (1, 4, 3, 128, 32) and kp == 128
            ei = ei.to(dev)
            self._keep.append(ei)
            s.exp_h1_half_img = ei.data_ptr()
        self.struct = s

    def data_ptr(self) -> int:
        return ctypes.addressof(self.struct)


def context(meas_ctx=None, prop_ctx=None) -> MixedCtx:
    """Mixed operands for this (meas_ctx, prop_ctx) pair (either may be None),
    built on first use and cached on the context object."""
    owner = meas_ctx if meas_ctx is not None else prop_ctx
    cache = owner.__dict__.setdefault("_mixed_cache", {})
    key = id(prop_ctx) if meas_ctx is not None else None
    hit = cache.get(key)
    if hit is not None and hit[0] is prop_ctx:
        return hit[1]
    ra = rb = None
    if meas_ctx is not None:
        _, _, ra, rb = meas_ctx.spin_arrays()
        ra = ra.cpu().numpy()
        rb = None if rb is None else rb.cpu().numpy()
    cf = eh = None
    if prop_ctx is not None:
        cf, eh = prop_ctx.chol_flat.cpu().numpy(), prop_ctx.exp_h1_half.cpu().numpy()
    m = MixedCtx(ra, rb, cf, eh)
    cache[key] = (prop_ctx, m)
    return m
