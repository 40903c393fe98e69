"""Energy gradients through a phaseless AFQMC run: the hand-written adjoint.

The objective is the weighted mixed energy of a run without stochastic
reconfiguration (SR breaks differentiability by index selection)::

    J(h1) = sum_b sum_w wt_bw E~_bw / sum_b sum_w wt_bw

over blocks b of ``steps_per_block`` phaseless steps (trot/prop/afqmc.py:79-144)
each followed by the block tail of trot/prop/blocks.py:228-263: QR
orthonormalisation, overlaps, local energies E_bw, the clamp
|E - e_estimate| > sqrt(2/dt) -> e_estimate (E~), the block energy and the
e_estimate update with ``shift_ema``.  h1 enters through exp(-dt/2 h1_eff) in
every step and through rot_h1 = C^T h1 in the local energy.

Every operator is a ``torch.autograd.Function`` whose forward is the CUDA
library's forward and whose backward is its hand-written vector-Jacobian
product (``trot_prop_step_vjp``, ``trot_local_energy_vjp``,
``trot_overlap_vjp``, ``trot_orthonormalize_vjp``, ``trot_prop_ctx_vjp``);
torch's autograd only chains them and the O(W) block scalars.  Each block runs
under ``torch.utils.checkpoint``: its walkers are kept at the block start and
the block is recomputed during the backward pass, so memory is one block of
states, not the whole run.

Kinds: RHF trial with restricted walkers, RHF or UHF trial with unrestricted
walkers (a (wa, wb) tuple); FP64.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Any

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import _lib, native
from . import ctx as ctx_dev
from .prop import pack_symmetric
from .core import QmcParams
from .trial import RhfTrial, UhfTrial


def _cdev(x) -> torch.Tensor:
    t = x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))
    return t.to(device="cuda", dtype=torch.complex128).contiguous()


@dataclass
class AdjointProblem:
    """Everything but h1: h0, chol (G, N, N), the trial (RhfTrial or UhfTrial),
    the walker kind, the trial 1-RDM used for the mean-field shifts, the run
    parameters, the fields of every step (T, W, G), the initial walkers ((W, N, n)
    or a (wa, wb) tuple) and e_estimate."""

    h0: float
    chol: torch.Tensor
    trial: Any
    rdm1: torch.Tensor
    params: QmcParams
    fields: torch.Tensor
    walkers0: Any
    e_estimate0: float
    steps_per_block: int
    weights0: torch.Tensor | None = None
    walker_kind: str = "restricted"

    def __post_init__(self):
        self.chol = ctx_dev.real_dev(self.chol, "chol")
        self.fields = ctx_dev.real_dev(self.fields, "fields")
        uhf = isinstance(self.trial, UhfTrial)
        self.unrestricted = self.walker_kind == "unrestricted" or uhf
        if uhf and self.walker_kind != "unrestricted":
            raise ValueError("a UHF trial needs unrestricted walkers")
        self.kind = _lib.UHF_U if uhf else (_lib.RHF_U if self.unrestricted else _lib.RHF_R)
        mo_a, mo_b = self.trial.coeffs()
        self.mo = (mo_a, mo_b)
        if self.unrestricted:
            if not isinstance(self.walkers0, tuple) or len(self.walkers0) != 2:
                raise TypeError("unrestricted walkers0 must be a (wa, wb) tuple")
            self.walkers0 = (_cdev(self.walkers0[0]), _cdev(self.walkers0[1]))
        else:
            self.walkers0 = _cdev(self.walkers0)
        T, W, G = self.fields.shape
        if T % self.steps_per_block:
            raise ValueError(f"{T} steps are not a whole number of blocks of {self.steps_per_block}")
        ws = self.walkers0 if self.unrestricted else (self.walkers0,)
        for w, mo in zip(ws, self.mo):
            if tuple(w.shape[1:]) != tuple(mo.shape) or W != w.shape[0]:
                raise ValueError("walkers0 must be (W, N, n) per spin, matching the trial and the fields")
        N = int(self.chol.shape[1])
        self.n_walkers, self.norb, self.nchol = W, N, G
        self.rot_chol = []
        for mo in (self.mo if uhf else self.mo[:1]):
            n = int(mo.shape[1])
            r = torch.empty((G, n, N), dtype=torch.float64, device=self.chol.device)
            _lib.call("trot_half_rotate", N, G, n, mo.data_ptr(), 0, self.chol.data_ptr(), 0, r.data_ptr(),
                      native.stream_ptr())
            self.rot_chol.append(r)
        # h1-independent propagation constants (mean-field shifts, h0_prop)
        zero = torch.zeros((N, N), dtype=torch.float64, device=self.chol.device)
        mf_im, h0p, _, _ = ctx_dev.prop_ctx(self.h0, zero, self.chol, self.rdm1, self.params.dt)
        self.mf_im, self.h0_prop = mf_im, h0p
        self.chol_flat = self.chol.reshape(G, N * N)
        self.chol_packed = pack_symmetric(self.chol)

    def system(self, exp_h1_half=None, rot_h1=(None, None)) -> _lib.TrotSystem:
        s = _lib.TrotSystem()
        s.kind, s.precision = self.kind, _lib.FP64
        s.n_walkers, s.norb, s.nchol = self.n_walkers, self.norb, self.nchol
        s.nocc_a = int(self.mo[0].shape[1])
        s.nocc_b = int(self.mo[1].shape[1]) if self.unrestricted else 0
        p = self.params
        s.n_exp_terms = int(p.n_exp_terms)
        s.h0, s.h0_prop, s.dt, s.sqrt_dt = float(self.h0), float(self.h0_prop), float(p.dt), math.sqrt(p.dt)
        s.weight_floor, s.weight_cap = float(p.weight_floor), float(p.weight_cap)
        s.pop_control_damping = float(p.pop_control_damping)
        s.mo_a = self.mo[0].data_ptr()
        s.mo_b = self.mo[1].data_ptr() if self.kind == _lib.UHF_U else 0
        s.rot_chol_a = self.rot_chol[0].data_ptr()
        s.rot_chol_b = self.rot_chol[1].data_ptr() if self.kind == _lib.UHF_U else 0
        s.rot_h1_a = native.ptr(rot_h1[0])
        s.rot_h1_b = native.ptr(rot_h1[1]) if self.kind == _lib.UHF_U else 0
        s.exp_h1_half = native.ptr(exp_h1_half)
        s.chol_flat = self.chol_flat.data_ptr()
        s.chol_packed = native.ptr(self.chol_packed)
        s.mf_shifts_im = self.mf_im.data_ptr()
        return s


def _ptr(t) -> int:
    return 0 if t is None or t.numel() == 0 else t.data_ptr()


def _ws(nbytes: int) -> torch.Tensor:
    if nbytes == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    return torch.empty(nbytes, dtype=torch.uint8, device="cuda")


def _vjp_ws(s, op) -> torch.Tensor:
    return _ws(_lib.load().trot_vjp_workspace_size(ctypes.byref(s), op))


def _empty(like: torch.Tensor) -> torch.Tensor:
    return torch.empty(0, dtype=like.dtype, device=like.device)


def _grad_or_zero(g, like):
    if like.numel() == 0:
        return _empty(like)
    return torch.zeros_like(like) if g is None else g.contiguous()


class ExpH1Half(torch.autograd.Function):
    """exp(-dt/2 h1_eff(h1)) (trot_build_prop_ctx); backward trot_prop_ctx_vjp."""

    @staticmethod
    def forward(ctx, h1, prob: AdjointProblem):
        _, _, eh, _ = ctx_dev.prop_ctx(prob.h0, h1.detach(), prob.chol, prob.rdm1, prob.params.dt)
        ctx.save_for_backward(h1)
        ctx.prob = prob
        return eh

    @staticmethod
    def backward(ctx, g):
        (h1,) = ctx.saved_tensors
        prob = ctx.prob
        N, G = prob.norb, prob.nchol
        rd = ctx_dev._spin_summed(prob.rdm1)
        gh1 = torch.zeros((N, N), dtype=torch.float64, device=h1.device)
        ws = _ws(_lib.load().trot_prop_ctx_vjp_workspace_size(N, G))
        g = g.contiguous()
        _lib.call("trot_prop_ctx_vjp", N, G, float(prob.params.dt), h1.detach().contiguous().data_ptr(),
                  prob.chol.data_ptr(), rd.data_ptr(), g.data_ptr(), gh1.data_ptr(), ws.data_ptr(), ws.numel(),
                  native.stream_ptr())
        return gh1, None


class Step(torch.autograd.Function):
    """One phaseless step (trot_prop_step, FP64); backward trot_prop_step_vjp.
    wb is an empty tensor for restricted walkers."""

    @staticmethod
    def forward(ctx, wa, wb, wt, ov, scal, eh, x, prob: AdjointProblem):
        s = prob.system(exp_h1_half=eh)
        st = _lib.TrotState()
        woa, wob = wa.clone(), wb.clone()
        wto, ovo, sco = wt.clone(), ov.clone(), scal.clone()
        nodes = torch.zeros(1, dtype=torch.int64, device=wa.device)
        st.walkers_a, st.walkers_b = woa.data_ptr(), _ptr(wob)
        st.weights, st.overlaps, st.scalars = wto.data_ptr(), ovo.data_ptr(), sco.data_ptr()
        st.node_encounters = nodes.data_ptr()
        wsp, wsn = native.ws_for(s, _lib.OP_PROP_STEP)
        _lib.call("trot_prop_step", ctypes.byref(s), ctypes.byref(st), x.data_ptr(), None, wsp, wsn,
                  native.stream_ptr())
        ctx.save_for_backward(wa, wb, wt, ov, scal, eh, x)
        ctx.prob = prob
        return woa, wob, wto, ovo, sco

    @staticmethod
    def backward(ctx, gwa, gwb, gwt, gov, gsc):
        wa, wb, wt, ov, scal, eh, x = ctx.saved_tensors
        prob = ctx.prob
        s = prob.system(exp_h1_half=eh)
        st = _lib.TrotState()
        st.walkers_a, st.walkers_b = wa.data_ptr(), _ptr(wb)
        st.weights, st.overlaps, st.scalars = wt.data_ptr(), ov.data_ptr(), scal.data_ptr()
        gwa = _grad_or_zero(gwa, wa)
        gwb = _grad_or_zero(gwb, wb)
        gsc = torch.zeros_like(scal) if gsc is None else gsc.contiguous()
        gwt = None if gwt is None else gwt.contiguous()
        gov = None if gov is None else gov.contiguous()
        gwa_in, gwb_in = torch.empty_like(wa), torch.empty_like(wb)
        gwt_in, gov_in, gsc_in = torch.empty_like(wt), torch.empty_like(ov), torch.empty_like(scal)
        geh = torch.zeros_like(eh)
        ws = _vjp_ws(s, _lib.OP_PROP_STEP)
        _lib.call("trot_prop_step_vjp", ctypes.byref(s), ctypes.byref(st), x.data_ptr(), gwa.data_ptr(), _ptr(gwb),
                  native.ptr(gwt), native.ptr(gov), gsc.data_ptr(), gwa_in.data_ptr(), _ptr(gwb_in),
                  gwt_in.data_ptr(), gov_in.data_ptr(), gsc_in.data_ptr(), geh.data_ptr(), ws.data_ptr(), ws.numel(),
                  native.stream_ptr())
        return gwa_in, gwb_in, gwt_in, gov_in, gsc_in, geh, None, None


class Orthonormalize(torch.autograd.Function):
    """QR per spin with the phase convention of trot/walkers.py:137-148; backward g_q (w^H q)^-1."""

    @staticmethod
    def forward(ctx, wa, wb, prob: AdjointProblem):
        from .walkers import orthonormalize

        if prob.unrestricted:
            qa, qb = orthonormalize((wa, wb), "unrestricted")
        else:
            qa, qb = orthonormalize(wa, "restricted"), _empty(wa)
        ctx.save_for_backward(wa, wb, qa, qb)
        ctx.prob = prob
        return qa, qb

    @staticmethod
    def backward(ctx, gqa, gqb):
        wa, wb, qa, qb = ctx.saved_tensors
        s = ctx.prob.system()
        gqa, gqb = _grad_or_zero(gqa, qa), _grad_or_zero(gqb, qb)
        gwa, gwb = torch.empty_like(wa), torch.empty_like(wb)
        _lib.call("trot_orthonormalize_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), qa.data_ptr(), _ptr(qb),
                  gqa.data_ptr(), _ptr(gqb), gwa.data_ptr(), _ptr(gwb), native.stream_ptr())
        return gwa, gwb, None


class Overlap(torch.autograd.Function):
    """prod_s det(C_s^T w_s)^mult_s (trot_overlap); backward trot_overlap_vjp."""

    @staticmethod
    def forward(ctx, wa, wb, prob: AdjointProblem):
        s = prob.system()
        out = torch.empty(wa.shape[0], dtype=torch.complex128, device=wa.device)
        _lib.call("trot_overlap", ctypes.byref(s), wa.data_ptr(), _ptr(wb), out.data_ptr(), native.stream_ptr())
        ctx.save_for_backward(wa, wb)
        ctx.prob = prob
        return out

    @staticmethod
    def backward(ctx, gov):
        wa, wb = ctx.saved_tensors
        s = ctx.prob.system()
        gwa, gwb = torch.zeros_like(wa), torch.zeros_like(wb)
        ws = _vjp_ws(s, _lib.OP_OVERLAP)
        _lib.call("trot_overlap_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), gov.contiguous().data_ptr(),
                  gwa.data_ptr(), _ptr(gwb), ws.data_ptr(), ws.numel(), native.stream_ptr())
        return gwa, gwb, None


class LocalEnergy(torch.autograd.Function):
    """Re E_L (trot_local_energy); backward trot_local_energy_vjp (walkers and h1 via rot_h1)."""

    @staticmethod
    def forward(ctx, wa, wb, h1, prob: AdjointProblem):
        rot = _rot_h1(prob, h1.detach())
        s = prob.system(rot_h1=rot)
        e = torch.empty(wa.shape[0], dtype=torch.complex128, device=wa.device)
        wsp, wsn = native.ws_for(s, _lib.OP_LOCAL_ENERGY)
        _lib.call("trot_local_energy", ctypes.byref(s), wa.data_ptr(), _ptr(wb), e.data_ptr(), wsp, wsn,
                  native.stream_ptr())
        ctx.save_for_backward(wa, wb, *[r for r in rot if r is not None])
        ctx.prob = prob
        return e.real.contiguous()

    @staticmethod
    def backward(ctx, ge):
        wa, wb, *rot = ctx.saved_tensors
        prob = ctx.prob
        s = prob.system(rot_h1=(rot[0], rot[1] if len(rot) > 1 else None))
        gwa, gwb = torch.zeros_like(wa), torch.zeros_like(wb)
        gh1 = torch.zeros((prob.norb, prob.norb), dtype=torch.float64, device=wa.device)
        ws = _vjp_ws(s, _lib.OP_LOCAL_ENERGY)
        _lib.call("trot_local_energy_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), ge.contiguous().data_ptr(),
                  gwa.data_ptr(), _ptr(gwb), gh1.data_ptr(), ws.data_ptr(), ws.numel(), native.stream_ptr())
        return gwa, gwb, gh1, None


def _rot_h1(prob: AdjointProblem, h1: torch.Tensor):
    """(C_a^T h1, C_b^T h1) for a UHF trial, (C^T h1, None) otherwise."""
    out = []
    for mo in (prob.mo if prob.kind == _lib.UHF_U else prob.mo[:1]):
        N, n = prob.norb, int(mo.shape[1])
        rot = torch.empty((n, N), dtype=torch.float64, device=h1.device)
        _lib.call("trot_half_rotate", N, 0, n, mo.data_ptr(), h1.contiguous().data_ptr(), 0, rot.data_ptr(), 0,
                  native.stream_ptr())
        out.append(rot)
    return (out[0], out[1] if len(out) > 1 else None)


def _block(prob: AdjointProblem, b: int, wa, wb, wt, ov, scal, eh, h1):
    """One block: steps, QR, overlaps, energies, clamp, block energy, e_estimate update.
    Returns the new state and this block's sums (sum wt E~, sum wt)."""
    k = prob.steps_per_block
    for t in range(b * k, (b + 1) * k):
        wa, wb, wt, ov, scal = Step.apply(wa, wb, wt, ov, scal, eh, prob.fields[t], prob)
    wa, wb = Orthonormalize.apply(wa, wb, prob)
    ov = Overlap.apply(wa, wb, prob)
    e = LocalEnergy.apply(wa, wb, h1, prob)
    ee = scal[1]
    thresh = math.sqrt(2.0 / prob.params.dt)
    finite = torch.isfinite(e)
    keep = finite & ((e - ee).abs() <= thresh)
    e_t = torch.where(keep, torch.where(finite, e, torch.zeros_like(e)), ee.expand_as(e))
    wt = torch.where(finite, wt, torch.zeros_like(wt))
    num = torch.sum(wt * e_t)
    den = torch.sum(wt)
    e_block = torch.where(den == 0, ee, num / torch.where(den == 0, torch.ones_like(den), den))
    alpha = float(prob.params.shift_ema)
    scal = torch.stack([scal[0], (1.0 - alpha) * ee + alpha * e_block])
    return wa, wb, wt, ov, scal, num, den


def mixed_energy(h1: torch.Tensor, prob: AdjointProblem, checkpoint_blocks: bool = True) -> torch.Tensor:
    """J(h1) as a differentiable 0-d tensor (see the module docstring)."""
    eh = ExpH1Half.apply(h1, prob)
    if prob.unrestricted:
        wa, wb = prob.walkers0
    else:
        wa, wb = prob.walkers0, _empty(prob.walkers0)
    W = prob.n_walkers
    dev = wa.device
    wt = (torch.ones(W, dtype=torch.float64, device=dev) if prob.weights0 is None
          else ctx_dev.real_dev(prob.weights0, "weights0"))
    ov = Overlap.apply(wa, wb, prob).detach()
    scal = torch.tensor([prob.e_estimate0, prob.e_estimate0], dtype=torch.float64, device=dev)
    num = torch.zeros((), dtype=torch.float64, device=dev)
    den = torch.zeros((), dtype=torch.float64, device=dev)
    nblocks = prob.fields.shape[0] // prob.steps_per_block
    for b in range(nblocks):
        if checkpoint_blocks:
            wa, wb, wt, ov, scal, nb, db = checkpoint(_block, prob, b, wa, wb, wt, ov, scal, eh, h1,
                                                      use_reentrant=False)
        else:
            wa, wb, wt, ov, scal, nb, db = _block(prob, b, wa, wb, wt, ov, scal, eh, h1)
        num = num + nb
        den = den + db
    return num / den


def energy_and_grad(h1, prob: AdjointProblem, checkpoint_blocks: bool = True):
    """(J, dJ/dh1): one forward run and one adjoint run."""
    h1 = ctx_dev.real_dev(h1, "h1").clone().requires_grad_(True)
    J = mixed_energy(h1, prob, checkpoint_blocks)
    (g,) = torch.autograd.grad(J, h1)
    return J.detach(), g


def energy(h1, prob: AdjointProblem) -> float:
    """J(h1) without gradient bookkeeping (for finite differences)."""
    with torch.no_grad():
        return float(mixed_energy(ctx_dev.real_dev(h1, "h1"), prob, checkpoint_blocks=False))


def initial_walkers(trial, n_walkers: int, walker_kind: str = "restricted"):
    """Walkers equal to the trial's occupied orbitals, complex128 (W, N, n) per spin."""
    mo_a, mo_b = trial.coeffs()
    rep = lambda mo: mo.to(torch.complex128).unsqueeze(0).repeat(n_walkers, 1, 1).contiguous()
    return (rep(mo_a), rep(mo_b)) if walker_kind == "unrestricted" else rep(mo_a)


def as_problem(h0, chol, trial, params, fields, walkers0=None, e_estimate0=None, steps_per_block=None,
               weights0=None, walker_kind=None):
    """Convenience constructor; e_estimate0 defaults to 0 (it only enters the
    clamp and the population-control shift); weights0 defaults to ones; the walker
    kind defaults to unrestricted for a UHF trial, restricted otherwise."""
    W = int(fields.shape[1])
    wk = walker_kind or ("unrestricted" if isinstance(trial, UhfTrial) else "restricted")
    if walkers0 is None:
        walkers0 = initial_walkers(trial, W, wk)
    mo_a, mo_b = trial.coeffs()
    rdm1 = torch.stack([mo_a @ mo_a.T, mo_b @ mo_b.T])
    return AdjointProblem(h0=float(h0), chol=chol, trial=trial, rdm1=rdm1, params=params, fields=fields,
                          walkers0=walkers0, e_estimate0=float(e_estimate0 or 0.0),
                          steps_per_block=int(steps_per_block or params.n_prop_steps), weights0=weights0,
                          walker_kind=wk)


__all__ = ["AdjointProblem", "mixed_energy", "energy_and_grad", "energy", "as_problem", "initial_walkers",
           "ExpH1Half", "Step", "Orthonormalize", "Overlap", "LocalEnergy", "RhfTrial", "UhfTrial"]
