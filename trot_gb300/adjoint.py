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

RHF trial, restricted walkers, FP64 (the library's adjoint scope).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import _lib, native
from . import ctx as ctx_dev
from .core import QmcParams
from .trial import RhfTrial


@dataclass
class AdjointProblem:
    """Everything but h1: h0, chol (G, N, N), the RHF trial (N, n), the trial
    1-RDM used for the mean-field shifts, the run parameters, the fields of
    every step (T, W, G), the initial walkers (W, N, n) and e_estimate."""

    h0: float
    chol: torch.Tensor
    trial: RhfTrial
    rdm1: torch.Tensor
    params: QmcParams
    fields: torch.Tensor
    walkers0: torch.Tensor
    e_estimate0: float
    steps_per_block: int
    weights0: torch.Tensor | None = None

    def __post_init__(self):
        self.chol = ctx_dev.real_dev(self.chol, "chol")
        self.fields = ctx_dev.real_dev(self.fields, "fields")
        if not isinstance(self.walkers0, torch.Tensor) or not self.walkers0.is_cuda:
            self.walkers0 = torch.as_tensor(np.asarray(self.walkers0)).cuda()
        self.walkers0 = self.walkers0.to(torch.complex128).contiguous()
        T, W, G = self.fields.shape
        if T % self.steps_per_block:
            raise ValueError(f"{T} steps are not a whole number of blocks of {self.steps_per_block}")
        if tuple(self.walkers0.shape[1:]) != tuple(self.trial.mo_coeff.shape) or W != self.walkers0.shape[0]:
            raise ValueError("walkers0 must be (W, N, n) matching the trial and the fields")
        N, n = int(self.chol.shape[1]), int(self.trial.mo_coeff.shape[1])
        self.n_walkers, self.norb, self.nchol = W, N, G
        self.rot_chol = torch.empty((G, n, N), dtype=torch.float64, device=self.chol.device)
        _lib.call("trot_half_rotate", N, G, n, self.trial.mo_coeff.data_ptr(), 0, self.chol.data_ptr(), 0,
                  self.rot_chol.data_ptr(), native.stream_ptr())
        # h1-independent propagation constants (mean-field shifts, h0_prop)
        zero = torch.zeros((N, N), dtype=torch.float64, device=self.chol.device)
        mf_im, h0p, _, _ = ctx_dev.prop_ctx(self.h0, zero, self.chol, self.rdm1, self.params.dt)
        self.mf_im, self.h0_prop = mf_im, h0p
        self.chol_flat = self.chol.reshape(G, N * N)

    def system(self, exp_h1_half=None, rot_h1=None) -> _lib.TrotSystem:
        s = _lib.TrotSystem()
        s.kind, s.precision = _lib.RHF_R, _lib.FP64
        s.n_walkers, s.norb, s.nchol = self.n_walkers, self.norb, self.nchol
        s.nocc_a, s.nocc_b = int(self.trial.mo_coeff.shape[1]), 0
        p = self.params
        s.n_exp_terms = int(p.n_exp_terms)
        s.h0, s.h0_prop, s.dt, s.sqrt_dt = float(self.h0), float(self.h0_prop), float(p.dt), math.sqrt(p.dt)
        s.weight_floor, s.weight_cap = float(p.weight_floor), float(p.weight_cap)
        s.pop_control_damping = float(p.pop_control_damping)
        s.mo_a = self.trial.mo_coeff.data_ptr()
        s.rot_chol_a = self.rot_chol.data_ptr()
        s.rot_h1_a = native.ptr(rot_h1)
        s.exp_h1_half = native.ptr(exp_h1_half)
        s.chol_flat = self.chol_flat.data_ptr()
        s.mf_shifts_im = self.mf_im.data_ptr()
        return s


def _ws(nbytes: int) -> torch.Tensor:
    if nbytes == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    return torch.empty(nbytes, dtype=torch.uint8, device="cuda")


def _vjp_ws(s, op) -> torch.Tensor:
    return _ws(_lib.load().trot_vjp_workspace_size(ctypes.byref(s), op))


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
    """One phaseless step (trot_prop_step, FP64); backward trot_prop_step_vjp."""

    @staticmethod
    def forward(ctx, w, wt, ov, scal, eh, x, prob: AdjointProblem):
        s = prob.system(exp_h1_half=eh)
        st = _lib.TrotState()
        wo, wto, ovo, sco = w.clone(), wt.clone(), ov.clone(), scal.clone()
        nodes = torch.zeros(1, dtype=torch.int64, device=w.device)
        st.walkers_a, st.walkers_b = wo.data_ptr(), 0
        st.weights, st.overlaps, st.scalars = wto.data_ptr(), ovo.data_ptr(), sco.data_ptr()
        st.node_encounters = nodes.data_ptr()
        wsp, wsn = native.ws_for(s, _lib.OP_PROP_STEP)
        _lib.call("trot_prop_step", ctypes.byref(s), ctypes.byref(st), x.data_ptr(), None, wsp, wsn,
                  native.stream_ptr())
        ctx.save_for_backward(w, wt, ov, scal, eh, x)
        ctx.prob = prob
        return wo, wto, ovo, sco

    @staticmethod
    def backward(ctx, gw, gwt, gov, gsc):
        w, wt, ov, scal, eh, x = ctx.saved_tensors
        prob = ctx.prob
        s = prob.system(exp_h1_half=eh)
        st = _lib.TrotState()
        st.walkers_a, st.walkers_b = w.data_ptr(), 0
        st.weights, st.overlaps, st.scalars = wt.data_ptr(), ov.data_ptr(), scal.data_ptr()
        gw = torch.zeros_like(w) if gw is None else gw.contiguous()
        gsc = torch.zeros_like(scal) if gsc is None else gsc.contiguous()
        gwt = None if gwt is None else gwt.contiguous()
        gov = None if gov is None else gov.contiguous()
        gw_in, gwt_in = torch.empty_like(w), torch.empty_like(wt)
        gov_in, gsc_in = torch.empty_like(ov), torch.empty_like(scal)
        geh = torch.zeros_like(eh)
        ws = _vjp_ws(s, _lib.OP_PROP_STEP)
        _lib.call("trot_prop_step_vjp", ctypes.byref(s), ctypes.byref(st), x.data_ptr(), gw.data_ptr(),
                  native.ptr(gwt), native.ptr(gov), gsc.data_ptr(), gw_in.data_ptr(), gwt_in.data_ptr(),
                  gov_in.data_ptr(), gsc_in.data_ptr(), geh.data_ptr(), ws.data_ptr(), ws.numel(),
                  native.stream_ptr())
        return gw_in, gwt_in, gov_in, gsc_in, geh, None, None


class Orthonormalize(torch.autograd.Function):
    """QR with the phase convention of trot/walkers.py:137-148; backward g_q (w^H q)^-1."""

    @staticmethod
    def forward(ctx, w, prob: AdjointProblem):
        from .walkers import orthonormalize

        q = orthonormalize(w, "restricted")
        ctx.save_for_backward(w, q)
        ctx.prob = prob
        return q

    @staticmethod
    def backward(ctx, gq):
        w, q = ctx.saved_tensors
        s = ctx.prob.system()
        gw = torch.empty_like(w)
        _lib.call("trot_orthonormalize_vjp", ctypes.byref(s), w.data_ptr(), q.data_ptr(), gq.contiguous().data_ptr(),
                  gw.data_ptr(), native.stream_ptr())
        return gw, None


class Overlap(torch.autograd.Function):
    """det(C^T w)^2 (trot_overlap); backward trot_overlap_vjp."""

    @staticmethod
    def forward(ctx, w, prob: AdjointProblem):
        s = prob.system()
        out = torch.empty(w.shape[0], dtype=torch.complex128, device=w.device)
        _lib.call("trot_overlap", ctypes.byref(s), w.data_ptr(), 0, out.data_ptr(), native.stream_ptr())
        ctx.save_for_backward(w)
        ctx.prob = prob
        return out

    @staticmethod
    def backward(ctx, gov):
        (w,) = ctx.saved_tensors
        s = ctx.prob.system()
        gw = torch.zeros_like(w)
        ws = _vjp_ws(s, _lib.OP_OVERLAP)
        _lib.call("trot_overlap_vjp", ctypes.byref(s), w.data_ptr(), gov.contiguous().data_ptr(), gw.data_ptr(),
                  ws.data_ptr(), ws.numel(), native.stream_ptr())
        return gw, None


class LocalEnergy(torch.autograd.Function):
    """Re E_L (trot_local_energy); backward trot_local_energy_vjp (walkers and h1 via rot_h1)."""

    @staticmethod
    def forward(ctx, w, h1, prob: AdjointProblem):
        rot_h1 = _rot_h1(prob, h1.detach())
        s = prob.system(rot_h1=rot_h1)
        e = torch.empty(w.shape[0], dtype=torch.complex128, device=w.device)
        wsp, wsn = native.ws_for(s, _lib.OP_LOCAL_ENERGY)
        _lib.call("trot_local_energy", ctypes.byref(s), w.data_ptr(), 0, e.data_ptr(), wsp, wsn, native.stream_ptr())
        ctx.save_for_backward(w, rot_h1)
        ctx.prob = prob
        return e.real.contiguous()

    @staticmethod
    def backward(ctx, ge):
        w, rot_h1 = ctx.saved_tensors
        prob = ctx.prob
        s = prob.system(rot_h1=rot_h1)
        gw = torch.zeros_like(w)
        gh1 = torch.zeros((prob.norb, prob.norb), dtype=torch.float64, device=w.device)
        ws = _vjp_ws(s, _lib.OP_LOCAL_ENERGY)
        _lib.call("trot_local_energy_vjp", ctypes.byref(s), w.data_ptr(), ge.contiguous().data_ptr(), gw.data_ptr(),
                  gh1.data_ptr(), ws.data_ptr(), ws.numel(), native.stream_ptr())
        return gw, gh1, None


def _rot_h1(prob: AdjointProblem, h1: torch.Tensor) -> torch.Tensor:
    N, n = prob.norb, int(prob.trial.mo_coeff.shape[1])
    rot = torch.empty((n, N), dtype=torch.float64, device=h1.device)
    _lib.call("trot_half_rotate", N, 0, n, prob.trial.mo_coeff.data_ptr(), h1.contiguous().data_ptr(), 0,
              rot.data_ptr(), 0, native.stream_ptr())
    return rot


def _block(prob: AdjointProblem, b: int, w, wt, ov, scal, eh, h1):
    """One block: steps, QR, overlaps, energies, clamp, block energy, e_estimate update.
    Returns the new state and this block's sums (sum wt E~, sum wt)."""
    k = prob.steps_per_block
    for t in range(b * k, (b + 1) * k):
        w, wt, ov, scal = Step.apply(w, wt, ov, scal, eh, prob.fields[t], prob)
    q = Orthonormalize.apply(w, prob)
    ov = Overlap.apply(q, prob)
    e = LocalEnergy.apply(q, h1, prob)
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
    return q, wt, ov, scal, num, den


def mixed_energy(h1: torch.Tensor, prob: AdjointProblem, checkpoint_blocks: bool = True) -> torch.Tensor:
    """J(h1) as a differentiable 0-d tensor (see the module docstring)."""
    eh = ExpH1Half.apply(h1, prob)
    w = prob.walkers0
    W = prob.n_walkers
    wt = (torch.ones(W, dtype=torch.float64, device=w.device) if prob.weights0 is None
          else ctx_dev.real_dev(prob.weights0, "weights0"))
    ov = Overlap.apply(w, prob).detach()
    scal = torch.tensor([prob.e_estimate0, prob.e_estimate0], dtype=torch.float64, device=w.device)
    num = torch.zeros((), dtype=torch.float64, device=w.device)
    den = torch.zeros((), dtype=torch.float64, device=w.device)
    nblocks = prob.fields.shape[0] // prob.steps_per_block
    for b in range(nblocks):
        if checkpoint_blocks:
            w, wt, ov, scal, nb, db = checkpoint(_block, prob, b, w, wt, ov, scal, eh, h1, use_reentrant=False)
        else:
            w, wt, ov, scal, nb, db = _block(prob, b, w, wt, ov, scal, eh, h1)
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


def initial_walkers(trial: RhfTrial, n_walkers: int) -> torch.Tensor:
    """Walkers equal to the trial (the reference's init_walkers for an RHF trial's
    natural orbitals spans the same space), complex128 (W, N, n)."""
    mo = trial.mo_coeff.to(torch.complex128)
    return mo.unsqueeze(0).repeat(n_walkers, 1, 1).contiguous()


def as_problem(h0, chol, trial, params, fields, walkers0=None, e_estimate0=None, steps_per_block=None,
               weights0=None):
    """Convenience constructor; e_estimate0 defaults to 0 (it only enters the
    clamp and the population-control shift); weights0 defaults to ones."""
    W = int(fields.shape[1])
    if walkers0 is None:
        walkers0 = initial_walkers(trial, W)
    rdm1 = torch.stack([trial.mo_coeff @ trial.mo_coeff.T, trial.mo_coeff @ trial.mo_coeff.T])
    return AdjointProblem(h0=float(h0), chol=chol, trial=trial, rdm1=rdm1, params=params, fields=fields,
                          walkers0=walkers0, e_estimate0=float(e_estimate0 or 0.0),
                          steps_per_block=int(steps_per_block or params.n_prop_steps), weights0=weights0)


__all__ = ["AdjointProblem", "mixed_energy", "energy_and_grad", "energy", "as_problem", "initial_walkers",
           "ExpH1Half", "Step", "Orthonormalize", "Overlap", "LocalEnergy"]
