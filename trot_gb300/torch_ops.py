"""The C ABI as PyTorch operators: ``torch.ops.trot_gb300.*``.

Each operator takes plain tensors and scalars (no Python objects), so torch's
dispatcher can see it: it has a fake (meta) implementation for shape
propagation under ``FakeTensorMode`` / ``torch.compile`` tracing, and the
differentiable ones carry the library's hand-written vector-Jacobian products
as their backward.  They stand for the per-walker kernels the reference binds
through ``MeasOps`` / ``TrialOps`` / the walker functions
(trot/core/ops.py:49-166, trot/walkers.py:137-293, trot/prop/afqmc.py:79-144),
batched over the leading walker axis.

Conventions shared by every operator:

* ``kind``: 0 RHF trial + restricted walkers, 1 RHF trial + unrestricted
  walkers, 2 UHF trial + unrestricted walkers (``trot_kind``);
* walkers complex128 CUDA tensors (W, N, n); for ``kind`` 0 the beta walker
  argument is an empty tensor, and the beta trial / half-rotated arguments of
  RHF trials may repeat the alpha ones;
* ``mixed``: the tensor-core path (exact-digit FP16 exchange, split-BF16 VHS
  and Taylor action); its operands are derived from the given tensors on first
  use and cached while those tensors live unchanged;
* gradients (FP64 only): walkers through ``trot_overlap_vjp``,
  ``trot_local_energy_vjp`` (of Re E_L), ``trot_orthonormalize_vjp`` and
  ``trot_prop_step_vjp``; the other inputs are not differentiated.
"""
from __future__ import annotations

import ctypes
import math

import torch
from torch.library import custom_op

from . import _lib, native

_MIXED_CACHE: dict = {}


def _ptr(t) -> int:
    return 0 if t is None or t.numel() == 0 else t.data_ptr()


def _mixed(rot_chol_a, rot_chol_b, chol_flat=None, exp_h1_half=None):
    """The trot_mixed operands of these tensors (cached by address and version;
    the cache keeps the tensors alive, so an address is never reused under it)."""
    from . import mixed as _mx

    ts = [t for t in (rot_chol_a, rot_chol_b, chol_flat, exp_h1_half) if t is not None and t.numel()]
    key = tuple((t.data_ptr(), tuple(t.shape), t._version) for t in ts) + (rot_chol_b is None or
                                                                          rot_chol_b.numel() == 0,)
    hit = _MIXED_CACHE.get(key)
    if hit is None:
        rb = None if rot_chol_b is None or rot_chol_b.numel() == 0 else rot_chol_b.cpu().numpy()
        ra = None if rot_chol_a is None or rot_chol_a.numel() == 0 else rot_chol_a.cpu().numpy()
        cf = None if chol_flat is None or chol_flat.numel() == 0 else chol_flat.cpu().numpy()
        eh = None if exp_h1_half is None or exp_h1_half.numel() == 0 else exp_h1_half.cpu().numpy()
        hit = (_mx.MixedCtx(ra, rb, cf, eh), ts)
        _MIXED_CACHE[key] = hit
    return hit[0]


def _system(kind, walkers_a, mo_a, mo_b, *, rot_h1=(None, None), rot_chol=(None, None), h0=0.0, mixed=False,
            prop=None):
    """trot_system from tensors (prop: dict of the propagation context and parameters)."""
    s = _lib.TrotSystem()
    s.kind = int(kind)
    s.precision = _lib.MIXED if mixed else _lib.FP64
    s.n_walkers = int(walkers_a.shape[0])
    s.norb, s.nocc_a = int(mo_a.shape[0]), int(mo_a.shape[1])
    s.nocc_b = int(mo_b.shape[1]) if kind != _lib.RHF_R else 0
    s.mo_a = mo_a.data_ptr()
    s.mo_b = _ptr(mo_b) if kind == _lib.UHF_U else 0
    s.h0 = float(h0)
    ha, hb = rot_h1
    ra, rb = rot_chol
    uhf = kind == _lib.UHF_U
    s.rot_h1_a, s.rot_h1_b = _ptr(ha), (_ptr(hb) if uhf else 0)
    s.rot_chol_a, s.rot_chol_b = _ptr(ra), (_ptr(rb) if uhf else 0)
    if ra is not None and ra.numel():
        s.nchol = int(ra.shape[0])
    s.n_exp_terms = 6
    if prop is not None:
        s.nchol = int(prop["chol_flat"].shape[0])
        s.exp_h1_half = prop["exp_h1_half"].data_ptr()
        s.chol_flat = prop["chol_flat"].data_ptr()
        s.mf_shifts_im = prop["mf_shifts_im"].data_ptr()
        s.h0_prop, s.dt, s.sqrt_dt = float(prop["h0_prop"]), float(prop["dt"]), math.sqrt(float(prop["dt"]))
        s.n_exp_terms = int(prop["n_exp_terms"])
        s.weight_floor, s.weight_cap = float(prop["weight_floor"]), float(prop["weight_cap"])
        s.pop_control_damping = float(prop["pop_control_damping"])
    if mixed:
        mx = _mixed(ra, rb if uhf else None, None if prop is None else prop["chol_flat"],
                    None if prop is None else prop["exp_h1_half"])
        s.mixed = mx.data_ptr()  # kept alive by the cache
    return s


# ---------------------------------------------------------------- overlap


@custom_op("trot_gb300::overlap", mutates_args=())
def overlap(walkers_a: torch.Tensor, walkers_b: torch.Tensor, mo_a: torch.Tensor, mo_b: torch.Tensor,
            kind: int) -> torch.Tensor:
    """Trial overlaps (W,) (overlap_r / overlap_u, trot/trial/rhf.py:45-54, trot/trial/uhf.py:48-58)."""
    s = _system(kind, walkers_a, mo_a, mo_b)
    out = torch.empty(walkers_a.shape[0], dtype=torch.complex128, device=walkers_a.device)
    _lib.call("trot_overlap", ctypes.byref(s), walkers_a.data_ptr(), _ptr(walkers_b), out.data_ptr(),
              native.stream_ptr())
    return out


@overlap.register_fake
def _(walkers_a, walkers_b, mo_a, mo_b, kind):
    return walkers_a.new_empty((walkers_a.shape[0],))


def _overlap_setup(ctx, inputs, output):
    wa, wb, mo_a, mo_b, kind = inputs
    ctx.save_for_backward(wa, wb, mo_a, mo_b)
    ctx.kind = kind


def _overlap_backward(ctx, g):
    wa, wb, mo_a, mo_b = ctx.saved_tensors
    s = _system(ctx.kind, wa, mo_a, mo_b)
    ga, gb = torch.zeros_like(wa), torch.zeros_like(wb)
    nbytes = _lib.load().trot_vjp_workspace_size(ctypes.byref(s), _lib.OP_OVERLAP)
    ws = native.workspace(nbytes)
    _lib.call("trot_overlap_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), g.contiguous().data_ptr(), ga.data_ptr(),
              _ptr(gb), ws.data_ptr(), ws.numel(), native.stream_ptr())
    return ga, gb, None, None, None


overlap.register_autograd(_overlap_backward, setup_context=_overlap_setup)


# ---------------------------------------------------------------- force bias, local energy


@custom_op("trot_gb300::force_bias", mutates_args=())
def force_bias(walkers_a: torch.Tensor, walkers_b: torch.Tensor, mo_a: torch.Tensor, mo_b: torch.Tensor,
               rot_chol_a: torch.Tensor, rot_chol_b: torch.Tensor, kind: int, mixed: bool) -> torch.Tensor:
    """Force bias (W, G) (force_bias_kernel_rw_rh / _uw_rh, trot/meas/rhf.py:119-153, trot/meas/uhf.py:43-57)."""
    s = _system(kind, walkers_a, mo_a, mo_b, rot_chol=(rot_chol_a, rot_chol_b), mixed=mixed)
    out = torch.empty((walkers_a.shape[0], s.nchol), dtype=torch.complex128, device=walkers_a.device)
    ws, nws = native.ws_for(s, _lib.OP_FORCE_BIAS)
    _lib.call("trot_force_bias", ctypes.byref(s), walkers_a.data_ptr(), _ptr(walkers_b), out.data_ptr(), ws, nws,
              native.stream_ptr())
    if mixed:
        native.raise_on_timeout(ws, "force bias")
    return out


@force_bias.register_fake
def _(walkers_a, walkers_b, mo_a, mo_b, rot_chol_a, rot_chol_b, kind, mixed):
    return walkers_a.new_empty((walkers_a.shape[0], rot_chol_a.shape[0]))


@custom_op("trot_gb300::local_energy", mutates_args=())
def local_energy(walkers_a: torch.Tensor, walkers_b: torch.Tensor, mo_a: torch.Tensor, mo_b: torch.Tensor,
                 rot_h1_a: torch.Tensor, rot_h1_b: torch.Tensor, rot_chol_a: torch.Tensor, rot_chol_b: torch.Tensor,
                 h0: float, kind: int, mixed: bool) -> torch.Tensor:
    """Local energies (W,) (energy_kernel_rw_rh / _uw_rh, trot/meas/rhf.py:128-172, trot/meas/uhf.py:205-231)."""
    s = _system(kind, walkers_a, mo_a, mo_b, rot_h1=(rot_h1_a, rot_h1_b), rot_chol=(rot_chol_a, rot_chol_b), h0=h0,
                mixed=mixed)
    out = torch.empty(walkers_a.shape[0], dtype=torch.complex128, device=walkers_a.device)
    ws, nws = native.ws_for(s, _lib.OP_LOCAL_ENERGY)
    _lib.call("trot_local_energy", ctypes.byref(s), walkers_a.data_ptr(), _ptr(walkers_b), out.data_ptr(), ws, nws,
              native.stream_ptr())
    if mixed:
        native.raise_on_timeout(ws, "local energy")
    return out


@local_energy.register_fake
def _(walkers_a, walkers_b, mo_a, mo_b, rot_h1_a, rot_h1_b, rot_chol_a, rot_chol_b, h0, kind, mixed):
    return walkers_a.new_empty((walkers_a.shape[0],))


def _energy_setup(ctx, inputs, output):
    wa, wb, mo_a, mo_b, ha, hb, ra, rb, h0, kind, mixed = inputs
    ctx.save_for_backward(wa, wb, mo_a, mo_b, ha, hb, ra, rb)
    ctx.h0, ctx.kind, ctx.mixed = h0, kind, mixed


def _energy_backward(ctx, g):
    if ctx.mixed:
        raise NotImplementedError("trot_gb300::local_energy: gradients need mixed=False (FP64 adjoint)")
    wa, wb, mo_a, mo_b, ha, hb, ra, rb = ctx.saved_tensors
    if bool((g.imag != 0).any()):
        raise NotImplementedError("trot_gb300::local_energy: only Re E_L is differentiated")
    s = _system(ctx.kind, wa, mo_a, mo_b, rot_h1=(ha, hb), rot_chol=(ra, rb), h0=ctx.h0)
    gre = g.real.contiguous()
    ga, gb = torch.zeros_like(wa), torch.zeros_like(wb)
    N = int(mo_a.shape[0])
    gh1 = torch.zeros((N, N), dtype=torch.float64, device=wa.device)  # through rot_h1 = C^T h1: not returned
    nbytes = _lib.load().trot_vjp_workspace_size(ctypes.byref(s), _lib.OP_LOCAL_ENERGY)
    ws = native.workspace(nbytes)
    _lib.call("trot_local_energy_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), gre.data_ptr(), ga.data_ptr(),
              _ptr(gb), gh1.data_ptr(), ws.data_ptr(), ws.numel(), native.stream_ptr())
    return ga, gb, None, None, None, None, None, None, None, None, None


local_energy.register_autograd(_energy_backward, setup_context=_energy_setup)


# ---------------------------------------------------------------- walkers: QR, SR


def _walker_system(kind, wa, wb):
    s = _lib.TrotSystem()
    s.kind, s.n_walkers, s.norb, s.nocc_a = int(kind), int(wa.shape[0]), int(wa.shape[1]), int(wa.shape[2])
    s.nocc_b = int(wb.shape[2]) if kind != _lib.RHF_R else 0
    s.mo_a = s.mo_b = wa.data_ptr()  # not read by QR / SR
    return s


@custom_op("trot_gb300::orthonormalize", mutates_args=())
def orthonormalize(walkers_a: torch.Tensor, walkers_b: torch.Tensor, kind: int) -> tuple[torch.Tensor, torch.Tensor,
                                                                                         torch.Tensor]:
    """(Q_a, Q_b, norm): reduced QR per walker and spin with diag(R) real >= 0, and det(R)^2 (restricted)
    or det(R_a) det(R_b) (orthogonalize / orthonormalize, trot/walkers.py:137-179)."""
    qa, qb = walkers_a.clone(), walkers_b.clone()
    norm = torch.empty(walkers_a.shape[0], dtype=torch.complex128, device=walkers_a.device)
    s = _walker_system(kind, qa, qb)
    _lib.call("trot_orthonormalize", ctypes.byref(s), qa.data_ptr(), _ptr(qb), norm.data_ptr(), native.stream_ptr())
    return qa, qb, norm


@orthonormalize.register_fake
def _(walkers_a, walkers_b, kind):
    return torch.empty_like(walkers_a), torch.empty_like(walkers_b), walkers_a.new_empty((walkers_a.shape[0],))


def _qr_setup(ctx, inputs, output):
    wa, wb, kind = inputs
    qa, qb, _ = output
    ctx.save_for_backward(wa, wb, qa, qb)
    ctx.kind = kind


def _qr_backward(ctx, gqa, gqb, gnorm):
    wa, wb, qa, qb = ctx.saved_tensors
    if gnorm is not None and bool((gnorm != 0).any()):
        raise NotImplementedError("trot_gb300::orthonormalize: the norm output is not differentiated")
    s = _walker_system(ctx.kind, wa, wb)
    gqa = torch.zeros_like(qa) if gqa is None else gqa.contiguous()
    gqb = torch.zeros_like(qb) if gqb is None else gqb.contiguous()
    gwa, gwb = torch.empty_like(wa), torch.empty_like(wb)
    _lib.call("trot_orthonormalize_vjp", ctypes.byref(s), wa.data_ptr(), _ptr(wb), qa.data_ptr(), _ptr(qb),
              gqa.data_ptr(), _ptr(gqb), gwa.data_ptr(), _ptr(gwb), native.stream_ptr())
    return gwa, gwb, None


orthonormalize.register_autograd(_qr_backward, setup_context=_qr_setup)


@custom_op("trot_gb300::sr_resample", mutates_args=())
def sr_resample(walkers_a: torch.Tensor, walkers_b: torch.Tensor, weights: torch.Tensor, zeta: float,
                kind: int) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor, torch.Tensor]:
    """(walkers_a, walkers_b, weights, indices) after comb resampling with the given zeta
    (stochastic_reconfiguration, trot/walkers.py:249-293)."""
    s = _walker_system(kind, walkers_a, walkers_b)
    oa, ob = torch.empty_like(walkers_a), torch.empty_like(walkers_b)
    wout = torch.empty_like(weights)
    idx = torch.empty(walkers_a.shape[0], dtype=torch.int64, device=walkers_a.device)
    ws = native.workspace(_lib.load().trot_workspace_size(ctypes.byref(s), _lib.OP_SR))
    _lib.call("trot_sr_resample", ctypes.byref(s), weights.contiguous().data_ptr(), 0, float(zeta),
              walkers_a.data_ptr(), _ptr(walkers_b), oa.data_ptr(), _ptr(ob), wout.data_ptr(), idx.data_ptr(),
              ws.data_ptr(), ws.numel(), native.stream_ptr())
    return oa, ob, wout, idx


@sr_resample.register_fake
def _(walkers_a, walkers_b, weights, zeta, kind):
    return (torch.empty_like(walkers_a), torch.empty_like(walkers_b), torch.empty_like(weights),
            weights.new_empty((walkers_a.shape[0],), dtype=torch.int64))


# ---------------------------------------------------------------- the phaseless step


def _prop(exp_h1_half, chol_flat, mf_shifts_im, h0_prop, dt, n_exp_terms, weight_floor, weight_cap, damping):
    return dict(exp_h1_half=exp_h1_half, chol_flat=chol_flat, mf_shifts_im=mf_shifts_im, h0_prop=h0_prop, dt=dt,
                n_exp_terms=n_exp_terms, weight_floor=weight_floor, weight_cap=weight_cap,
                pop_control_damping=damping)


@custom_op("trot_gb300::prop_step", mutates_args=("walkers_a", "walkers_b", "weights", "overlaps", "scalars",
                                                  "node_encounters"))
def prop_step(walkers_a: torch.Tensor, walkers_b: torch.Tensor, weights: torch.Tensor, overlaps: torch.Tensor,
              scalars: torch.Tensor, node_encounters: torch.Tensor, fields: torch.Tensor, mo_a: torch.Tensor,
              mo_b: torch.Tensor, rot_h1_a: torch.Tensor, rot_h1_b: torch.Tensor, rot_chol_a: torch.Tensor,
              rot_chol_b: torch.Tensor, exp_h1_half: torch.Tensor, chol_flat: torch.Tensor,
              mf_shifts_im: torch.Tensor, h0: float, h0_prop: float, dt: float, n_exp_terms: int,
              weight_floor: float, weight_cap: float, pop_control_damping: float, kind: int,
              mixed: bool) -> torch.Tensor:
    """One phaseless step with injected fields (W, G) (afqmc_step, trot/prop/afqmc.py:79-144), updating the
    state tensors in place (walkers, weights, overlaps, scalars = [E_shift, e_estimate], node count);
    returns the local energies (W,) of the walkers entering the step."""
    prop = _prop(exp_h1_half, chol_flat, mf_shifts_im, h0_prop, dt, n_exp_terms, weight_floor, weight_cap,
                 pop_control_damping)
    s = _system(kind, walkers_a, mo_a, mo_b, rot_h1=(rot_h1_a, rot_h1_b), rot_chol=(rot_chol_a, rot_chol_b),
                h0=h0, mixed=mixed, prop=prop)
    st = _lib.TrotState()
    st.walkers_a, st.walkers_b = walkers_a.data_ptr(), _ptr(walkers_b)
    st.weights, st.overlaps, st.scalars = weights.data_ptr(), overlaps.data_ptr(), scalars.data_ptr()
    st.node_encounters = node_encounters.data_ptr()
    e = torch.empty(walkers_a.shape[0], dtype=torch.complex128, device=walkers_a.device)
    ws, nws = native.ws_for(s, _lib.OP_PROP_STEP)
    _lib.call("trot_prop_step", ctypes.byref(s), ctypes.byref(st), fields.contiguous().data_ptr(), e.data_ptr(),
              ws, nws, native.stream_ptr())
    return e


@prop_step.register_fake
def _(walkers_a, *args):
    return walkers_a.new_empty((walkers_a.shape[0],))


@custom_op("trot_gb300::prop_step_functional", mutates_args=())
def prop_step_functional(walkers_a: torch.Tensor, walkers_b: torch.Tensor, weights: torch.Tensor,
                         overlaps: torch.Tensor, scalars: torch.Tensor, fields: torch.Tensor, mo_a: torch.Tensor,
                         mo_b: torch.Tensor, rot_chol_a: torch.Tensor, rot_chol_b: torch.Tensor,
                         exp_h1_half: torch.Tensor, chol_flat: torch.Tensor, mf_shifts_im: torch.Tensor,
                         h0_prop: float, dt: float, n_exp_terms: int, weight_floor: float, weight_cap: float,
                         pop_control_damping: float, kind: int) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor,
                                                                         torch.Tensor, torch.Tensor]:
    """prop_step without mutation (FP64): returns the new (walkers_a, walkers_b, weights, overlaps,
    scalars); differentiable in the walkers, weights, overlaps, scalars and exp_h1_half through
    trot_prop_step_vjp (the step is recomputed inside the backward)."""
    out = [walkers_a.clone(), walkers_b.clone(), weights.clone(), overlaps.clone(), scalars.clone()]
    nodes = torch.zeros(1, dtype=torch.int64, device=walkers_a.device)
    empty = walkers_a.new_empty((0,), dtype=torch.float64)
    prop_step(out[0], out[1], out[2], out[3], out[4], nodes, fields, mo_a, mo_b, empty, empty, rot_chol_a,
              rot_chol_b, exp_h1_half, chol_flat, mf_shifts_im, 0.0, h0_prop, dt, n_exp_terms, weight_floor,
              weight_cap, pop_control_damping, kind, False)
    return tuple(out)


@prop_step_functional.register_fake
def _(walkers_a, walkers_b, weights, overlaps, scalars, *args):
    return (torch.empty_like(walkers_a), torch.empty_like(walkers_b), torch.empty_like(weights),
            torch.empty_like(overlaps), torch.empty_like(scalars))


def _step_setup(ctx, inputs, output):
    (wa, wb, wt, ov, scal, x, mo_a, mo_b, ra, rb, eh, cf, mf, h0_prop, dt, nterms, wfl, wcap, damp, kind) = inputs
    ctx.save_for_backward(wa, wb, wt, ov, scal, x, mo_a, mo_b, ra, rb, eh, cf, mf)
    ctx.args = (h0_prop, dt, nterms, wfl, wcap, damp, kind)


def _step_backward(ctx, gwa, gwb, gwt, gov, gsc):
    wa, wb, wt, ov, scal, x, mo_a, mo_b, ra, rb, eh, cf, mf = ctx.saved_tensors
    h0_prop, dt, nterms, wfl, wcap, damp, kind = ctx.args
    prop = _prop(eh, cf, mf, h0_prop, dt, nterms, wfl, wcap, damp)
    s = _system(kind, wa, mo_a, mo_b, rot_chol=(ra, rb), prop=prop)
    st = _lib.TrotState()
    st.walkers_a, st.walkers_b = wa.data_ptr(), _ptr(wb)
    st.weights, st.overlaps, st.scalars = wt.data_ptr(), ov.data_ptr(), scal.data_ptr()

    def g_or_zero(g, like):
        return torch.zeros_like(like) if g is None else g.contiguous()

    gwa, gwb, gsc = g_or_zero(gwa, wa), g_or_zero(gwb, wb), g_or_zero(gsc, scal)
    gwt = None if gwt is None else gwt.contiguous()
    gov = None if gov is None else gov.contiguous()
    gwa_in, gwb_in = torch.empty_like(wa), torch.empty_like(wb)
    gwt_in, gov_in, gsc_in = torch.empty_like(wt), torch.empty_like(ov), torch.empty_like(scal)
    geh = torch.zeros_like(eh)
    ws = native.workspace(_lib.load().trot_vjp_workspace_size(ctypes.byref(s), _lib.OP_PROP_STEP))
    _lib.call("trot_prop_step_vjp", ctypes.byref(s), ctypes.byref(st), x.contiguous().data_ptr(), gwa.data_ptr(),
              _ptr(gwb), native.ptr(gwt), native.ptr(gov), gsc.data_ptr(), gwa_in.data_ptr(), _ptr(gwb_in),
              gwt_in.data_ptr(), gov_in.data_ptr(), gsc_in.data_ptr(), geh.data_ptr(), ws.data_ptr(), ws.numel(),
              native.stream_ptr())
    return (gwa_in, gwb_in, gwt_in, gov_in, gsc_in, None, None, None, None, None, geh) + (None,) * 9


prop_step_functional.register_autograd(_step_backward, setup_context=_step_setup)


def ops():
    """The registered operators (``torch.ops.trot_gb300``)."""
    return torch.ops.trot_gb300
