"""Hand-written adjoint (trot_*_vjp) vs torch autograd of the twin restatement
(oracle/afqmc_torch_twin.py, the gradient oracle) and vs central finite
differences of the CUDA forward with common random numbers.

Tolerances: vector-Jacobian products of single operators 1e-9 relative
(max-norm); whole-run gradient 1e-8 relative to the twin's autograd and 1e-6
relative to finite differences (lambda = +-1e-4)."""
import numpy as np
import pytest
import torch

from oracle import afqmc_torch_twin as twin
from tests.gpu_helpers import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _problem(N=12, n=3, G=20, W=6, T=8, spb=4, dt=0.01, noise=0.05, seed=4, kind="rhf_r", nb=None):
    """A small system; kind rhf_r (walkers (W, N, n)), rhf_u or uhf_u (walkers (wa, wb))."""
    import trot_gb300 as tg
    from trot_gb300 import adjoint, synthetic

    nb = n if nb is None else nb
    ss = synthetic.make_system(N, (n, nb if kind == "uhf_u" else n), G, decay=30.0, seed=seed, h0=0.3)
    rng = np.random.default_rng(seed + 1)
    fields = rng.standard_normal((T, W, G))
    params = tg.QmcParams(dt=dt, n_exp_terms=6, n_prop_steps=spb, n_walkers=W)
    if kind == "rhf_r":
        w0 = synthetic.perturbed_walkers(ss.mo_a, W, noise, seed + 2)
        trial, walkers = tg.RhfTrial(ss.mo_a), torch.as_tensor(w0).cuda()
    else:
        mo_b = ss.mo_b if kind == "uhf_u" else ss.mo_a
        w0 = (synthetic.perturbed_walkers(ss.mo_a, W, noise, seed + 2),
              synthetic.perturbed_walkers(mo_b, W, noise, seed + 3))
        trial = tg.UhfTrial(ss.mo_a, mo_b) if kind == "uhf_u" else tg.RhfTrial(ss.mo_a)
        walkers = (torch.as_tensor(w0[0]).cuda(), torch.as_tensor(w0[1]).cuda())
    prob = adjoint.as_problem(ss.h0, ss.chol, trial, params, torch.as_tensor(fields).cuda(), walkers0=walkers,
                              e_estimate0=-2.0, steps_per_block=spb,
                              walker_kind="restricted" if kind == "rhf_r" else "unrestricted")
    return ss, fields, w0, prob


def _c(x):
    return torch.as_tensor(np.asarray(x))


def _rand_like(x, seed):
    g = torch.Generator().manual_seed(seed)
    if x.is_complex():
        return torch.complex(torch.randn(x.shape, generator=g, dtype=torch.float64),
                             torch.randn(x.shape, generator=g, dtype=torch.float64))
    return torch.randn(x.shape, generator=g, dtype=torch.float64)


def test_prop_ctx_vjp():
    from trot_gb300 import adjoint

    ss, _, _, prob = _problem()
    h1 = torch.as_tensor(ss.h1).cuda().requires_grad_(True)
    eh = adjoint.ExpH1Half.apply(h1, prob)
    g = _rand_like(eh.detach().cpu(), 1)
    (gh1,) = torch.autograd.grad(eh, h1, g.cuda())
    h1c = _c(ss.h1).clone().requires_grad_(True)
    _, _, ehc = twin.prop_consts(ss.h0, h1c, _c(ss.chol), prob.rdm1.cpu(), prob.params.dt)
    assert rel(eh.detach().cpu().numpy(), ehc.detach().numpy()) < 1e-12
    (ref,) = torch.autograd.grad(ehc, h1c, g)
    assert rel(gh1.cpu().numpy(), ref.numpy()) < 1e-9


def test_step_vjp():
    from trot_gb300 import adjoint

    ss, fields, w0, prob = _problem()
    W = w0.shape[0]
    dev = lambda x: x.cuda().requires_grad_(True)
    w = dev(_c(w0))
    wb = torch.empty(0, dtype=torch.complex128, device="cuda", requires_grad=True)
    wt = dev(torch.linspace(0.5, 1.5, W, dtype=torch.float64))
    ov = dev(twin.overlap(_c(w0), _c(ss.mo_a)).detach())
    scal = dev(torch.tensor([-1.7, -2.1], dtype=torch.float64))
    h1 = torch.as_tensor(ss.h1).cuda()
    eh = dev(adjoint.ExpH1Half.apply(h1, prob).detach())
    x = torch.as_tensor(fields[0]).cuda()
    wa_o, _, wt_o, ov_o, sc_o = adjoint.Step.apply(w, wb, wt, ov, scal, eh, x, prob)
    outs = (wa_o, wt_o, ov_o, sc_o)
    gs = [_rand_like(o.detach().cpu(), 10 + i) for i, o in enumerate(outs)]
    grads = torch.autograd.grad(outs, (w, wt, ov, scal, eh), [g.cuda() for g in gs])

    cw, cwt, cov = _c(w0).requires_grad_(True), wt.detach().cpu().requires_grad_(True), ov.detach().cpu().requires_grad_(True)
    ces = torch.tensor(-1.7, dtype=torch.float64, requires_grad=True)
    cee = torch.tensor(-2.1, dtype=torch.float64, requires_grad=True)
    ceh = eh.detach().cpu().requires_grad_(True)
    rot_chol = torch.einsum("pi,gpj->gij", _c(ss.mo_a), _c(ss.chol))
    p = prob.params
    wn, wtn, ovn, esn = twin.step(cw, cwt, cov, ces, cee, _c(fields[0]), mo=_c(ss.mo_a), rot_chol=rot_chol,
                                  chol=_c(ss.chol), mf_im=prob.mf_im.cpu(), h0_prop=prob.h0_prop, eh=ceh, dt=p.dt,
                                  n_terms=6)
    # forward parity of the library step and the twin
    assert rel(outs[0].detach().cpu().numpy(), wn.detach().numpy()) < 1e-12
    assert rel(outs[1].detach().cpu().numpy(), wtn.detach().numpy()) < 1e-12
    scal_n = torch.stack([esn, cee])
    loss = sum(torch.sum((g.conj() * o).real) if o.is_complex() else torch.sum(g * o)
               for g, o in zip(gs, (wn, wtn, ovn, scal_n)))
    ref = torch.autograd.grad(loss, (cw, cwt, cov, ces, cee, ceh))
    assert rel(grads[0].cpu().numpy(), ref[0].numpy()) < 1e-9
    assert rel(grads[1].cpu().numpy(), ref[1].numpy()) < 1e-9
    assert rel(grads[2].cpu().numpy(), ref[2].numpy()) < 1e-9
    assert rel(grads[3].cpu().numpy(), np.array([ref[3].item(), ref[4].item()])) < 1e-9
    assert rel(grads[4].cpu().numpy(), ref[5].numpy()) < 1e-9


@pytest.mark.parametrize("kind", ["rhf_u", "uhf_u"])
def test_step_vjp_unrestricted(kind):
    from trot_gb300 import adjoint

    ss, fields, w0, prob = _problem(kind=kind, nb=2)
    W = w0[0].shape[0]
    dev = lambda x: x.cuda().requires_grad_(True)
    wa, wb = dev(_c(w0[0])), dev(_c(w0[1]))
    mo = (_c(prob.mo[0].cpu()), _c(prob.mo[1].cpu()))
    kind_t = kind
    mo_t = mo if kind == "uhf_u" else mo[0]
    ov0 = twin._overlap_k((_c(w0[0]), _c(w0[1])), mo_t, kind_t).detach()
    wt = dev(torch.linspace(0.5, 1.5, W, dtype=torch.float64))
    ov = dev(ov0)
    scal = dev(torch.tensor([-1.7, -2.1], dtype=torch.float64))
    eh = dev(adjoint.ExpH1Half.apply(torch.as_tensor(ss.h1).cuda(), prob).detach())
    x = torch.as_tensor(fields[0]).cuda()
    outs = adjoint.Step.apply(wa, wb, wt, ov, scal, eh, x, prob)
    gs = [_rand_like(o.detach().cpu(), 20 + i) for i, o in enumerate(outs)]
    grads = torch.autograd.grad(outs, (wa, wb, wt, ov, scal, eh), [g.cuda() for g in gs])
    cwa, cwb = _c(w0[0]).requires_grad_(True), _c(w0[1]).requires_grad_(True)
    cwt, cov = wt.detach().cpu().requires_grad_(True), ov0.clone().requires_grad_(True)
    ces = torch.tensor(-1.7, dtype=torch.float64, requires_grad=True)
    cee = torch.tensor(-2.1, dtype=torch.float64, requires_grad=True)
    ceh = eh.detach().cpu().requires_grad_(True)
    rot = lambda m: torch.einsum("pi,gpj->gij", m, _c(ss.chol))
    rot_chol = (rot(mo[0]), rot(mo[1])) if kind == "uhf_u" else rot(mo[0])
    wn, wtn, ovn, esn = twin.step((cwa, cwb), cwt, cov, ces, cee, _c(fields[0]), mo=mo_t, rot_chol=rot_chol,
                                  chol=_c(ss.chol), mf_im=prob.mf_im.cpu(), h0_prop=prob.h0_prop, eh=ceh,
                                  dt=prob.params.dt, n_terms=6, kind=kind)
    assert rel(outs[0].detach().cpu().numpy(), wn[0].detach().numpy()) < 1e-12
    assert rel(outs[1].detach().cpu().numpy(), wn[1].detach().numpy()) < 1e-12
    loss = sum(torch.sum((g.conj() * o).real) if o.is_complex() else torch.sum(g * o)
               for g, o in zip(gs, (wn[0], wn[1], wtn, ovn, torch.stack([esn, cee]))))
    ref = torch.autograd.grad(loss, (cwa, cwb, cwt, cov, ces, cee, ceh))
    for k in range(4):
        assert rel(grads[k].cpu().numpy(), ref[k].numpy()) < 1e-9, k
    assert rel(grads[4].cpu().numpy(), np.array([ref[4].item(), ref[5].item()])) < 1e-9
    assert rel(grads[5].cpu().numpy(), ref[6].numpy()) < 1e-9


def test_local_energy_overlap_qr_vjp():
    from trot_gb300 import adjoint

    ss, _, w0, prob = _problem(N=14, n=4, G=24, W=5)
    w = torch.as_tensor(w0).cuda().requires_grad_(True)
    h1 = torch.as_tensor(ss.h1).cuda().requires_grad_(True)
    e0 = torch.empty(0, dtype=torch.complex128, device="cuda")
    e = adjoint.LocalEnergy.apply(w, e0, h1, prob)
    ov = adjoint.Overlap.apply(w, e0, prob)
    ge = _rand_like(e.detach().cpu(), 3)
    gov = _rand_like(ov.detach().cpu(), 4)
    gw, gh1 = torch.autograd.grad((e, ov), (w, h1), (ge.cuda(), gov.cuda()))
    cw = _c(w0).requires_grad_(True)
    ch1 = _c(ss.h1).requires_grad_(True)
    rot_chol = torch.einsum("pi,gpj->gij", _c(ss.mo_a), _c(ss.chol))
    ce = twin.local_energy(cw, _c(ss.mo_a), ss.h0, _c(ss.mo_a).T @ ch1, rot_chol).real
    cov = twin.overlap(cw, _c(ss.mo_a))
    assert rel(e.detach().cpu().numpy(), ce.detach().numpy()) < 1e-12
    loss = torch.sum(ge * ce) + torch.sum((gov.conj() * cov).real)
    rw, rh1 = torch.autograd.grad(loss, (cw, ch1))
    assert rel(gw.cpu().numpy(), rw.numpy()) < 1e-9
    assert rel(gh1.cpu().numpy(), rh1.numpy()) < 1e-9
    # QR: the energy is invariant under w -> w R, so E(qr(w)) has the gradient of E(w)
    w2 = torch.as_tensor(w0).cuda().requires_grad_(True)
    q2, _ = adjoint.Orthonormalize.apply(w2, e0, prob)
    e2 = adjoint.LocalEnergy.apply(q2, e0, h1.detach(), prob)
    (gq,) = torch.autograd.grad(e2, w2, ge.cuda())
    w3 = torch.as_tensor(w0).cuda().requires_grad_(True)
    e3 = adjoint.LocalEnergy.apply(w3, e0, h1.detach(), prob)
    (gd,) = torch.autograd.grad(e3, w3, ge.cuda())
    assert rel(gq.cpu().numpy(), gd.cpu().numpy()) < 1e-9


@pytest.mark.parametrize("kind,spb,T", [("rhf_r", 4, 8), ("rhf_r", 3, 9), ("rhf_u", 4, 8), ("uhf_u", 4, 8)])
def test_mixed_energy_gradient(kind, spb, T):
    """Whole run (steps, QR, overlaps, energies, clamps, e_estimate updates, checkpointed blocks)."""
    from trot_gb300 import adjoint

    ss, fields, w0, prob = _problem(T=T, spb=spb, kind=kind, nb=2)
    J, g = adjoint.energy_and_grad(ss.h1, prob)
    mo = (_c(prob.mo[0].cpu()), _c(prob.mo[1].cpu()))
    kw = dict(h0=ss.h0, chol=_c(ss.chol), mo=mo if kind == "uhf_u" else mo[0], rdm1=prob.rdm1.cpu(),
              fields=_c(fields), walkers0=(_c(w0[0]), _c(w0[1])) if kind != "rhf_r" else _c(w0), e_estimate0=-2.0,
              steps_per_block=spb, dt=prob.params.dt, n_terms=6, kind=kind)
    h1c = _c(ss.h1).clone().requires_grad_(True)
    Jc = twin.mixed_energy(h1c, **kw)
    (gc,) = torch.autograd.grad(Jc, h1c)
    assert abs(float(J) - float(Jc.detach())) <= 1e-11 * abs(float(Jc.detach()))
    assert rel(g.cpu().numpy(), gc.numpy()) < 1e-8
    # finite differences of the CUDA forward along a symmetric one-body perturbation O
    O = np.random.default_rng(9).normal(scale=0.1, size=ss.h1.shape)
    O = 0.5 * (O + O.T)
    eps = 1e-4
    fd = (adjoint.energy(ss.h1 + eps * O, prob) - adjoint.energy(ss.h1 - eps * O, prob)) / (2 * eps)
    ad = float(torch.sum(g.cpu() * _c(O)))
    assert abs(ad - fd) <= 1e-6 * abs(fd), (ad, fd)


def test_checkpointing_is_exact():
    from trot_gb300 import adjoint

    ss, _, _, prob = _problem()
    _, g1 = adjoint.energy_and_grad(ss.h1, prob, checkpoint_blocks=True)
    _, g2 = adjoint.energy_and_grad(ss.h1, prob, checkpoint_blocks=False)
    assert torch.equal(g1, g2)


def test_adjoint_rejects_mixed_precision():
    import ctypes

    from trot_gb300 import _lib

    _, _, _, prob = _problem()
    s = prob.system()
    s.precision = _lib.MIXED
    assert _lib.load().trot_vjp_workspace_size(ctypes.byref(s), _lib.OP_PROP_STEP) == 0
    assert b"FP64" in _lib.load().trot_last_error()


def test_dead_walkers_pass_no_gradient():
    """Walkers with zero weight cannot influence the objective: the gradient stays
    finite when such a walker holds NaN and does not depend on its values."""
    import trot_gb300 as tg
    from trot_gb300 import adjoint

    ss, fields, w0, prob = _problem()
    W = w0.shape[0]
    wt0 = torch.ones(W, dtype=torch.float64)
    wt0[1] = 0.0
    wt0[4] = 0.0
    grads = []
    for fill in (np.nan, 0.37):
        w = w0.copy()
        w[1] = fill
        w[4] = fill * 2
        p = adjoint.as_problem(ss.h0, ss.chol, tg.RhfTrial(ss.mo_a), prob.params, prob.fields,
                               walkers0=torch.as_tensor(w).cuda(), e_estimate0=-2.0,
                               steps_per_block=prob.steps_per_block, weights0=wt0.cuda())
        J, g = adjoint.energy_and_grad(ss.h1, p)
        assert np.isfinite(float(J)) and bool(torch.isfinite(g).all())
        grads.append(g)
    assert torch.equal(grads[0], grads[1])
