"""The torch autograd twin (gradient oracle of the adjoint) on the CPU:
its forward step equals the numpy oracle's (which the reference's golden
vectors pin), and its autograd gradient of the mixed energy matches central
finite differences with common random numbers (same fields)."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from oracle import afqmc_torch_twin as twin


def _small(N=10, n=3, G=16, W=5, T=6, seed=4):
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, (n, n), G, decay=30.0, seed=seed, h0=0.3)
    rng = np.random.default_rng(seed + 1)
    fields = rng.standard_normal((T, W, G))
    w0 = synthetic.perturbed_walkers(ss.mo_a, W, 0.05, seed + 2)
    return ss, fields, w0


def test_twin_step_matches_numpy_oracle():
    ss, fields, w0 = _small()
    dt = 0.01
    rdm1 = np.stack([ss.mo_a @ ss.mo_a.T] * 2)
    prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, rdm1, dt)
    meas = orc.build_rhf_meas_ctx(ss.h1, ss.chol, ss.mo_a)
    model = orc.Model(kind="rhf_r", h0=ss.h0, mo=ss.mo_a, meas=meas, prop=prop)
    params = orc.Params(dt=dt, n_exp_terms=6)
    W = w0.shape[0]
    ov0 = orc.overlap_rhf_r(w0, ss.mo_a)
    st = orc.State(walkers=w0, weights=np.ones(W), overlaps=ov0, pop_control_ene_shift=-1.0, e_estimate=-1.0)
    ref = orc.afqmc_step(st, model, params, fields[0])

    t = lambda a: torch.as_tensor(np.asarray(a))
    mf_im, h0p, eh = twin.prop_consts(ss.h0, t(ss.h1), t(ss.chol), t(rdm1), dt)
    rot_chol = torch.einsum("pi,gpj->gij", t(ss.mo_a), t(ss.chol))
    wn, wtn, ovn, esn = twin.step(t(w0), torch.ones(W, dtype=torch.float64), t(ov0), torch.tensor(-1.0),
                                  torch.tensor(-1.0), t(fields[0]), mo=t(ss.mo_a), rot_chol=rot_chol, chol=t(ss.chol),
                                  mf_im=mf_im, h0_prop=h0p, eh=eh, dt=dt, n_terms=6)
    assert np.max(np.abs(wn.numpy() - ref.walkers)) <= 1e-12 * np.max(np.abs(ref.walkers))
    assert np.max(np.abs(wtn.numpy() - ref.weights)) <= 1e-12
    assert np.max(np.abs(ovn.numpy() - ref.overlaps)) <= 1e-12 * np.max(np.abs(ref.overlaps))
    assert abs(float(esn) - ref.pop_control_ene_shift) <= 1e-10
    e_ref = orc.energy_rhf_r(ref.walkers, ss.mo_a, ss.h0, meas)
    e_tw = twin.local_energy(wn, t(ss.mo_a), ss.h0, t(ss.mo_a).T @ t(ss.h1), rot_chol)
    assert np.max(np.abs(e_tw.detach().numpy() - e_ref)) <= 1e-10


@pytest.mark.parametrize("spb", [3, 6])
def test_twin_gradient_vs_finite_differences(spb):
    ss, fields, w0 = _small()
    dt = 0.01
    t = lambda a: torch.as_tensor(np.asarray(a))
    rdm1 = t(np.stack([ss.mo_a @ ss.mo_a.T] * 2))
    O = np.random.default_rng(9).normal(scale=0.1, size=ss.h1.shape)
    O = t(0.5 * (O + O.T))
    kw = dict(h0=ss.h0, chol=t(ss.chol), mo=t(ss.mo_a), rdm1=rdm1, fields=t(fields), walkers0=t(w0),
              e_estimate0=-2.0, steps_per_block=spb, dt=dt, n_terms=6)
    h1 = t(ss.h1).clone().requires_grad_(True)
    J = twin.mixed_energy(h1, **kw)
    (g,) = torch.autograd.grad(J, h1)
    eps = 1e-4
    with torch.no_grad():
        jp = float(twin.mixed_energy(t(ss.h1) + eps * O, **kw))
        jm = float(twin.mixed_energy(t(ss.h1) - eps * O, **kw))
    fd = (jp - jm) / (2 * eps)
    ad = float(torch.sum(g * O))
    assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-12), (ad, fd)


@pytest.mark.parametrize("kind", ["rhf_u", "uhf_u"])
def test_twin_unrestricted_step_and_gradient(kind):
    """Unrestricted walkers (RHF or UHF trial): the twin step equals the numpy oracle's, and
    its autograd gradient of the mixed energy matches central finite differences."""
    from trot_gb300 import synthetic

    N, na, nb, G, W, T, dt = 10, 3, 2, 16, 4, 6, 0.01
    ss = synthetic.make_system(N, (na, nb), G, decay=30.0, seed=6, h0=0.3)
    rng = np.random.default_rng(7)
    fields = rng.standard_normal((T, W, G))
    mo_a = ss.mo_a
    mo_b = ss.mo_b if kind == "uhf_u" else ss.mo_a[:, :nb]
    wa = synthetic.perturbed_walkers(mo_a, W, 0.05, 8)
    wb = synthetic.perturbed_walkers(mo_b, W, 0.05, 9)
    t = lambda a: torch.as_tensor(np.asarray(a))
    if kind == "uhf_u":
        rdm1 = np.stack([mo_a @ mo_a.T, mo_b @ mo_b.T])
        meas = orc.build_uhf_meas_ctx(ss.h1, ss.chol, mo_a, mo_b)
        mo_o, mo_t = (mo_a, mo_b), (t(mo_a), t(mo_b))
    else:
        # RHF trial with unrestricted walkers: both spins use the alpha orbitals (nb = na here)
        nb = na
        mo_b = mo_a
        wb = synthetic.perturbed_walkers(mo_b, W, 0.05, 9)
        rdm1 = np.stack([mo_a @ mo_a.T] * 2)
        meas = orc.build_rhf_meas_ctx(ss.h1, ss.chol, mo_a)
        mo_o, mo_t = mo_a, t(mo_a)
    prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, rdm1, dt)
    model = orc.Model(kind=kind, h0=ss.h0, mo=mo_o, meas=meas, prop=prop)
    ov0 = model.overlap((wa, wb))
    st = orc.State(walkers=(wa, wb), weights=np.ones(W), overlaps=ov0, pop_control_ene_shift=-1.0, e_estimate=-1.0)
    ref = orc.afqmc_step(st, model, orc.Params(dt=dt, n_exp_terms=6), fields[0])
    mf_im, h0p, eh = twin.prop_consts(ss.h0, t(ss.h1), t(ss.chol), t(rdm1), dt)
    rot = lambda m: torch.einsum("pi,gpj->gij", m, t(ss.chol))
    rot_chol = (rot(mo_t[0]), rot(mo_t[1])) if kind == "uhf_u" else rot(mo_t)
    wn, wtn, ovn, esn = twin.step((t(wa), t(wb)), torch.ones(W, dtype=torch.float64), t(ov0), torch.tensor(-1.0),
                                  torch.tensor(-1.0), t(fields[0]), mo=mo_t, rot_chol=rot_chol, chol=t(ss.chol),
                                  mf_im=mf_im, h0_prop=h0p, eh=eh, dt=dt, n_terms=6, kind=kind)
    for s in range(2):
        assert np.max(np.abs(wn[s].numpy() - ref.walkers[s])) <= 1e-12 * np.max(np.abs(ref.walkers[s]))
    assert np.max(np.abs(wtn.numpy() - ref.weights)) <= 1e-12
    assert np.max(np.abs(ovn.numpy() - ref.overlaps)) <= 1e-12 * np.max(np.abs(ref.overlaps))
    # gradient vs finite differences
    O = np.random.default_rng(10).normal(scale=0.1, size=ss.h1.shape)
    O = t(0.5 * (O + O.T))
    kw = dict(h0=ss.h0, chol=t(ss.chol), mo=mo_t, rdm1=t(rdm1), fields=t(fields), walkers0=(t(wa), t(wb)),
              e_estimate0=-2.0, steps_per_block=3, dt=dt, n_terms=6, kind=kind)
    h1 = t(ss.h1).clone().requires_grad_(True)
    (g,) = torch.autograd.grad(twin.mixed_energy(h1, **kw), h1)
    eps = 1e-4
    with torch.no_grad():
        fd = (float(twin.mixed_energy(t(ss.h1) + eps * O, **kw)) - float(twin.mixed_energy(t(ss.h1) - eps * O, **kw))) / (2 * eps)
    ad = float(torch.sum(g * O))
    assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-12), (ad, fd)
