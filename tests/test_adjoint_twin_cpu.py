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
