"""Known-answer cases and invariants from the reference's own tests
(trot tests/test_prop_afqmc_step.py, tests/test_trial_rhf.py), checked on the
CPU oracle and (gpu-marked) on the CUDA path."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from trot_gb300 import synthetic


def _rand_orthonormal(rng, n, k):
    a = rng.normal(size=(n, k)) + 1j * rng.normal(size=(n, k))
    return np.linalg.qr(a)[0][:, :k]


def _zero_ham_model(norb, nocc, n_fields, h0, dt):
    h1 = np.zeros((norb, norb))
    chol = np.zeros((n_fields, norb, norb))
    mo = np.eye(norb)[:, :nocc]
    prop = orc.build_prop_ctx(h0, h1, chol, np.zeros((2, norb, norb)), dt)
    return orc.Model("rhf_r", h0, mo, orc.build_rhf_meas_ctx(h1, chol, mo), prop)


def test_weight_update_known_answer():
    """h1 = L = 0, h0 = 1: weights -> exp(-dt), pop-control shift -> 0.1
    (tests/test_prop_afqmc_step.py:33-82)."""
    norb, nocc, nw, nf, dt = 4, 2, 8, 3, 0.2
    m = _zero_ham_model(norb, nocc, nf, 1.0, dt)
    w = np.ones((nw, norb, nocc), dtype=np.complex128)
    w[:, :nocc, :] += np.eye(nocc)  # full-rank overlap matrices
    st = orc.State(w, np.ones(nw), m.overlap(w), 0.0, 0.0, 0)
    out = orc.afqmc_step(st, m, orc.Params(dt=dt), np.random.default_rng(0).normal(size=(nw, nf)))
    np.testing.assert_allclose(out.weights, np.exp(-dt) * np.ones(nw), rtol=1e-14)
    assert abs(out.pop_control_ene_shift - 0.1) < 1e-14
    assert out.e_estimate == 0.0


def test_energy_is_h0_when_h1_and_chol_zero():
    """tests/test_trial_rhf.py:91-113."""
    rng = np.random.default_rng(3)
    m = _zero_ham_model(5, 2, 4, 1.234, 0.01)
    c = _rand_orthonormal(rng, 5, 2)
    mo = np.real(c) if False else np.eye(5)[:, :2]
    w = (mo @ (np.eye(2) * (1.1 + 0.2j)))[None]
    np.testing.assert_allclose(orc.energy_rhf_r(w, mo, 1.234, m.meas), 1.234, rtol=1e-14)
    np.testing.assert_allclose(orc.energy_rhf_u(w, w, mo, 1.234, m.meas), 1.234, rtol=1e-14)


def test_force_bias_hand_formula_and_restricted_equals_unrestricted():
    """tests/test_trial_rhf.py:52-89."""
    ss = synthetic.make_system(6, (3, 3), 5, seed=2)
    ctx = orc.build_rhf_meas_ctx(ss.h1, ss.chol, ss.mo_a)
    rng = np.random.default_rng(4)
    A = rng.normal(size=(3, 3)) + 1.5 * np.eye(3)
    w = (ss.mo_a @ A)[None].astype(np.complex128)
    fb = orc.force_bias_rhf_r(w, ss.mo_a, ctx)
    m = ss.mo_a.T @ w[0]
    g = np.linalg.solve(m.T, w[0].T)
    np.testing.assert_allclose(fb[0], 2.0 * ctx.rot_chol_flat @ g.reshape(-1), rtol=1e-13)
    np.testing.assert_allclose(orc.force_bias_rhf_u(w, w, ss.mo_a, ctx), fb, rtol=1e-13)
    e_r = orc.energy_rhf_r(w, ss.mo_a, 0.5, ctx)
    e_u = orc.energy_rhf_u(w, w, ss.mo_a, 0.5, ctx)
    np.testing.assert_allclose(e_u, e_r, rtol=1e-13)
    uctx = orc.build_uhf_meas_ctx(ss.h1, ss.chol, ss.mo_a, ss.mo_a)
    np.testing.assert_allclose(orc.energy_uhf_u(w, w, ss.mo_a, ss.mo_a, 0.5, uctx), e_r, rtol=1e-13)


def test_step_equals_manual_trotter_with_zero_force_bias():
    """tests/test_prop_afqmc_step.py:85-146: with zero force bias and zero
    mean-field shift the step applies the Trotter propagator to the raw fields."""
    rng = np.random.default_rng(42)
    norb, nocc, nw, nf, dt = 5, 2, 6, 4, 0.1
    a = rng.normal(size=(norb, norb))
    h1 = 0.05 * (a + a.T)
    chol = 0.02 * rng.normal(size=(nf, norb, norb))
    chol = 0.5 * (chol + chol.transpose(0, 2, 1))
    prop = orc.build_prop_ctx(0.0, h1, chol, np.zeros((2, norb, norb)), dt)
    w = rng.normal(size=(nw, norb, nocc)) + 1j * rng.normal(size=(nw, norb, nocc))
    x = rng.normal(size=(nw, nf))
    # zero-rot_chol measurement context -> zero force bias; mf = 0 because rdm1 = 0
    mo = np.eye(norb)[:, :nocc]
    meas = orc.RhfMeasCtx(np.zeros((nocc, norb)), np.zeros((nf, nocc, norb)), np.zeros((nf, nocc * norb)))
    m = orc.Model("rhf_r", 0.0, mo, meas, prop)
    st = orc.State(w, np.ones(nw), m.overlap(w), 0.0, 0.0, 0)
    out = orc.afqmc_step(st, m, orc.Params(dt=dt), x)
    np.testing.assert_allclose(out.walkers, orc.apply_trotter_r(w, x + 0j, prop, 6), rtol=1e-13)


# ------------------------------------------------------------------ same invariants on the GPU

@pytest.mark.gpu
def test_gpu_weight_update_known_answer():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tests.gpu_helpers import Setup, cpu, dev

    norb, nocc, nw, nf, dt = 4, 2, 8, 3, 0.2
    S = Setup("rhf_r", 1.0, np.zeros((norb, norb)), np.zeros((nf, norb, norb)), np.eye(norb)[:, :nocc],
              np.eye(norb)[:, :nocc], dt, nw)
    w = np.ones((nw, norb, nocc), dtype=np.complex128)
    w[:, :nocc, :] += np.eye(nocc)
    wd = dev(w)
    st = S.state(wd, np.ones(nw), cpu(S.overlap(wd)), 0.0, 0.0)
    st = S.step(st, dev(np.random.default_rng(0).normal(size=(nw, nf))))
    np.testing.assert_allclose(cpu(st.weights), np.exp(-dt) * np.ones(nw), rtol=1e-14)
    assert abs(float(st.pop_control_ene_shift) - 0.1) < 1e-13
    assert float(st.e_estimate) == 0.0


@pytest.mark.gpu
def test_gpu_energy_is_h0_when_h1_and_chol_zero():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tests.gpu_helpers import Setup, cpu, dev

    mo = np.eye(5)[:, :2]
    w = dev((mo @ (np.eye(2) * (1.1 + 0.2j)))[None])
    for kind, walkers in (("rhf_r", w), ("rhf_u", (w, w))):
        S = Setup(kind, 1.234, np.zeros((5, 5)), np.zeros((4, 5, 5)), mo, mo, 0.01, 1)
        np.testing.assert_allclose(cpu(S.energy(walkers)), 1.234, rtol=1e-14)


@pytest.mark.gpu
def test_gpu_restricted_equals_unrestricted():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from tests.gpu_helpers import Setup, cpu, dev

    ss = synthetic.make_system(12, (4, 4), 20, seed=5)
    w = dev(synthetic.perturbed_walkers(ss.mo_a, 6, 0.2, 9))
    R = Setup("rhf_r", 0.3, ss.h1, ss.chol, ss.mo_a, ss.mo_a, 0.01, 6)
    U = Setup("rhf_u", 0.3, ss.h1, ss.chol, ss.mo_a, ss.mo_a, 0.01, 6)
    H = Setup("uhf_u", 0.3, ss.h1, ss.chol, ss.mo_a, ss.mo_a, 0.01, 6)
    for a, b in ((R.force_bias(w), U.force_bias((w, w))), (R.energy(w), U.energy((w, w))),
                 (R.energy(w), H.energy((w, w))), (R.overlap(w), U.overlap((w, w)))):
        np.testing.assert_allclose(cpu(b), cpu(a), rtol=1e-12)
