"""CISD trial on the GPU (FP64) vs the reference's golden vectors and the CISD oracle.

Tolerance: 1e-10 relative (max |diff| / max |reference|) for overlaps, force
bias, local energies, 1-RDMs, walkers and weights."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as ao
from oracle import cisd_oracle as co
from tests.conftest import load_golden
from tests.gpu_helpers import cpu, dev, rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


class CisdSetup:
    def __init__(self, h0, h1, chol, ci1, ci2, W, dt=0.005, mixed=False):
        import trot_gb300 as tg

        N, n = h1.shape[0], ci1.shape[0]
        self.sys = tg.System(norb=N, nelec=(n, n), walker_kind="restricted")
        self.ham = tg.HamChol(h0=h0, h1=h1, chol=chol)
        self.trial = tg.CisdTrial(ci1, ci2)
        self.trial_ops = tg.make_cisd_trial_ops(self.sys)
        if mixed:  # the reference's defaults: float32 gl / l2ci2
            self.meas_ops = tg.make_cisd_meas_ops(self.sys)
        else:
            self.meas_ops = tg.make_cisd_meas_ops(self.sys, memory_mode="high", mixed_precision=False, testing=True)
        self.meas_ctx = self.meas_ops.build_meas_ctx(self.ham, self.trial)
        self.params = tg.QmcParams(dt=dt, n_walkers=W, n_exp_terms=6, seed=3)
        self.prop_ops = tg.make_prop_ops("restricted", "restricted")
        self.prop_ctx = self.prop_ops.build_prop_ctx(self.ham, self.trial_ops.get_rdm1(self.trial), self.params)

    def overlap(self, w):
        return self.trial_ops.overlap(w, self.trial)

    def force_bias(self, w):
        return self.meas_ops.kernels["force_bias"](w, self.ham, self.meas_ctx, self.trial)

    def energy(self, w):
        return self.meas_ops.kernels["energy"](w, self.ham, self.meas_ctx, self.trial)

    def rdm1(self, w):
        return self.meas_ops.observables["rdm1"](w, self.ham, self.meas_ctx, self.trial)


@pytest.mark.parametrize("name", ["cisd_small", "cisd_n20"])
def test_cisd_golden(name):
    g = load_golden(name)
    S = CisdSetup(float(g["h0"]), g["h1"], g["chol"], g["ci1"], g["ci2"], g["walkers"].shape[0])
    w = dev(g["walkers"])
    assert rel(cpu(S.overlap(w)), g["overlap"]) <= TOL
    assert rel(cpu(S.meas_ops.overlap(w, S.trial)), g["overlap_meas"]) <= TOL
    assert rel(cpu(S.force_bias(w)), g["force_bias"]) <= TOL
    assert rel(cpu(S.energy(w)), g["energy"]) <= TOL
    assert rel(cpu(S.rdm1(w)), g["rdm1"]) <= TOL


def _synthetic(N, n, G, W, noise, seed=0):
    from trot_gb300 import synthetic

    cs = synthetic.make_cisd_system(N, n, G, seed=seed, h0=0.4)
    w = synthetic.perturbed_walkers(np.eye(N)[:, :n], W, noise, seed + 5)
    return cs, w


@pytest.mark.parametrize("N,n,G,W,noise", [(60, 8, 300, 5, 0.1), (31, 6, 70, 37, 0.3), (9, 2, 11, 3, 0.05),
                                           (44, 11, 130, 4, 0.2)])
def test_cisd_vs_oracle(N, n, G, W, noise):
    cs, w = _synthetic(N, n, G, W, noise)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W)
    tr = co.CisdTrial(cs.ci1, cs.ci2)
    wd = dev(w)
    assert rel(cpu(S.overlap(wd)), co.overlap(w, tr)) <= TOL
    assert rel(cpu(S.force_bias(wd)), co.force_bias(w, tr, cs.chol)) <= TOL
    assert rel(cpu(S.energy(wd)), co.energy(w, tr, cs.h0, cs.h1, cs.chol)) <= TOL
    assert rel(cpu(S.rdm1(wd))[:, 0], co.rdm1(w, tr)) <= TOL


@pytest.mark.parametrize("mixed", [False, True])
def test_cisd_symmetric_and_general_cholesky(mixed):
    """The Cholesky contraction runs over the packed upper triangle only when every
    Cholesky matrix is symmetric to working precision; a general (non-symmetric) set
    takes the full N^2 contraction and still matches the oracle."""
    N, n, G, W = 24, 5, 40, 6
    cs, w = _synthetic(N, n, G, W, 0.1, seed=3)
    tr = co.CisdTrial(cs.ci1, cs.ci2)
    wd = dev(w)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W, mixed=mixed)
    assert S.meas_ctx.chol_symmetric
    skew = np.random.default_rng(8).normal(scale=1e-3, size=cs.chol.shape)
    chol_g = cs.chol + (skew - skew.transpose(0, 2, 1))
    Sg = CisdSetup(cs.h0, cs.h1, chol_g, cs.ci1, cs.ci2, W, mixed=mixed)
    assert not Sg.meas_ctx.chol_symmetric
    e_tol = 1e-5 if mixed else TOL  # mixed: FP32-class gl and l2ci2, absolute Ha
    for setup, chol in ((S, cs.chol), (Sg, chol_g)):
        assert rel(cpu(setup.force_bias(wd)), co.force_bias(w, tr, chol)) <= TOL
        e_ref = co.energy(w, tr, cs.h0, cs.h1, chol)
        e = cpu(setup.energy(wd))
        if mixed:
            assert np.max(np.abs(e - e_ref)) <= e_tol
        else:
            assert rel(e, e_ref) <= TOL


@pytest.mark.parametrize("N,n,G,W,noise", [(60, 8, 300, 6, 0.1), (31, 6, 70, 37, 0.3), (44, 11, 130, 5, 0.2),
                                           (9, 2, 11, 3, 0.05), (31, 6, 70, 37, 0.1)])
def test_cisd_mixed_energy(N, n, G, W, noise):
    """Reference-default meas ops (tensor-core l2ci2 and FP32 gl, FP32-level like the
    reference's float32 there).  Per walker against the FP64 path: |dE_L| <= 1e-5 Ha
    for walkers near the trial (noise <= 0.1); for strongly perturbed walkers
    |dE_L| <= 1e-5 max|E_L| (observed 2.3e-6 relative at noise 0.3).  Force bias and
    overlaps are computed in FP64 either way."""
    cs, w = _synthetic(N, n, G, W, noise)
    F = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W)
    M = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W, mixed=True)
    wd = dev(w)
    e64, emx = cpu(F.energy(wd)), cpu(M.energy(wd))
    err = np.max(np.abs(emx - e64))
    bound = 1e-5 if noise <= 0.1 else 1e-5 * np.max(np.abs(e64))
    assert err <= bound, (err, bound)
    assert rel(cpu(M.force_bias(wd)), cpu(F.force_bias(wd))) <= 1e-12
    assert rel(cpu(M.overlap(wd)), cpu(F.overlap(wd))) <= 1e-14


def test_cisd_step_and_block_vs_oracle():
    """One phaseless step, then a block (2 steps, QR, energy, SR) with injected
    fields and zeta, against the generic oracle step driven by the CISD model."""
    from trot_gb300 import synthetic

    N, n, G, W = 24, 4, 60, 16
    cs, w = _synthetic(N, n, G, W, 0.05, seed=2)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W, dt=0.01)
    tr = co.CisdTrial(cs.ci1, cs.ci2)
    mo = np.eye(N)[:, :n]
    prop = ao.build_prop_ctx(cs.h0, cs.h1, cs.chol, np.stack([mo @ mo.T, mo @ mo.T]), 0.01)
    model = co.CisdModel(tr, cs.h0, cs.h1, cs.chol, prop)
    p = ao.Params(dt=0.01, n_prop_steps=2)
    ov = co.overlap(w, tr)
    e0 = float(np.real(co.energy(w[:1], tr, cs.h0, cs.h1, cs.chol))[0])
    weights = 0.5 + np.random.default_rng(1).uniform(size=W)
    fields = synthetic.fields(W, G, 3, seed=11)

    import trot_gb300 as tg

    state = tg.PropState(walkers=dev(w), weights=dev(weights), overlaps=dev(ov), rng_key=tg.rng.key(0),
                         scalars=dev(np.array([e0 - 0.2, e0])), node_encounters=dev(np.zeros(1, np.int64)))
    energy = torch.empty(W, dtype=torch.complex128, device="cuda")
    state = S.prop_ops.step(state, params=S.params, ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops,
                            meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ctx=S.prop_ctx,
                            fields=dev(fields[0]), energy_out=energy)
    ref = ao.afqmc_step(ao.State(w, weights, ov, e0 - 0.2, e0), model, p, fields[0])
    assert rel(cpu(energy), co.energy(w, tr, cs.h0, cs.h1, cs.chol)) <= TOL
    assert rel(cpu(state.walkers), ref.walkers) <= TOL
    assert rel(cpu(state.overlaps), ref.overlaps) <= TOL
    assert rel(cpu(state.weights), ref.weights) <= TOL
    assert abs(float(cpu(state.scalars)[0]) - ref.pop_control_ene_shift) <= 1e-10 * abs(ref.pop_control_ene_shift)
    assert int(cpu(state.node_encounters)[0]) == ref.node_encounters

    zeta = 0.37
    st2, obs = tg.block(state, sys=S.sys, params=tg.QmcParams(dt=0.01, n_walkers=W, n_prop_steps=2, seed=3),
                        ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops, meas_ops=S.meas_ops,
                        meas_ctx=S.meas_ctx, prop_ops=S.prop_ops, prop_ctx=S.prop_ctx,
                        fields_seq=dev(fields[1:]), zeta=torch.tensor([zeta], dtype=torch.float64, device="cuda"))
    rb, e_block, w_sum = ao.block(ref, model, p, fields[1:], zeta)
    assert rel(cpu(st2.walkers), rb.walkers) <= TOL
    assert rel(cpu(st2.weights), rb.weights) <= TOL
    assert rel(cpu(st2.overlaps), rb.overlaps) <= TOL
    assert abs(float(obs.scalars["energy"]) - e_block) <= 1e-10 * abs(e_block)


def test_cisd_init_prop_state():
    import trot_gb300 as tg

    cs, _ = _synthetic(20, 5, 40, 1, 0.0, seed=6)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, 8)
    st = S.prop_ops.init_prop_state(sys=S.sys, ham_data=S.ham, trial_ops=S.trial_ops, trial_data=S.trial,
                                    meas_ops=S.meas_ops, params=S.params)
    tr = co.CisdTrial(cs.ci1, cs.ci2)
    w = cpu(st.walkers)
    assert rel(cpu(st.overlaps), co.overlap(w, tr)) <= TOL
    e = float(np.real(co.energy(w[:1], tr, cs.h0, cs.h1, cs.chol))[0])
    assert abs(float(cpu(st.scalars)[1]) - e) <= 1e-10 * abs(e)


def test_cisd_rejects_bad_inputs():
    import trot_gb300 as tg

    cs, w = _synthetic(12, 3, 20, 2, 0.1)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, 2)
    with pytest.raises(ValueError):
        S.energy(dev(w[:, :, :2]))
    with pytest.raises(TypeError):
        S.energy((dev(w), dev(w)))
    with pytest.raises(ValueError):
        tg.make_cisd_meas_ops(tg.System(norb=12, nelec=(3, 3), walker_kind="unrestricted"))
    core = tg.CisdTrial(cs.ci1[1:], cs.ci2[1:, :, 1:, :], nocc_t_core=1)
    with pytest.raises(NotImplementedError):
        S.trial_ops.overlap(dev(w), core)


def test_cisd_step_mixed_propagation():
    """Tensor-core VHS / Taylor action in the CISD step: walkers within 2e-5 relative of the FP64
    step on the same fields; weights within 1e-3 on live walkers; same local energy (FP64 meas)."""
    import trot_gb300 as tg
    from trot_gb300 import synthetic

    N, n, G, W = 40, 6, 100, 24
    cs, w = _synthetic(N, n, G, W, 0.05, seed=3)
    S = CisdSetup(cs.h0, cs.h1, cs.chol, cs.ci1, cs.ci2, W, dt=0.01)
    pm = tg.make_prop_ops("restricted", "restricted", mixed_precision=True)
    pcm = pm.build_prop_ctx(S.ham, S.trial_ops.get_rdm1(S.trial), S.params)
    ov = cpu(S.overlap(dev(w)))
    fields = dev(synthetic.fields(W, G, 1, seed=4)[0])

    def run(ops, ctx):
        st = tg.PropState(walkers=dev(w), weights=dev(np.ones(W)), overlaps=dev(ov), rng_key=tg.rng.key(0),
                          scalars=dev(np.array([0.1, 0.1])), node_encounters=dev(np.zeros(1, np.int64)))
        e = torch.empty(W, dtype=torch.complex128, device="cuda")
        st = ops.step(st, params=S.params, ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops,
                      meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ctx=ctx, fields=fields, energy_out=e)
        return st, e

    s64, e64 = run(S.prop_ops, S.prop_ctx)
    smx, emx = run(pm, pcm)
    assert rel(cpu(smx.walkers), cpu(s64.walkers)) <= 2e-5
    assert np.array_equal(cpu(emx), cpu(e64))
    wf, wm = cpu(s64.weights), cpu(smx.weights)
    assert np.array_equal(wf > 0, wm > 0)
    live = wf > 0
    if live.any():
        assert rel(wm[live], wf[live]) <= 1e-3
