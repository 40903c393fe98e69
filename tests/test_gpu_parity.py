"""FP64 CUDA path vs the reference's golden vectors and the CPU oracle.

Tolerance: 1e-10 relative (the FP64 parity bar) unless stated."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from tests.golden_model import model_from_golden, state_from_golden, walkers_from_golden
from tests.gpu_helpers import Setup, cpu, dev, rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _w(g, prefix=""):
    w = walkers_from_golden(g, prefix)
    return (dev(w[0]), dev(w[1])) if isinstance(w, tuple) else dev(w)


def test_overlap_force_bias_energy_vs_golden(golden):
    S = Setup.from_golden(golden)
    w = _w(golden)
    assert rel(cpu(S.overlap(w)), golden["overlap"]) < TOL
    assert rel(cpu(S.force_bias(w)), golden["force_bias"]) < TOL
    assert rel(cpu(S.energy(w)), golden["energy"]) < TOL


def test_prop_ctx_vs_golden(golden):
    S = Setup.from_golden(golden)
    assert rel(cpu(S.prop_ctx.mf_shifts), golden["mf_shifts"]) < 1e-12
    assert rel(cpu(S.prop_ctx.exp_h1_half), golden["exp_h1_half"]) < 1e-12
    assert abs(S.prop_ctx.h0_prop - complex(golden["h0_prop"]).real) < 1e-10


def test_trotter_vs_golden(golden):
    import trot_gb300 as tg

    S = Setup.from_golden(golden)
    ops = tg.make_trotter_ops("restricted", S.walker_kind)
    out = ops.apply_trotter(_w(golden), dev(golden["trotter_fields"]), S.prop_ctx, 6)
    if S.kind == "rhf_r":
        assert rel(cpu(out), golden["trotter_out"]) < TOL
    else:
        assert rel(cpu(out[0]), golden["trotter_out_u"]) < TOL
        assert rel(cpu(out[1]), golden["trotter_out_d"]) < TOL


def _check_state(st, g, prefix, kind):
    w = walkers_from_golden(g, prefix)
    if kind == "rhf_r":
        assert rel(cpu(st.walkers), w) < TOL
    else:
        assert rel(cpu(st.walkers[0]), w[0]) < TOL
        assert rel(cpu(st.walkers[1]), w[1]) < TOL
    assert rel(cpu(st.weights), g[prefix + "weights"]) < TOL
    assert rel(cpu(st.overlaps), g[prefix + "overlaps"]) < TOL
    assert abs(float(st.pop_control_ene_shift) - float(g[prefix + "shift"])) < 1e-8
    assert abs(float(st.e_estimate) - float(g[prefix + "e_estimate"])) < 1e-8
    assert int(st.node_encounters.item()) == int(g[prefix + "nodes"])


def _state(S, g):
    return S.state(_w(g), g["state_weights"], g["overlap"], float(g["state_shift"]), float(g["state_e_estimate"]))


def test_step_vs_golden(golden):
    S = Setup.from_golden(golden)
    st = S.step(_state(S, golden), dev(golden["step_fields"][0]))
    _check_state(st, golden, "step1_", S.kind)


def test_block_vs_golden(golden):
    import trot_gb300 as tg

    S = Setup.from_golden(golden)
    params = tg.QmcParams(dt=float(golden["dt"]), n_prop_steps=golden["step_fields"].shape[0],
                          n_walkers=S.params.n_walkers, seed=1)
    st, obs = tg.block(_state(S, golden), sys=S.sys, params=params, ham_data=S.ham, trial_data=S.trial,
                       trial_ops=S.trial_ops, meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ops=S.prop_ops,
                       prop_ctx=S.prop_ctx, fields_seq=dev(golden["step_fields"]), zeta=float(golden["zeta"]))
    _check_state(st, golden, "block_", S.kind)
    assert abs(float(obs.scalars["energy"]) - float(golden["block_energy"])) < 1e-9 * max(1, abs(float(golden["block_energy"])))
    assert abs(float(obs.scalars["weight"]) - float(golden["block_weight"])) < 1e-11 * float(golden["block_weight"])


def test_block_rdm1_vs_golden(golden):
    """The block's rdm1 observable (the reference's weighted rdm1_kernel_* average)."""
    import trot_gb300 as tg

    S = Setup.from_golden(golden)
    params = tg.QmcParams(dt=float(golden["dt"]), n_prop_steps=golden["step_fields"].shape[0],
                          n_walkers=S.params.n_walkers, seed=1)
    _, obs = tg.block(_state(S, golden), sys=S.sys, params=params, ham_data=S.ham, trial_data=S.trial,
                      trial_ops=S.trial_ops, meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ops=S.prop_ops,
                      prop_ctx=S.prop_ctx, fields_seq=dev(golden["step_fields"]), zeta=float(golden["zeta"]),
                      observable_names=("rdm1",))
    assert rel(cpu(obs.observables["rdm1"]), golden["block_rdm1"]) < 1e-10


def test_qr_sr_vs_golden(golden):
    import trot_gb300 as tg

    S = Setup.from_golden(golden)
    w = _w(golden)
    q, norm = tg.walkers.orthogonalize(w, S.walker_kind)
    if S.kind == "rhf_r":
        assert rel(cpu(q), golden["qr_out"]) < 1e-12
    else:
        assert rel(cpu(q[0]), golden["qr_out_u"]) < 1e-12
        assert rel(cpu(q[1]), golden["qr_out_d"]) < 1e-12
    assert rel(cpu(norm), golden["qr_norm"]) < 1e-12
    wsr, wts, idx = tg.walkers.stochastic_reconfiguration(w, dev(golden["sr_weights_in"]), float(golden["sr_zeta"]),
                                                          S.walker_kind, return_indices=True)
    np.testing.assert_array_equal(cpu(idx), golden["sr_idx"])
    np.testing.assert_array_equal(cpu(wts), golden["sr_weights_out"])
    src = walkers_from_golden(golden)
    if S.kind == "rhf_r":
        np.testing.assert_array_equal(cpu(wsr), src[golden["sr_idx"]])
    else:
        np.testing.assert_array_equal(cpu(wsr[0]), src[0][golden["sr_idx"]])
        np.testing.assert_array_equal(cpu(wsr[1]), src[1][golden["sr_idx"]])


# ---------------------------------------------------------------- oracle at larger / odd sizes

SIZES = [
    # kind, N, (na, nb), G, W
    ("rhf_r", 7, (3, 3), 5, 3),
    ("rhf_r", 24, (5, 5), 120, 64),
    ("rhf_u", 13, (4, 4), 9, 2),
    ("uhf_u", 17, (5, 3), 33, 5),
    ("uhf_u", 40, (6, 5), 96, 7),
    ("rhf_r", 9, (1, 1), 1, 1),
]


def _synthetic(kind, N, nelec, G, W, seed=11):
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=seed, h0=0.3)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.2, seed + 1)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.2, seed + 2)
    walkers = wa if kind == "rhf_r" else (wa, wb)
    return ss, walkers


def _oracle_model(kind, ss, dt):
    rdm1 = ss.rdm1()
    prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, rdm1, dt)
    if kind == "uhf_u":
        return orc.Model(kind, ss.h0, (ss.mo_a, ss.mo_b), orc.build_uhf_meas_ctx(ss.h1, ss.chol, ss.mo_a, ss.mo_b), prop)
    return orc.Model(kind, ss.h0, ss.mo_a, orc.build_rhf_meas_ctx(ss.h1, ss.chol, ss.mo_a), prop)


@pytest.mark.parametrize("kind,N,nelec,G,W", SIZES)
def test_measurements_vs_oracle(kind, N, nelec, G, W):
    ss, walkers = _synthetic(kind, N, nelec, G, W)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.01, W)
    m = _oracle_model(kind, ss, 0.01)
    w = S.walkers(walkers)
    assert rel(cpu(S.overlap(w)), m.overlap(walkers)) < TOL
    assert rel(cpu(S.force_bias(w)), m.force_bias(walkers)) < TOL
    assert rel(cpu(S.energy(w)), m.energy(walkers)) < TOL


@pytest.mark.parametrize("kind,N,nelec,G,W", SIZES)
def test_steps_vs_oracle(kind, N, nelec, G, W):
    from trot_gb300 import synthetic

    ss, walkers = _synthetic(kind, N, nelec, G, W)
    dt = 0.01
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, W)
    m = _oracle_model(kind, ss, dt)
    ov = m.overlap(walkers)
    e0 = float(np.real(m.energy(walkers))[0])
    ost = orc.State(walkers, np.ones(W), ov, e0, e0, 0)
    st = S.state(S.walkers(walkers), np.ones(W), ov, e0, e0)
    fields = synthetic.fields(W, G, 4, seed=5)
    params = orc.Params(dt=dt)
    e_out = torch.empty(W, dtype=torch.complex128, device="cuda")
    for k in range(4):
        e_ref = m.energy(ost.walkers)
        ost = orc.afqmc_step(ost, m, params, fields[k])
        st = S.step(st, dev(fields[k]), energy_out=e_out)
        assert rel(cpu(e_out), e_ref) < TOL
    if kind == "rhf_r":
        assert rel(cpu(st.walkers), ost.walkers) < TOL
    else:
        assert rel(cpu(st.walkers[0]), ost.walkers[0]) < TOL
        assert rel(cpu(st.walkers[1]), ost.walkers[1]) < TOL
    assert rel(cpu(st.weights), ost.weights) < TOL
    assert rel(cpu(st.overlaps), ost.overlaps) < TOL
    assert abs(float(st.pop_control_ene_shift) - ost.pop_control_ene_shift) < 1e-8 * max(1, abs(ost.pop_control_ene_shift))
    assert int(st.node_encounters.item()) == ost.node_encounters


def test_chunk_invariance():
    """vmap_chunked over batched kernels gives the same numbers for any n_chunks
    (trot tests/test_walkers.py, tests/test_prop_afqmc_step.py:148-162)."""
    import trot_gb300 as tg

    ss, walkers = _synthetic("uhf_u", 16, (4, 3), 20, 9)
    S = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.01, 9)
    w = S.walkers(walkers)
    fb = S.meas_ops.kernels["force_bias"]
    ref = cpu(tg.walkers.vmap_chunked(fb, 1, in_axes=(0, None, None, None))(w, S.ham, S.meas_ctx, S.trial))
    for nc in (2, 3, 4):
        out = cpu(tg.walkers.vmap_chunked(fb, nc, in_axes=(0, None, None, None))(w, S.ham, S.meas_ctx, S.trial))
        assert rel(out, ref) < 1e-15


def test_deterministic_repeat():
    """Fixed-order reductions: two runs give bitwise-identical results."""
    ss, walkers = _synthetic("uhf_u", 30, (6, 4), 64, 16)
    S = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.01, 16)
    w = S.walkers(walkers)
    e1, e2 = cpu(S.energy(w)), cpu(S.energy(w))
    np.testing.assert_array_equal(e1, e2)
