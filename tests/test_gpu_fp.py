"""Free-projection step on the GPU vs the reference's golden vectors and the oracle.

Tolerances: FP64 path 1e-10 relative (walkers, weights); mixed path (tensor-core
VHS / Taylor action) 2e-5 relative in the walkers and 1e-4 in the weights."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as ao
from tests.conftest import load_golden
from tests.gpu_helpers import cpu, dev, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _setup(kind, h0, h1, chol, mo_a, mo_b, dt, ene0, W, mixed=False):
    import trot_gb300 as tg
    from trot_gb300.prop_fp import make_prop_ops_fp

    wk = "restricted" if kind == "rhf_r" else "unrestricted"
    N = h1.shape[0]
    sysm = tg.System(norb=N, nelec=(mo_a.shape[1], mo_b.shape[1]), walker_kind=wk)
    ham = tg.HamChol(h0=h0, h1=h1, chol=chol)
    if kind == "uhf_u":
        trial, trial_ops = tg.UhfTrial(mo_a, mo_b), tg.make_uhf_trial_ops(sysm)
    else:
        trial, trial_ops = tg.RhfTrial(mo_a), tg.make_rhf_trial_ops(sysm)
    params = tg.QmcParamsFp(dt=dt, n_walkers=W, ene0=ene0, seed=1)
    ops = make_prop_ops_fp("restricted", wk, sysm, mixed_precision=mixed)
    ctx = ops.build_prop_ctx(ham, trial_ops.get_rdm1(trial), params)
    return dict(tg=tg, sys=sysm, ham=ham, trial=trial, trial_ops=trial_ops, params=params, ops=ops, ctx=ctx, wk=wk)


def _run(S, walkers, weights, fields, zeta):
    tg = S["tg"]
    W = len(weights)
    w = tuple(dev(x) for x in walkers) if isinstance(walkers, tuple) else dev(walkers)
    st = tg.PropState(walkers=w, weights=dev(weights), overlaps=torch.ones(W, dtype=torch.complex128, device="cuda"),
                      rng_key=tg.rng.key(0), scalars=dev(np.zeros(2)), node_encounters=dev(np.zeros(1, np.int64)))
    st = S["ops"].step(st, params=S["params"], ham_data=S["ham"], trial_data=S["trial"], trial_ops=S["trial_ops"],
                       meas_ops=None, meas_ctx=None, prop_ctx=S["ctx"], fields=dev(fields),
                       zeta=torch.tensor([zeta], dtype=torch.float64, device="cuda"))
    return st


@pytest.mark.parametrize("name", ["fp_rhf_r", "fp_uhf_u"])
def test_fp_step_golden(name):
    g = load_golden(name)
    kind = str(g["kind"])
    w = g["walkers"] if kind == "rhf_r" else (g["walkers_u"], g["walkers_d"])
    S = _setup(kind, float(g["h0"]), g["h1"], g["chol"], g["mo_a"], g["mo_b"], float(g["dt"]), float(g["ene0"]),
               len(g["weights"]))
    assert abs(S["ctx"].h0_prop - float(np.real(g["h0_prop"]))) <= 1e-12 * abs(S["ctx"].h0_prop)
    st = _run(S, w, g["weights"], g["fields"], float(g["zeta"]))
    assert rel(cpu(st.weights), g["out_weights"]) <= 1e-10
    if kind == "rhf_r":
        assert rel(cpu(st.walkers), g["out_walkers"]) <= 1e-10
    else:
        assert rel(cpu(st.walkers[0]), g["out_walkers_u"]) <= 1e-10
        assert rel(cpu(st.walkers[1]), g["out_walkers_d"]) <= 1e-10


@pytest.mark.parametrize("kind,N,nelec,G,W", [("uhf_u", 60, (8, 6), 150, 40), ("rhf_r", 40, (7, 7), 90, 33)])
def test_fp_step_vs_oracle_and_mixed(kind, N, nelec, G, W):
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=4, h0=0.3)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 5)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 6)
    walkers = wa if kind == "rhf_r" else (wa, wb)
    rng = np.random.default_rng(2)
    weights = 0.5 + rng.uniform(size=W)
    fields = rng.standard_normal((W, G))
    zeta = 0.61
    dt, ene0 = 0.02, -0.7
    F = _setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, ene0, W)
    st = _run(F, walkers, weights, fields, zeta)
    dm = np.stack([ss.mo_a @ ss.mo_a.T, ss.mo_b @ ss.mo_b.T]) if kind == "uhf_u" else np.stack([ss.mo_a @ ss.mo_a.T] * 2)
    prop = ao.build_prop_ctx(ss.h0, ss.h1, ss.chol, dm, dt)
    prop = ao.PropCtx(prop.dt, prop.sqrt_dt, prop.exp_h1_half, prop.mf_shifts, prop.h0_prop + ene0, prop.chol_flat,
                      prop.norb)
    model = ao.Model(kind, ss.h0, ss.mo_a if kind != "uhf_u" else (ss.mo_a, ss.mo_b), None, prop)
    ref = ao.afqmc_step_fp(ao.State(walkers, weights, np.ones(W, complex), 0.0, 0.0), model, fields, zeta)
    assert rel(cpu(st.weights), ref.weights) <= 1e-10
    if kind == "rhf_r":
        assert rel(cpu(st.walkers), ref.walkers) <= 1e-10
    else:
        assert rel(cpu(st.walkers[0]), ref.walkers[0]) <= 1e-10
        assert rel(cpu(st.walkers[1]), ref.walkers[1]) <= 1e-10
    M = _setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, ene0, W, mixed=True)
    sm = _run(M, walkers, weights, fields, zeta)
    # same resampling indices (the weights differ only at the 1e-6 level)
    assert rel(cpu(sm.weights), ref.weights) <= 1e-4
    if kind == "rhf_r":
        assert rel(cpu(sm.walkers), ref.walkers) <= 2e-5
    else:
        assert rel(cpu(sm.walkers[0]), ref.walkers[0]) <= 2e-5
