"""FP64 CUDA path vs the CPU oracle at the benchmark workloads' shapes, the
reference's numeric guards, and the product's init_walkers vs the golden
vectors of the reference's own init_walkers.

Tolerance: 1e-10 relative (the FP64 parity bar) unless stated."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from tests.gpu_helpers import Setup, cpu, dev, rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _model(kind, ss, dt):
    rdm1 = ss.rdm1()
    prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, rdm1, dt)
    if kind == "uhf_u":
        return orc.Model(kind, ss.h0, (ss.mo_a, ss.mo_b), orc.build_uhf_meas_ctx(ss.h1, ss.chol, ss.mo_a, ss.mo_b), prop)
    return orc.Model(kind, ss.h0, ss.mo_a, orc.build_rhf_meas_ctx(ss.h1, ss.chol, ss.mo_a), prop)


def _cmp_walkers(kind, got, ref, tol=TOL):
    if kind == "rhf_r":
        assert rel(cpu(got), ref) < tol
    else:
        assert rel(cpu(got[0]), ref[0]) < tol
        assert rel(cpu(got[1]), ref[1]) < tol


# The benchmark workloads' shapes with their own recipes (decay length, dt), a few walkers:
#   UHF N=120 (12, 10) G=600 decay 150 dt 0.005 (the mixed-precision headline workload's system);
#   RHF N=80 n=10 G=400 decay 30 dt 0.01 (the energy-gradient workload's system);
#   RHF N=160 n=19 G=640 (the largest fragment of the 24-fragment batch: N in [30, 160],
#   n = round(0.12 N), G = 4 N); N > 128 and n > 16 take the general FP64 kernels.  With this
#   recipe at N = 160 the walkers grow by ~10^6 per step (sqrt(dt) ||VHS|| >> 1), so the
#   relative rounding differences of two FP64 implementations grow with every step: two steps
#   there, three elsewhere.
SHAPES = [
    ("uhf_u", 120, (12, 10), 600, 150.0, 0.005, 8, 3),
    ("rhf_r", 80, (10, 10), 400, 30.0, 0.01, 8, 3),
    ("rhf_r", 160, (19, 19), 640, 30.0, 0.005, 4, 2),
]


@pytest.mark.parametrize("kind,N,nelec,G,decay,dt,W,n_steps", SHAPES)
def test_benchmark_shapes_vs_oracle(kind, N, nelec, G, decay, dt, W, n_steps):
    """Overlaps, force bias, local energy and phaseless steps (walkers, weights,
    overlaps, shift, node count, E_L of the incoming walkers) against the oracle
    on identical injected fields."""
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, nelec, G, decay=decay, seed=0, h0=0.0)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.05, 31)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.05, 32)
    walkers = wa if kind == "rhf_r" else (wa, wb)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, W)
    m = _model(kind, ss, dt)
    w = S.walkers(walkers)
    assert rel(cpu(S.overlap(w)), m.overlap(walkers)) < TOL
    assert rel(cpu(S.force_bias(w)), m.force_bias(walkers)) < TOL
    assert rel(cpu(S.energy(w)), m.energy(walkers)) < TOL
    ov = m.overlap(walkers)
    e0 = float(np.real(m.energy(walkers))[0])
    ost = orc.State(walkers, np.ones(W), ov, e0, e0, 0)
    st = S.state(S.walkers(walkers), np.ones(W), ov, e0, e0)
    fields = synthetic.fields(W, G, n_steps, seed=41)
    e_out = torch.empty(W, dtype=torch.complex128, device="cuda")
    for k in range(n_steps):
        e_ref = m.energy(ost.walkers)
        ost = orc.afqmc_step(ost, m, orc.Params(dt=dt), fields[k])
        st = S.step(st, dev(fields[k]), energy_out=e_out)
        assert rel(cpu(e_out), e_ref) < TOL
    _cmp_walkers(kind, st.walkers, ost.walkers)
    assert rel(cpu(st.weights), ost.weights) < TOL
    assert rel(cpu(st.overlaps), ost.overlaps) < TOL
    assert abs(float(st.pop_control_ene_shift) - ost.pop_control_ene_shift) < 1e-8 * max(1, abs(ost.pop_control_ene_shift))
    assert int(st.node_encounters.item()) == ost.node_encounters


# ---------------------------------------------------------------- numeric guards


@pytest.mark.parametrize("kind", ["rhf_r", "uhf_u"])
def test_step_guards_vs_oracle(kind):
    """Guards of afqmc_step (trot/prop/afqmc.py:122-134): a walker whose
    importance ratio is non-finite (NaN orbitals; a zero stored overlap, so
    ratio = ov_new / 0) gets weight 0 and counts as a node encounter; a walker
    whose weight passes the cap gets weight 0; the other walkers are untouched
    and the population shift uses the mean of the guarded weights."""
    from trot_gb300 import synthetic

    N, G, W, dt = 14, 30, 6, 0.01
    nelec = (4, 4) if kind == "rhf_r" else (4, 3)
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=5, h0=0.2)
    m = _model(kind, ss, dt)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 6)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 7)
    wa[1] = np.nan  # walker 1: NaN orbitals
    if kind == "rhf_r":
        walkers = wa
    else:
        wb[1] = np.nan
        walkers = (wa, wb)
    with np.errstate(all="ignore"):
        ov = m.overlap(walkers)
    ov[2] = 0.0  # walker 2: zero stored overlap -> non-finite ratio
    weights = np.ones(W)
    weights[3] = 150.0  # walker 3: weight * importance passes the cap of 100
    e0 = -1.0
    ost = orc.State(walkers, weights.copy(), ov.copy(), 0.0, e0, 0)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, W)
    st = S.state(S.walkers(walkers), weights, ov, 0.0, e0)
    x = synthetic.fields(W, G, 1, seed=8)[0]
    with np.errstate(all="ignore"):
        ost = orc.afqmc_step(ost, m, orc.Params(dt=dt), x)
    st = S.step(st, dev(x))
    wt = cpu(st.weights)
    assert wt[1] == 0.0 and wt[2] == 0.0
    assert ost.weights[1] == 0.0 and ost.weights[2] == 0.0
    np.testing.assert_array_equal(wt == 0.0, ost.weights == 0.0)
    assert int(st.node_encounters.item()) == ost.node_encounters >= 2
    ok = np.isfinite(ost.weights) & (ost.weights > 0)
    assert rel(wt[ok], ost.weights[ok]) < TOL
    assert abs(float(st.pop_control_ene_shift) - ost.pop_control_ene_shift) < 1e-8 * max(1, abs(ost.pop_control_ene_shift))
    # the finite walkers propagate exactly as the oracle's
    good = [b for b in range(W) if b != 1]
    if kind == "rhf_r":
        assert rel(cpu(st.walkers)[good], ost.walkers[good]) < TOL
    else:
        assert rel(cpu(st.walkers[0])[good], ost.walkers[0][good]) < TOL


def _block_energy_ref(e, weights, e_est, dt, alpha):
    """The block's clamp / weighting / EMA (trot/prop/blocks.py:236-257)."""
    e = np.real(e).astype(np.float64)
    with np.errstate(invalid="ignore"):
        is_nan = ~np.isfinite(e)
        e = np.where(is_nan | (np.abs(e - e_est) > np.sqrt(2.0 / dt)), e_est, e)
    w = np.where(is_nan, 0.0, weights)
    ws = float(np.sum(w))
    eb = e_est if ws == 0 else float(np.sum(w * e) / ws)
    return eb, ws, w, (1 - alpha) * e_est + alpha * eb


@pytest.mark.parametrize("case", ["mixed", "all_nan", "zero_weight", "clamped"])
def test_block_energy_guards(case):
    """trot_block_energy: non-finite E_L -> e_estimate and weight 0; |E_L -
    e_estimate| > sqrt(2/dt) -> e_estimate; zero total weight -> block energy =
    e_estimate; then the EMA of e_estimate."""
    from trot_gb300 import _lib, native

    W, dt, alpha, e_est = 9, 0.005, 0.1, -3.0
    rng = np.random.default_rng(3)
    e = (e_est + rng.normal(scale=5.0, size=W)) + 1j * rng.normal(size=W)
    weights = rng.uniform(0.5, 2.0, W)
    if case == "mixed":
        e[1] = np.nan
        e[2] = np.inf + 0j
        e[4] = e_est + 25.0  # beyond sqrt(2/dt) = 20
        e[5] = e_est - 19.0  # inside
        weights[6] = 0.0
    elif case == "all_nan":
        e[:] = np.nan
    elif case == "zero_weight":
        weights[:] = 0.0
    else:
        e[:] = e_est + 1e6
    eb, ws, w_ref, e_new = _block_energy_ref(e, weights, e_est, dt, alpha)
    ed, wd = dev(e), dev(weights)
    sc = dev(np.array([0.7, e_est]))
    obs = torch.empty(2, dtype=torch.float64, device="cuda")
    _lib.call("trot_block_energy", W, ed.data_ptr(), wd.data_ptr(), sc.data_ptr(), float(dt), float(alpha),
              obs.data_ptr(), native.stream_ptr())
    o = cpu(obs)
    assert abs(o[0] - eb) <= 1e-12 * max(1.0, abs(eb))
    assert abs(o[1] - ws) <= 1e-12 * max(1.0, abs(ws))
    np.testing.assert_array_equal(cpu(wd), w_ref)
    s = cpu(sc)
    assert s[0] == 0.7 and abs(s[1] - e_new) <= 1e-12 * max(1.0, abs(e_new))


def test_block_with_dead_walkers_vs_oracle():
    """A whole block (steps, QR, overlaps, energy, clamp, EMA, SR) with a NaN
    walker in the population: its weight drops to 0, SR never selects it, and
    the block energy, weights and e_estimate match the oracle's block."""
    import trot_gb300 as tg
    from trot_gb300 import synthetic

    kind, N, nelec, G, W, dt = "uhf_u", 12, (3, 2), 20, 8, 0.01
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=9, h0=0.1)
    m = _model(kind, ss, dt)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 10)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 11)
    wa[5] = np.nan
    wb[5] = np.nan
    walkers = (wa, wb)
    with np.errstate(all="ignore"):
        ov = m.overlap(walkers)
        e0 = float(np.real(m.energy(walkers))[0])
    ost = orc.State(walkers, np.ones(W), ov.copy(), e0, e0, 0)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, dt, W)
    st = S.state(S.walkers(walkers), np.ones(W), ov, e0, e0)
    fields = synthetic.fields(W, G, 3, seed=12)
    zeta = 0.37
    with np.errstate(all="ignore"):
        ost, eb, ws = orc.block(ost, m, orc.Params(dt=dt), fields, zeta)
    params = tg.QmcParams(dt=dt, n_prop_steps=3, n_walkers=W, seed=1)
    st, obs = tg.block(st, sys=S.sys, params=params, ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops,
                       meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ops=S.prop_ops, prop_ctx=S.prop_ctx,
                       fields_seq=dev(fields), zeta=zeta)
    assert abs(float(obs.scalars["energy"]) - eb) < 1e-9 * max(1, abs(eb))
    assert abs(float(obs.scalars["weight"]) - ws) < 1e-11 * max(1, ws)
    assert rel(cpu(st.weights), ost.weights) < TOL
    assert abs(float(st.e_estimate) - ost.e_estimate) < 1e-9 * max(1, abs(ost.e_estimate))
    assert np.all(np.isfinite(cpu(st.walkers[0]))) and np.all(np.isfinite(ost.walkers[0]))
    _cmp_walkers(kind, st.walkers, ost.walkers)
    assert int(st.node_encounters.item()) == ost.node_encounters


# ---------------------------------------------------------------- init_walkers


def test_init_walkers_vs_golden(golden):
    """The product's init_walkers (natural orbitals of the trial 1-RDM broadcast
    to every walker, trot/walkers.py:20-78) against the reference's own output;
    eigenvectors are unique up to sign, so the projectors w w^H are compared."""
    import trot_gb300 as tg

    kind = str(golden["kind"])
    mo_a, mo_b = golden["mo_a"], golden["mo_b"]
    na, nb = mo_a.shape[1], mo_b.shape[1]
    wk = "restricted" if kind == "rhf_r" else "unrestricted"
    sysm = tg.System(norb=mo_a.shape[0], nelec=(na, nb), walker_kind=wk)
    rdm1 = np.stack([mo_a @ mo_a.T, mo_b @ mo_b.T])
    iw = tg.walkers.init_walkers(sysm, rdm1, 3)
    if kind == "rhf_r":
        pairs = [(cpu(iw), golden["init_walkers"])]
    else:
        pairs = [(cpu(iw[0]), golden["init_walkers_u"]), (cpu(iw[1]), golden["init_walkers_d"])]
    for a, b in pairs:
        assert a.shape[0] == 3 and a.shape[1:] == b.shape[1:]
        pa = a @ np.conj(np.swapaxes(a, -1, -2))
        pb = b[:1] @ np.conj(np.swapaxes(b[:1], -1, -2))
        assert rel(pa, np.broadcast_to(pb, pa.shape)) < 1e-10
    # init_prop_state: overlaps of the initial walkers and e_estimate = E_L of walker 0
    S = Setup.from_golden(golden)
    st = S.prop_ops.init_prop_state(sys=S.sys, ham_data=S.ham, trial_ops=S.trial_ops, trial_data=S.trial,
                                    meas_ops=S.meas_ops, params=S.params)
    w0 = st.walkers
    assert rel(cpu(st.overlaps), cpu(S.overlap(w0))) < 1e-13
    assert abs(float(st.e_estimate) - float(np.real(cpu(S.energy(w0))[0]))) < 1e-10 * max(1, abs(float(st.e_estimate)))
