"""Mixed-precision (tensor-core) path vs the FP64 path on identical walkers.

Tolerances (stated per quantity):
* local energy: |dE_L| <= 1e-5 Ha per walker (the precision target of the path);
* force bias: 1e-9 relative (exact-slice products);
* Trotter propagation (FP32 VHS / Taylor): 2e-5 relative."""
import numpy as np
import pytest
import torch

from tests.gpu_helpers import Setup, cpu, dev, rel

pytestmark = pytest.mark.gpu

CASES = [
    # kind, N, (na, nb), G, W, decay
    ("uhf_u", 120, (12, 10), 600, 12, 150.0),
    ("rhf_r", 24, (5, 5), 120, 20, 30.0),
    ("rhf_u", 24, (5, 5), 120, 7, 30.0),
    ("uhf_u", 17, (5, 3), 33, 9, 30.0),
    ("rhf_r", 7, (3, 3), 5, 3, 30.0),
    ("uhf_u", 80, (16, 9), 300, 13, 30.0),
    # 48.7 KB of dynamic shared memory in the Green's-function kernel: needs the opt-in limit
    ("rhf_r", 117, (14, 14), 468, 5, 30.0),
]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _setups(kind, N, nelec, G, W, decay, noise, seed=3):
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, nelec, G, decay=decay, seed=seed, h0=0.2)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, noise, seed + 1)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, noise, seed + 2)
    walkers = wa if kind == "rhf_r" else (wa, wb)
    F = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W)
    M = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W, mixed=True)
    return ss, walkers, F, M


@pytest.mark.parametrize("noise", [0.05, 0.3])
@pytest.mark.parametrize("kind,N,nelec,G,W,decay", CASES)
def test_mixed_energy_and_force_bias(kind, N, nelec, G, W, decay, noise):
    ss, walkers, F, M = _setups(kind, N, nelec, G, W, decay, noise)
    w = F.walkers(walkers)
    e64 = cpu(F.energy(w))
    emx = cpu(M.energy(w))
    assert np.max(np.abs(emx - e64)) <= 1e-5, np.max(np.abs(emx - e64))
    assert rel(cpu(M.force_bias(w)), cpu(F.force_bias(w))) <= 1e-9


@pytest.mark.parametrize("kind,N,nelec,G,W,decay", CASES)
def test_mixed_trotter(kind, N, nelec, G, W, decay):
    import trot_gb300 as tg

    ss, walkers, F, M = _setups(kind, N, nelec, G, W, decay, 0.1)
    rng = np.random.default_rng(5)
    xs = dev(rng.normal(size=(W, G)) + 0.3j * rng.normal(size=(W, G)))
    w = F.walkers(walkers)
    o64 = tg.make_trotter_ops("restricted", F.walker_kind).apply_trotter(w, xs, F.prop_ctx, 6)
    omx = tg.make_trotter_ops("restricted", F.walker_kind, mixed_precision=True).apply_trotter(w, xs, M.prop_ctx, 6)
    if kind == "rhf_r":
        assert rel(cpu(omx), cpu(o64)) <= 2e-5
    else:
        assert rel(cpu(omx[0]), cpu(o64[0])) <= 2e-5
        assert rel(cpu(omx[1]), cpu(o64[1])) <= 2e-5


@pytest.mark.parametrize("kind,N,nelec,G,W,decay", CASES)
def test_mixed_step(kind, N, nelec, G, W, decay):
    from trot_gb300 import synthetic

    ss, walkers, F, M = _setups(kind, N, nelec, G, W, decay, 0.05)
    ov = cpu(F.overlap(F.walkers(walkers)))
    e0 = float(np.real(cpu(F.energy(F.walkers(walkers))))[0])
    x = dev(synthetic.fields(W, G, 1, seed=8)[0])
    sF = F.state(F.walkers(walkers), np.ones(W), ov, e0, e0)
    sM = M.state(M.walkers(walkers), np.ones(W), ov, e0, e0)
    eF = torch.empty(W, dtype=torch.complex128, device="cuda")
    eM = torch.empty(W, dtype=torch.complex128, device="cuda")
    sF = F.step(sF, x, energy_out=eF)
    sM = M.step(sM, x, energy_out=eM)
    assert np.max(np.abs(cpu(eM) - cpu(eF))) <= 1e-5
    if kind == "rhf_r":
        assert rel(cpu(sM.walkers), cpu(sF.walkers)) <= 2e-5
    else:
        assert rel(cpu(sM.walkers[0]), cpu(sF.walkers[0])) <= 2e-5
        assert rel(cpu(sM.walkers[1]), cpu(sF.walkers[1])) <= 2e-5
    wf, wm = cpu(sF.weights), cpu(sM.weights)
    live = (wf > 0) & (wm > 0)
    assert np.array_equal(wf > 0, wm > 0)
    if live.any():
        assert rel(wm[live], wf[live]) <= 1e-3


@pytest.mark.parametrize("kind,N,nelec,G,W", [("uhf_u", 40, (6, 5), 96, 700), ("rhf_r", 30, (7, 7), 64, 333)])
def test_mixed_energy_many_walker_tiles(kind, N, nelec, G, W):
    """Enough walkers that every CTA of the exchange kernel runs several walker
    tiles (both TMEM accumulator buffers, ring wrap-around)."""
    ss, walkers, F, M = _setups(kind, N, nelec, G, W, 30.0, 0.1)
    w = F.walkers(walkers)
    e64 = cpu(F.energy(w))
    emx = cpu(M.energy(w))
    assert np.max(np.abs(emx - e64)) <= 1e-5
    assert rel(cpu(M.force_bias(w)), cpu(F.force_bias(w))) <= 1e-9


@pytest.mark.parametrize("kind,N,nelec,G,W", [("uhf_u", 64, (9, 7), 128, 300), ("rhf_r", 100, (16, 16), 200, 160),
                                              ("rhf_u", 128, (16, 16), 150, 40)])
def test_mixed_trotter_many_walkers(kind, N, nelec, G, W):
    """Tensor-core Taylor action over several waves of CTAs and at the largest
    supported tile (N = 128, 32 occupied columns)."""
    import trot_gb300 as tg

    ss, walkers, F, M = _setups(kind, N, nelec, G, W, 30.0, 0.1)
    rng = np.random.default_rng(6)
    xs = dev(rng.normal(size=(W, G)) + 0.3j * rng.normal(size=(W, G)))
    w = F.walkers(walkers)
    o64 = tg.make_trotter_ops("restricted", F.walker_kind).apply_trotter(w, xs, F.prop_ctx, 6)
    omx = tg.make_trotter_ops("restricted", F.walker_kind, mixed_precision=True).apply_trotter(w, xs, M.prop_ctx, 6)
    if kind == "rhf_r":
        assert rel(cpu(omx), cpu(o64)) <= 2e-5
    else:
        assert rel(cpu(omx[0]), cpu(o64[0])) <= 2e-5
        assert rel(cpu(omx[1]), cpu(o64[1])) <= 2e-5
