"""torch.ops.trot_gb300.* on the GPU against the CPU oracle: the same numbers
through the dispatcher as through the C ABI, and the walker gradient of the
FP64 local energy (the library's hand-written VJP as the operator's backward)
against a central finite difference.

Tolerance: 1e-10 relative for FP64 (the parity bar); the mixed-precision
energies within 1e-6 Ha of the oracle on walkers near the trial."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from tests.gpu_helpers import cpu, dev, rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def sysdata():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import trot_gb300.torch_ops  # noqa: F401
    from trot_gb300 import synthetic

    N, nelec, G, W, dt = 22, (5, 4), 70, 12, 0.01
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=17, h0=0.4)
    meas = orc.build_uhf_meas_ctx(ss.h1, ss.chol, ss.mo_a, ss.mo_b)
    prop = orc.build_prop_ctx(ss.h0, ss.h1, ss.chol, ss.rdm1(), dt)
    model = orc.Model("uhf_u", ss.h0, (ss.mo_a, ss.mo_b), meas, prop)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 18)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 19)
    t = dict(wa=dev(wa), wb=dev(wb), mo_a=dev(ss.mo_a), mo_b=dev(ss.mo_b), ha=dev(meas.rot_h1_a),
             hb=dev(meas.rot_h1_b), ra=dev(meas.rot_chol_a), rb=dev(meas.rot_chol_b),
             eh=dev(prop.exp_h1_half), cf=dev(prop.chol_flat), mf=dev(np.imag(prop.mf_shifts)))
    return dict(ss=ss, meas=meas, prop=prop, model=model, walkers=(wa, wb), t=t, W=W, G=G, dt=dt)


def test_measurements_vs_oracle(sysdata):
    o, t, m = torch.ops.trot_gb300, sysdata["t"], sysdata["model"]
    w = sysdata["walkers"]
    assert rel(cpu(o.overlap(t["wa"], t["wb"], t["mo_a"], t["mo_b"], 2)), m.overlap(w)) < TOL
    fb = o.force_bias(t["wa"], t["wb"], t["mo_a"], t["mo_b"], t["ra"], t["rb"], 2, False)
    assert rel(cpu(fb), m.force_bias(w)) < TOL
    e_ref = m.energy(w)
    h0 = float(sysdata["ss"].h0)
    e = o.local_energy(t["wa"], t["wb"], t["mo_a"], t["mo_b"], t["ha"], t["hb"], t["ra"], t["rb"], h0, 2, False)
    assert rel(cpu(e), e_ref) < TOL
    emx = o.local_energy(t["wa"], t["wb"], t["mo_a"], t["mo_b"], t["ha"], t["hb"], t["ra"], t["rb"], h0, 2, True)
    assert np.max(np.abs(cpu(emx) - e_ref)) < 1e-6


def test_walker_ops_vs_oracle(sysdata):
    o, t = torch.ops.trot_gb300, sysdata["t"]
    wa, wb = sysdata["walkers"]
    qa, qb, norm = o.orthonormalize(t["wa"], t["wb"], 2)
    ra, rb = orc.orthonormalize((wa, wb), "unrestricted")
    assert rel(cpu(qa), ra) < TOL and rel(cpu(qb), rb) < TOL
    # diag(R) real and non-negative: the norm is prod_j |R_jj| over both spins
    dets = [np.prod(np.abs(np.diagonal(np.linalg.qr(x, mode="r"), axis1=-2, axis2=-1)), axis=-1) for x in (wa, wb)]
    assert rel(cpu(norm), dets[0] * dets[1]) < TOL
    W = sysdata["W"]
    weights = np.random.default_rng(4).uniform(0.2, 2.0, W)
    sa, sb, sw, idx = o.sr_resample(t["wa"], t["wb"], dev(weights), 0.61, 2)
    idx_ref = orc.sr_indices(weights, 0.61, W)
    np.testing.assert_array_equal(cpu(idx), idx_ref)
    np.testing.assert_array_equal(cpu(sa), wa[idx_ref])
    np.testing.assert_array_equal(cpu(sb), wb[idx_ref])
    assert rel(cpu(sw), np.full(W, np.cumsum(weights)[-1] / W)) < 1e-14


def test_prop_step_vs_oracle(sysdata):
    o, t, m, prop = torch.ops.trot_gb300, sysdata["t"], sysdata["model"], sysdata["prop"]
    W, G, dt = sysdata["W"], sysdata["G"], sysdata["dt"]
    w = sysdata["walkers"]
    ov = m.overlap(w)
    e0 = float(np.real(m.energy(w))[0])
    ost = orc.State(w, np.ones(W), ov, e0, e0, 0)
    x = np.random.default_rng(5).standard_normal((W, G))
    e_ref = m.energy(w)
    p = orc.Params(dt=dt)
    ost = orc.afqmc_step(ost, m, p, x)
    wa, wb = t["wa"].clone(), t["wb"].clone()
    weights, overlaps = dev(np.ones(W)), dev(ov)
    scalars, nodes = dev(np.array([e0, e0])), torch.zeros(1, dtype=torch.int64, device="cuda")
    e = o.prop_step(wa, wb, weights, overlaps, scalars, nodes, dev(x), t["mo_a"], t["mo_b"], t["ha"], t["hb"],
                    t["ra"], t["rb"], t["eh"], t["cf"], t["mf"], float(sysdata["ss"].h0), float(prop.h0_prop), dt,
                    p.n_exp_terms, p.weight_floor, p.weight_cap, p.pop_control_damping, 2, False)
    assert rel(cpu(e), e_ref) < TOL
    assert rel(cpu(wa), ost.walkers[0]) < TOL and rel(cpu(wb), ost.walkers[1]) < TOL
    assert rel(cpu(weights), ost.weights) < TOL
    assert rel(cpu(overlaps), ost.overlaps) < TOL
    assert abs(float(scalars[0]) - ost.pop_control_ene_shift) < 1e-9 * max(1.0, abs(ost.pop_control_ene_shift))
    assert int(nodes.item()) == ost.node_encounters


def test_energy_gradient_vs_finite_differences(sysdata):
    """d Re(sum_w c_w E_L(w)) / d walkers from the operator's backward, checked by a
    central difference along a random complex direction."""
    o, t = torch.ops.trot_gb300, sysdata["t"]
    h0 = float(sysdata["ss"].h0)
    rng = np.random.default_rng(6)
    c = dev(rng.normal(size=sysdata["W"]))
    wa = t["wa"].clone().requires_grad_(True)
    wb = t["wb"].clone().requires_grad_(True)

    def J(a, b):
        e = o.local_energy(a, b, t["mo_a"], t["mo_b"], t["ha"], t["hb"], t["ra"], t["rb"], h0, 2, False)
        return (e.real * c).sum()

    J(wa, wb).backward()
    da = dev(rng.normal(size=wa.shape) + 1j * rng.normal(size=wa.shape))
    db = dev(rng.normal(size=wb.shape) + 1j * rng.normal(size=wb.shape))
    eps = 1e-5
    with torch.no_grad():
        fd = (J(t["wa"] + eps * da, t["wb"] + eps * db) - J(t["wa"] - eps * da, t["wb"] - eps * db)) / (2 * eps)
    # torch's gradient of a real function of complex z is dJ/dRe z + i dJ/dIm z
    an = torch.real(torch.conj(wa.grad) * da).sum() + torch.real(torch.conj(wb.grad) * db).sum()
    assert abs(float(an) - float(fd)) <= 1e-6 * max(1.0, abs(float(fd)))
