"""One-time constants built on the device (trot_build_prop_ctx, trot_half_rotate,
trot_cisd_lci1) vs the oracle.

Tolerances: 1e-12 relative (max-norm) for mf_shifts, exp(-dt/2 h1_eff) and the
rotations; h0_prop 1e-12 relative.  The matrix exponential is checked against
scipy's Pade expm, including norms that need squarings."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from oracle import cisd_oracle as corc
from tests.gpu_helpers import cpu, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _system(N, G, seed, nocc=None, scale_h1=1.0):
    from trot_gb300 import synthetic

    n = nocc or max(1, N // 5)
    ss = synthetic.make_system(N, (n, n), G, decay=30.0, seed=seed, h0=0.7)
    return ss, ss.h1 * scale_h1


# (N, G, dt, h1 scale): N off the 32-wide tiles, G = 1, and norms that need 0 .. 8 squarings
CASES = [(7, 5, 0.005, 1.0), (24, 120, 0.005, 1.0), (45, 1, 0.01, 1.0), (33, 64, 0.5, 1.0),
         (120, 600, 0.005, 1.0), (64, 40, 0.2, 5.0), (17, 9, 0.2, 4.0), (130, 70, 0.01, 1.0)]


@pytest.mark.parametrize("N,G,dt,scale", CASES)
def test_prop_ctx_vs_oracle(N, G, dt, scale):
    from trot_gb300 import ctx

    ss, h1 = _system(N, G, seed=N + G)
    rdm1 = np.stack([ss.mo_a @ ss.mo_a.T, ss.mo_b @ ss.mo_b.T])
    ref = orc.build_prop_ctx(ss.h0, h1, ss.chol, rdm1, dt)
    mf_im, h0p, eh, _ = ctx.prop_ctx(ss.h0, h1, ss.chol, rdm1, dt)
    assert rel(cpu(mf_im), np.imag(ref.mf_shifts)) < 1e-12
    assert abs(h0p - ref.h0_prop) <= 1e-12 * max(1.0, abs(ref.h0_prop))
    assert rel(cpu(eh), ref.exp_h1_half) < 1e-12


def test_prop_ctx_rdm1_forms_and_device_inputs():
    """(2, N, N) and spin-summed (N, N) density matrices, numpy and device inputs agree bit for bit."""
    from trot_gb300 import ctx

    ss, h1 = _system(40, 30, seed=2)
    rdm1 = np.stack([ss.mo_a @ ss.mo_a.T, ss.mo_b @ ss.mo_b.T])
    a = ctx.prop_ctx(ss.h0, h1, ss.chol, rdm1, 0.01)
    b = ctx.prop_ctx(ss.h0, torch.as_tensor(h1).cuda(), torch.as_tensor(ss.chol).cuda(),
                     torch.as_tensor(rdm1[0] + rdm1[1]).cuda(), 0.01)
    assert torch.equal(a[0], b[0]) and a[1] == b[1] and torch.equal(a[2], b[2])


@pytest.mark.parametrize("N,G,n", [(7, 5, 1), (24, 120, 5), (45, 3, 16), (70, 33, 17), (130, 20, 33), (200, 8, 12)])
def test_half_rotation_vs_oracle(N, G, n):
    from trot_gb300 import ctx

    ss, h1 = _system(N, G, seed=3 * N + n, nocc=n)
    ref = orc.build_rhf_meas_ctx(h1, ss.chol, ss.mo_a)
    rot_h1, rot_chol = ctx.half_rotate(ss.mo_a, h1, ss.chol)
    assert rel(cpu(rot_h1), ref.rot_h1) < 1e-12
    assert rel(cpu(rot_chol), ref.rot_chol) < 1e-12


def test_uhf_meas_ctx_on_device():
    import trot_gb300 as tg

    ss, h1 = _system(36, 50, seed=9, nocc=6)
    ref = orc.build_uhf_meas_ctx(h1, ss.chol, ss.mo_a, ss.mo_b)
    m = tg.build_uhf_meas_ctx(tg.HamChol(h0=ss.h0, h1=h1, chol=ss.chol), tg.UhfTrial(ss.mo_a, ss.mo_b))
    for got, want in zip(m.spin_arrays(), (ref.rot_h1_a, ref.rot_h1_b, ref.rot_chol_a, ref.rot_chol_b)):
        assert rel(cpu(got), want) < 1e-12


@pytest.mark.parametrize("N,G,n", [(20, 48, 4), (60, 300, 8), (9, 2, 8)])
def test_cisd_lci1_vs_oracle(N, G, n):
    from trot_gb300 import ctx

    ss, _ = _system(N, G, seed=N, nocc=n)
    ci1 = np.random.default_rng(N).normal(scale=0.02, size=(n, N - n))
    got = ctx.cisd_lci1(ci1, ss.chol)
    assert rel(cpu(got), corc.meas_lci1(ss.chol, ci1, slice(n, N))) < 1e-12


def test_prop_ctx_numeric_guard():
    """A non-finite h1 and a norm past 2^39 come back as NUMERIC_GUARD (host-read device status)."""
    from trot_gb300 import _lib, ctx

    ss, h1 = _system(12, 6, seed=1)
    rdm1 = ss.mo_a @ ss.mo_a.T * 2
    bad = h1.copy()
    bad[3, 4] = np.nan
    with pytest.raises(_lib.TrotError, match="NUMERIC_GUARD"):
        ctx.prop_ctx(ss.h0, bad, ss.chol, rdm1, 0.01)
    with pytest.raises(_lib.TrotError, match="NUMERIC_GUARD"):
        ctx.prop_ctx(ss.h0, h1 * 1e15, ss.chol, rdm1, 1.0)
    # the library stays usable after a guarded failure
    ctx.prop_ctx(ss.h0, h1, ss.chol, rdm1, 0.01)
