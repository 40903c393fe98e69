"""Staged inputs on the device: ``staging.load(path, device=...)`` streams the cache's
payloads into HBM through pinned buffers (small chunks here, so the double-buffered
path runs many rounds), and the objects ``make_job_inputs`` builds from a file the
reference's ``dump`` wrote give the oracle's local energies and force biases."""
from __future__ import annotations

import os

import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as ao
from oracle import cisd_oracle as co
from tests.gpu_helpers import cpu, dev, rel

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("case", ["rhf", "uhf", "cisd"])
def test_device_load_matches_host(case):
    from trot_gb300 import staging
    path = os.path.join(GOLDEN, f"staged_{case}.h5")
    host = staging.load(path)
    d = staging.load(path, device="cuda", chunk_bytes=1024)
    assert d.ham.chol.is_cuda and d.ham.h1.is_cuda
    assert np.array_equal(cpu(d.ham.chol), host.ham.chol) and np.array_equal(cpu(d.ham.h1), host.ham.h1)
    for k, v in host.trial.data.items():
        assert d.trial.data[k].is_cuda and np.array_equal(cpu(d.trial.data[k]), v), k


def _walkers(N, n, W, seed, mo):
    rng = np.random.default_rng(seed)
    return mo[None, :, :n] + 0.2 * (rng.normal(size=(W, N, n)) + 1j * rng.normal(size=(W, N, n)))


@pytest.mark.parametrize("case", ["rhf", "uhf"])
def test_staged_job_vs_oracle(case):
    from trot_gb300 import staging
    st = staging.load(os.path.join(GOLDEN, f"staged_{case}.h5"), device="cuda")
    wk = "restricted" if case == "rhf" else "unrestricted"
    sys_, ham, trial, trial_ops, meas_ops = staging.make_job_inputs(st, walker_kind=wk)
    host = staging.load(os.path.join(GOLDEN, f"staged_{case}.h5"))
    N, (na, nb) = host.ham.norb, host.ham.nelec
    h1, chol, h0 = host.ham.h1, host.ham.chol, host.ham.h0
    if case == "rhf":
        mo = host.trial.data["mo"][:, :na]
        model = ao.Model("rhf_r", h0, mo, ao.build_rhf_meas_ctx(h1, chol, mo), None)
        w = _walkers(N, na, 6, 1, host.trial.data["mo"])
        wd = dev(w)
    else:
        mo_a, mo_b = host.trial.data["mo_a"][:, :na], host.trial.data["mo_b"][:, :nb]
        model = ao.Model("uhf_u", h0, (mo_a, mo_b), ao.build_uhf_meas_ctx(h1, chol, mo_a, mo_b), None)
        w = (_walkers(N, na, 6, 1, host.trial.data["mo_a"]), _walkers(N, nb, 6, 2, host.trial.data["mo_b"]))
        wd = (dev(w[0]), dev(w[1]))
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    e = cpu(meas_ops.kernels["energy"](wd, ham, meas_ctx, trial))
    fb = cpu(meas_ops.kernels["force_bias"](wd, ham, meas_ctx, trial))
    assert rel(e, model.energy(w)) < 1e-11
    assert rel(fb, model.force_bias(w)) < 1e-11


def test_staged_cisd_vs_oracle():
    from trot_gb300 import staging
    path = os.path.join(GOLDEN, "staged_cisd.h5")
    st = staging.load(path, device="cuda")
    sys_, ham, trial, trial_ops, meas_ops = staging.make_job_inputs(st, walker_kind="restricted",
                                                                     mixed_precision=False)
    host = staging.load(path)
    N, (no, _) = host.ham.norb, host.ham.nelec
    tr = co.CisdTrial(ci1=host.trial.data["ci1"], ci2=host.trial.data["ci2"])
    w = _walkers(N, no, 5, 3, np.eye(N))
    wd = dev(w)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    ov = cpu(trial_ops.overlap(wd, trial))
    e = cpu(meas_ops.kernels["energy"](wd, ham, meas_ctx, trial))
    assert rel(ov, co.overlap(w, tr)) < 1e-11
    fb = cpu(meas_ops.kernels["force_bias"](wd, ham, meas_ctx, trial))
    e_ref = co.energy(w, tr, host.ham.h0, host.ham.h1, host.ham.chol)
    # the bundle's meas ops keep the reference's default (testing=False: the l2ci2 quadratic
    # forms in 32-bit arithmetic, trot/meas/cisd.py:823-839), so the energy is FP32-class
    assert rel(e, e_ref) < 1e-6
    assert rel(fb, co.force_bias(w, tr, host.ham.chol)) < 1e-10
    import trot_gb300 as tg
    m64 = tg.make_cisd_meas_ops(sys_, mixed_precision=False, testing=True)
    e64 = cpu(m64.kernels["energy"](wd, ham, m64.build_meas_ctx(ham, trial), trial))
    assert rel(e64, e_ref) < 1e-10
