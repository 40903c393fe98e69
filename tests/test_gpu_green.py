"""Standalone half-rotated Green's functions (trot_half_green) against the oracle's
``_half_green_from_overlap_matrix`` restatement, per spin, with the trial overlaps."""
import numpy as np
import pytest
import torch

from oracle import afqmc_oracle as orc
from tests.gpu_helpers import Setup, cpu, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("kind,N,nelec,W", [("rhf_r", 20, (4, 4), 9), ("rhf_u", 20, (4, 4), 7),
                                            ("uhf_u", 31, (6, 4), 11)])
def test_half_green_matches_oracle(kind, N, nelec, W):
    from trot_gb300 import synthetic
    from trot_gb300.trial import half_green_batched

    ss = synthetic.make_system(N, nelec, 3 * N, decay=30.0, seed=5, h0=0.2)
    mo_b = ss.mo_b if kind == "uhf_u" else ss.mo_a
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, mo_b, 0.01, W)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 6)
    if kind == "rhf_r":
        walkers = S.walkers(wa)
        ref = orc.half_green(wa, ss.mo_a)
    else:
        wb = synthetic.perturbed_walkers(mo_b, W, 0.1, 7)
        walkers = S.walkers((wa, wb))
        ref = np.concatenate([orc.half_green(wa, ss.mo_a), orc.half_green(wb, mo_b)], axis=1)
    green, ov = half_green_batched(walkers, S.trial, S.walker_kind, with_overlaps=True)
    assert green.shape == ref.shape
    assert rel(cpu(green), ref) <= 1e-12
    assert rel(cpu(ov), cpu(S.trial_ops.overlap(walkers, S.trial))) <= 1e-14
    assert rel(cpu(half_green_batched(walkers, S.trial, S.walker_kind)), ref) <= 1e-12
