"""The autotuner picks the exchange kernel's launch shape by timing; every
candidate shape gives bit-identical energies."""
import numpy as np
import pytest
import torch

from tests.gpu_helpers import Setup, cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_autotune_exchange_shapes_identical():
    from trot_gb300 import autotune, synthetic

    ss = synthetic.make_system(60, (9, 7), 150, decay=30.0, seed=4, h0=0.1)
    W = 200
    M = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W, mixed=True)
    w = M.walkers((synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 1), synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 2)))
    try:
        ref = cpu(M.energy(w))
        for t, g in [(4, 152), (32, 152), (8, 304), (64, 100)]:
            autotune.set_exchange(t, g)
            assert np.array_equal(cpu(M.energy(w)), ref), (t, g)
        res = autotune.tune_exchange(w, M.ham, M.meas_ops, M.meas_ctx, M.trial, reps=1)
        assert res["tiles"] in autotune.EXCHANGE_TILES and res["grid"] in autotune.EXCHANGE_GRID
        assert np.array_equal(cpu(M.energy(w)), ref)
    finally:
        autotune.reset()
