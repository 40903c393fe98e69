"""A whole block captured as one CUDA graph continues the same Markov chain as
eager blocks: bit-identical walkers, weights, overlaps, scalars and block energies."""
import numpy as np
import pytest
import torch

from tests.gpu_helpers import Setup, cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("kind,N,nelec,G,W,mixed", [("rhf_r", 24, (5, 5), 120, 64, False),
                                                     ("uhf_u", 40, (7, 5), 96, 48, True)])
def test_graphed_block_matches_eager(kind, N, nelec, G, W, mixed):
    import trot_gb300 as tg
    from trot_gb300 import synthetic
    from trot_gb300.graphs import GraphedBlock

    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=2, h0=0.3)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W, mixed=mixed)
    params = tg.QmcParams(dt=0.005, n_walkers=W, n_prop_steps=4, seed=11)
    s0 = S.prop_ops.init_prop_state(sys=S.sys, ham_data=S.ham, trial_ops=S.trial_ops, trial_data=S.trial,
                                    meas_ops=S.meas_ops, params=params)
    kw = dict(sys=S.sys, params=params, ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops,
              meas_ops=S.meas_ops, meas_ctx=S.meas_ctx, prop_ops=S.prop_ops, prop_ctx=S.prop_ctx)
    eager = s0.clone()
    e_eager = []
    for _ in range(3):
        eager, obs = tg.block(eager, **kw)
        e_eager.append(float(obs.scalars["energy"]))
    gstate = s0.clone()
    gb = GraphedBlock(gstate, **kw)
    e_graph = [float(gb.replay()["energy"]) for _ in range(3)]
    torch.cuda.synchronize()
    assert e_graph == e_eager
    if kind == "rhf_r":
        assert np.array_equal(cpu(gstate.walkers), cpu(eager.walkers))
    else:
        assert np.array_equal(cpu(gstate.walkers[0]), cpu(eager.walkers[0]))
        assert np.array_equal(cpu(gstate.walkers[1]), cpu(eager.walkers[1]))
    for name in ("weights", "overlaps", "scalars", "rng_key", "node_encounters"):
        assert np.array_equal(cpu(getattr(gstate, name)), cpu(getattr(eager, name))), name
