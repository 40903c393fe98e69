"""Uneven fragment batches: concurrent per-fragment streams and the captured
batched step give bit-identical results to stepping each fragment alone."""
import numpy as np
import pytest
import torch

from tests.gpu_helpers import cpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def test_fragment_batch_matches_sequential():
    from trot_gb300.fragments import FragmentBatch, make_fragment

    sizes = [(30, 4, 120, 32), (70, 8, 280, 24), (140, 17, 560, 16), (50, 6, 200, 40)]  # N=140 runs FP64
    frags = [make_fragment(n, o, g, w, seed=i) for i, (n, o, g, w) in enumerate(sizes)]
    assert [f.mixed for f in frags] == [True, True, False, True]
    refs = [f.state.clone() for f in frags]
    ref_e = [torch.empty_like(f.energy) for f in frags]

    def seq_step():
        for f, st, e in zip(frags, refs, ref_e):
            f.prop_ops.step(st, params=f.params, ham_data=f.ham, trial_data=f.trial, trial_ops=f.trial_ops,
                            meas_ops=f.meas_ops, meas_ctx=f.meas_ctx, prop_ctx=f.prop_ctx, energy_out=e)

    batch = FragmentBatch(frags)
    assert [f.norb for f in batch.fragments] == [140, 70, 50, 30]  # largest work first
    batch.step()  # eager, concurrent streams
    seq_step()
    torch.cuda.synchronize()
    for f, st, e in zip(frags, refs, ref_e):
        assert np.array_equal(cpu(f.state.walkers), cpu(st.walkers))
        assert np.array_equal(cpu(f.state.weights), cpu(st.weights))
        assert np.array_equal(cpu(f.energy), cpu(e))
    batch.capture()
    for _ in range(2):
        batch.step()  # graph replays
        seq_step()
    torch.cuda.synchronize()
    for f, st, e in zip(frags, refs, ref_e):
        assert np.array_equal(cpu(f.state.walkers), cpu(st.walkers))
        assert np.array_equal(cpu(f.state.weights), cpu(st.weights))
        assert np.array_equal(cpu(f.state.scalars), cpu(st.scalars))
        assert np.array_equal(cpu(f.energy), cpu(e))
