"""Per-kernel timers and the launch counter the benchmark reports: while enabled,
every kernel launch of the library is counted (timed or not), the timers sum per
kernel name, and nothing is counted while disabled."""
import pytest
import torch

from tests.gpu_helpers import Setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("mixed", [False, True])
def test_launch_counter_and_timers(mixed):
    import trot_gb300 as tg
    from trot_gb300 import _lib, synthetic

    N, nelec, G, W = 40, (7, 5), 96, 48
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=2, h0=0.3)
    S = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W, mixed=mixed)
    params = tg.QmcParams(dt=0.005, n_walkers=W, n_prop_steps=4, seed=11)
    st = S.prop_ops.init_prop_state(sys=S.sys, ham_data=S.ham, trial_ops=S.trial_ops, trial_data=S.trial,
                                    meas_ops=S.meas_ops, params=params)
    energy = torch.empty(W, dtype=torch.complex128, device="cuda")
    kw = dict(params=params, ham_data=S.ham, trial_data=S.trial, trial_ops=S.trial_ops, meas_ops=S.meas_ops,
              meas_ctx=S.meas_ctx, prop_ctx=S.prop_ctx, energy_out=energy)
    st = S.prop_ops.step(st, **kw)  # first launches and workspaces outside the counted region
    torch.cuda.synchronize()
    _lib.profile_enable(256)
    try:
        st = S.prop_ops.step(st, **kw)
        prof = _lib.profile_collect()
        n_all = _lib.profile_launch_count()
    finally:
        _lib.profile_enable(0)
    timed = sum(c for _, c in prof.values())
    assert timed > 0 and all(ms >= 0.0 for ms, _ in prof.values())
    assert n_all >= timed
    expected = {"exchange_exact_tc", "trotter_tc"} if mixed else {"trotter_fp64"}
    assert expected <= set(prof), sorted(prof)
    # disabled: no counting, no records
    st = S.prop_ops.step(st, **kw)
    torch.cuda.synchronize()
    assert _lib.profile_launch_count() == 0
    assert _lib.profile_collect() == {}
