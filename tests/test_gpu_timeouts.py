"""The device-timeout path of the tensor-core kernels, exercised without a fault.

The exchange kernel's test switch (TROT_TUNE_TEST_TIMEOUT = v) makes its first
bounded wait be on a barrier nothing arrives on, limited to v polls.  The kernel
then records TROT_ERR_DEVICE_TIMEOUT in the workspace's status words, issues no
copies or MMAs, releases its epilogue, frees its tensor memory and returns.  The
combining kernels write NaN instead of numbers, the sticky status word keeps the
record, and the Python layer raises.  The context stays usable afterwards."""
import ctypes

import numpy as np
import pytest
import torch

from tests.gpu_helpers import Setup, cpu, dev

pytestmark = pytest.mark.gpu
POLLS = 64


@pytest.fixture(scope="module")
def setups():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trot_gb300 import synthetic

    N, nelec, G, W = 24, (5, 4), 120, 8
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=13, h0=0.3)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 14)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 15)
    F = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W)
    M = Setup("uhf_u", ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.005, W, mixed=True)
    return F, M, (wa, wb), G


class _TimeoutSwitch:
    def __enter__(self):
        from trot_gb300 import _lib

        _lib.call("trot_set_tuning", _lib.TUNE_TEST_TIMEOUT, POLLS)

    def __exit__(self, *exc):
        from trot_gb300 import _lib

        _lib.call("trot_set_tuning", _lib.TUNE_TEST_TIMEOUT, 0)


def test_timed_out_energy_raises_and_recovers(setups):
    from trot_gb300 import _lib

    F, M, walkers, _ = setups
    w = M.walkers(walkers)
    e64 = cpu(F.energy(w))
    with _TimeoutSwitch():
        with pytest.raises(_lib.TrotError) as ei:
            M.energy(w)
    assert ei.value.status == 6
    # the switch is off again: the same call gives numbers, and the record was cleared by the raise
    emx = cpu(M.energy(w))
    assert np.max(np.abs(emx - e64)) <= 1e-5


def test_timed_out_energy_is_nan_through_the_c_abi(setups):
    """Through the C ABI: NaN energies, trot_workspace_status / trot_workspace_timeouts
    report the timeout, the next call resets the call status but not the sticky word."""
    from trot_gb300 import _lib, native

    _, M, walkers, _ = setups
    wa, wb = M.walkers(walkers)
    s = native.system(_lib.UHF_U, wa.shape[0], M.trial, M.meas_ctx, h0=float(M.ham.h0), precision=_lib.MIXED)
    lib = _lib.load()
    n = lib.trot_workspace_size(ctypes.byref(s), _lib.OP_LOCAL_ENERGY)
    ws = torch.zeros(n, dtype=torch.uint8, device="cuda")
    out = torch.empty(wa.shape[0], dtype=torch.complex128, device="cuda")

    def call():
        _lib.check(lib.trot_local_energy(ctypes.byref(s), wa.data_ptr(), wb.data_ptr(), out.data_ptr(),
                                         ws.data_ptr(), n, native.stream_ptr()))
        torch.cuda.synchronize()

    st = ctypes.c_int(-1)
    with _TimeoutSwitch():
        call()
    e = cpu(out)
    assert np.all(np.isnan(e.real)) and np.all(np.isnan(e.imag))
    _lib.call("trot_workspace_status", ws.data_ptr(), ctypes.addressof(st))
    assert st.value == 6
    call()  # switch off: numbers again, call status OK, sticky word still set
    assert np.all(np.isfinite(cpu(out)))
    _lib.call("trot_workspace_status", ws.data_ptr(), ctypes.addressof(st))
    assert st.value == 0
    _lib.call("trot_workspace_timeouts", ws.data_ptr(), 1, ctypes.addressof(st))
    assert st.value == 6
    _lib.call("trot_workspace_timeouts", ws.data_ptr(), 0, ctypes.addressof(st))
    assert st.value == 0


def test_timed_out_step_poisons_weights(setups):
    """A mixed step whose exchange kernel timed out leaves NaN weights and a NaN
    population shift (no numbers computed from skipped results); the device check
    raises; later steps run normally."""
    from trot_gb300 import _lib, native, synthetic

    F, M, walkers, G = setups
    W = walkers[0].shape[0]
    ov = cpu(M.overlap(M.walkers(walkers)))
    st = M.state(M.walkers(walkers), np.ones(W), ov, 0.0, -1.0)
    x = dev(synthetic.fields(W, G, 2, seed=16))
    native.check_device_timeouts()  # start from a clear record
    with _TimeoutSwitch():
        st = M.step(st, x[0])
    torch.cuda.synchronize()
    assert np.all(np.isnan(cpu(st.weights)))
    assert np.isnan(float(st.pop_control_ene_shift))
    with pytest.raises(_lib.TrotError) as ei:
        native.check_device_timeouts()
    assert ei.value.status == 6
    st2 = M.state(M.walkers(walkers), np.ones(W), ov, 0.0, -1.0)
    st2 = M.step(st2, x[1])
    torch.cuda.synchronize()
    assert np.all(np.isfinite(cpu(st2.weights)))
    native.check_device_timeouts()
