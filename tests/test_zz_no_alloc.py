"""trot_local_energy_noalloc, the entry point for callers that cannot allocate
device memory (e.g. a JAX custom call in a process whose GPU memory XLA has
pre-allocated): it must give the same energies as trot_local_energy with a
caller workspace, call after call, while allocating nothing itself.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
TOL = 1e-10  # the FP64 parity tolerance used throughout the GPU tests


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import trot_gb300 as tg
    from trot_gb300 import _lib, native, synthetic

    N, nelec, G, W = 24, (5, 4), 120, 64
    ss = synthetic.make_system(N, nelec, G, decay=30.0, seed=21, h0=0.4)
    sysm = tg.System(norb=N, nelec=nelec, walker_kind="unrestricted")
    ham = tg.HamChol(h0=ss.h0, h1=ss.h1, chol=ss.chol)
    trial = tg.UhfTrial(ss.mo_a, ss.mo_b)
    meas_ctx = tg.make_uhf_meas_ops(sysm).build_meas_ctx(ham, trial)
    s = native.system(_lib.UHF_U, W, trial, meas_ctx, h0=ss.h0)
    # the same system on the tensor-core path: exact-digit exchange, status words in the scratch
    s_mixed = native.system(_lib.UHF_U, W, trial, meas_ctx, h0=ss.h0, precision=_lib.MIXED)
    walkers = []
    for seed in (31, 32):
        wa = torch.as_tensor(synthetic.perturbed_walkers(ss.mo_a, W, 0.2, seed)).cuda()
        wb = torch.as_tensor(synthetic.perturbed_walkers(ss.mo_b, W, 0.2, seed + 100)).cuda()
        walkers.append((wa, wb))
    # the struct holds raw device pointers: keep their owners (trial, meas_ctx) alive
    return dict(lib=_lib, native=native, s=s, s_mixed=s_mixed, walkers=walkers, W=W, owners=(trial, meas_ctx))


def _with_workspace(d, wa, wb, key="s"):
    lib, native, s = d["lib"], d["native"], d[key]
    out = torch.empty(d["W"], dtype=torch.complex128, device="cuda")
    n = lib.load().trot_workspace_size(ctypes.byref(s), lib.OP_LOCAL_ENERGY)
    ws = torch.empty(n, dtype=torch.uint8, device="cuda")
    lib.check(lib.load().trot_local_energy(ctypes.byref(s), wa.data_ptr(), wb.data_ptr(), out.data_ptr(),
                                           ws.data_ptr(), n, native.stream_ptr()))
    return out


def _no_alloc(d, wa, wb, key="s"):
    lib, native, s = d["lib"], d["native"], d[key]
    out = torch.empty(d["W"], dtype=torch.complex128, device="cuda")
    lib.check(lib.load().trot_local_energy_noalloc(ctypes.byref(s), wa.data_ptr(), wb.data_ptr(), out.data_ptr(),
                                                   native.stream_ptr()))
    return out


def test_no_alloc_matches_workspace_entry_point_twice(setup):
    for wa, wb in setup["walkers"]:  # two calls in a row on the shared scratch
        ref = _with_workspace(setup, wa, wb).cpu().numpy()
        got = _no_alloc(setup, wa, wb).cpu().numpy()
        assert np.max(np.abs(got - ref)) <= TOL * np.max(np.abs(ref))


def test_no_alloc_mixed_precision_twice(setup):
    """The tensor-core path through the built-in scratch (its status words, digit
    planes and exchange partial sums live there): same energies as the workspace
    entry point on two calls in a row, and the sticky timeout status reads OK."""
    lib = setup["lib"]
    st = ctypes.c_int(-1)
    lib.call("trot_local_energy_noalloc_status", 1, ctypes.addressof(st))
    for wa, wb in setup["walkers"]:
        ref = _with_workspace(setup, wa, wb, "s_mixed").cpu().numpy()
        got = _no_alloc(setup, wa, wb, "s_mixed").cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= TOL * np.max(np.abs(ref))
    lib.call("trot_local_energy_noalloc_status", 0, ctypes.addressof(st))
    assert st.value == 0


def test_no_alloc_rejects_oversized_system(setup):
    lib, native = setup["lib"], setup["native"]
    s = lib.TrotSystem()
    ctypes.pointer(s)[0] = setup["s"]
    s.n_walkers = 60000  # ~ 60000 * 9 * 24 * 16 B of Green's functions alone: beyond the 32 MiB scratch
    wa, wb = setup["walkers"][0]
    out = torch.empty(1, dtype=torch.complex128, device="cuda")
    rc = lib.load().trot_local_energy_noalloc(ctypes.byref(s), wa.data_ptr(), wb.data_ptr(), out.data_ptr(),
                                              native.stream_ptr())
    assert rc == 4
    assert b"scratch" in lib.load().trot_last_error()
