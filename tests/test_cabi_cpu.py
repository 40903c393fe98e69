"""C ABI checks that need no GPU: the library builds and loads, exports every
entry point include/trot_gb300.h declares, and rejects bad arguments with a
status code before launching anything."""
import ctypes
import os
import re

import pytest

from trot_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    txt = open(os.path.join(ROOT, "include", "trot_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(trot_[a-z0-9_]+)\s*\(", txt)))


def test_header_symbols_exported():
    lib = _lib.load()
    decl = _declared()
    assert len(decl) >= 14
    for name in decl:
        assert hasattr(lib, name), name
    assert set(decl) == set(_lib.exported_symbols())


def test_abi_version():
    assert _lib.load().trot_abi_version() == 4


def _sys(**kw):
    s = _lib.TrotSystem()
    s.kind, s.precision, s.n_walkers, s.norb, s.nchol, s.nocc_a, s.nocc_b = 0, 0, 4, 8, 5, 2, 2
    s.n_exp_terms = 6
    s.mo_a = s.mo_b = 0x1000
    s.rot_h1_a = s.rot_chol_a = s.exp_h1_half = s.chol_flat = s.mf_shifts_im = 0x1000
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def _status(fn, *args):
    return getattr(_lib.load(), fn)(*args)


def test_error_null_pointers():
    s = _sys()
    assert _status("trot_overlap", ctypes.byref(s), None, None, 0x1000, None) == 3
    assert _status("trot_overlap", ctypes.byref(s), 0x1000, None, None, None) == 3
    assert b"null" in _lib.load().trot_last_error()
    assert _status("trot_overlap", None, 0x1000, None, 0x1000, None) == 3
    s2 = _sys(kind=2)
    s2.mo_b = 0
    assert _status("trot_overlap", ctypes.byref(s2), 0x1000, 0x1000, 0x1000, None) == 3


def test_error_bad_shapes():
    for kw in (dict(n_walkers=0), dict(norb=0), dict(nocc_a=9), dict(kind=7), dict(kind=1, nocc_b=3)):
        s = _sys(**kw)
        assert _status("trot_overlap", ctypes.byref(s), 0x1000, 0x1000, 0x1000, None) == 1, kw
    s = _sys(precision=5)
    assert _status("trot_overlap", ctypes.byref(s), 0x1000, 0x1000, 0x1000, None) == 2


def test_error_workspace_too_small():
    s = _sys()
    need = _lib.load().trot_workspace_size(ctypes.byref(s), _lib.OP_FORCE_BIAS)
    assert need > 0
    assert _status("trot_force_bias", ctypes.byref(s), 0x1000, None, 0x1000, 0x1000, need // 2, None) == 4
    assert _status("trot_local_energy", ctypes.byref(s), 0x1000, None, 0x1000, None, 0, None) == 4
    st = _lib.TrotState()
    st.walkers_a = st.weights = st.overlaps = st.scalars = st.node_encounters = 0x1000
    assert _status("trot_prop_step", ctypes.byref(s), ctypes.byref(st), 0x1000, None, 0x1000, 16, None) == 4


def test_error_sr_arguments():
    s = _sys()
    assert _status("trot_sr_resample", ctypes.byref(s), 0x1000, None, 1.5, 0x1000, None, 0x2000, None,
                   0x1000, 0x1000, 0x1000, 1 << 20, None) == 1
    assert _status("trot_sr_resample", ctypes.byref(s), 0x1000, None, 0.5, 0x1000, None, 0x1000, None,
                   0x1000, 0x1000, 0x1000, 1 << 20, None) == 1


def test_mixed_requires_context():
    s = _sys(precision=1)
    st = _lib.TrotState()
    st.walkers_a = st.weights = st.overlaps = st.scalars = st.node_encounters = 0x1000
    assert _status("trot_prop_step", ctypes.byref(s), ctypes.byref(st), 0x1000, None, 0x1000, 1 << 30, None) == 3


def test_workspace_size_monotone():
    small = _lib.load().trot_workspace_size(ctypes.byref(_sys(n_walkers=4)), _lib.OP_PROP_STEP)
    big = _lib.load().trot_workspace_size(ctypes.byref(_sys(n_walkers=400)), _lib.OP_PROP_STEP)
    assert big > small > 0
    assert _lib.load().trot_workspace_size(ctypes.byref(_sys(n_walkers=0)), _lib.OP_PROP_STEP) == 0


def _cisd(**kw):
    c = _lib.TrotCisd()
    c.norb, c.nocc, c.nvir, c.nchol, c.h0 = 10, 3, 7, 12, 0.5
    c.ci1 = c.ci2m = c.h1 = c.chol = c.lci1 = c.mo = 0x1000
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def test_cisd_workspace_and_errors():
    lib = _lib.load()
    c = _cisd()
    sizes = [lib.trot_cisd_workspace_size(ctypes.byref(c), 8, op)
             for op in (_lib.OP_OVERLAP, _lib.OP_FORCE_BIAS, _lib.OP_LOCAL_ENERGY, _lib.OP_PROP_STEP)]
    assert 0 < sizes[0] < sizes[1] < sizes[2] < sizes[3]
    # the local energy keeps 2 W G nocc nvir complex values for the l2ci2 quadratic form
    assert sizes[2] - sizes[1] >= 2 * 8 * 12 * 21 * 16
    assert lib.trot_cisd_workspace_size(ctypes.byref(c), 800, _lib.OP_LOCAL_ENERGY) > sizes[2]
    assert lib.trot_cisd_workspace_size(ctypes.byref(c), 8, _lib.OP_QR) == 0
    assert lib.trot_cisd_workspace_size(ctypes.byref(_cisd(nvir=6)), 8, _lib.OP_OVERLAP) == 0
    assert b"nocc + nvir == norb" in lib.trot_last_error()
    assert lib.trot_cisd_workspace_size(None, 8, _lib.OP_OVERLAP) == 0
    # overlap needs no Hamiltonian; the energy does
    nh = _cisd(h1=0, chol=0, lci1=0)
    assert lib.trot_cisd_overlap(ctypes.byref(nh), 8, 0x1000, 0x1000, 0x1000, 16, None) == 4
    assert lib.trot_cisd_local_energy(ctypes.byref(nh), 8, 0x1000, 0x1000, 0x1000, 1 << 40, None) == 3
    assert lib.trot_cisd_force_bias(ctypes.byref(c), 8, None, 0x1000, 0x1000, 1 << 40, None) == 3
    assert lib.trot_cisd_local_energy(ctypes.byref(c), 0, 0x1000, 0x1000, 0x1000, 1 << 40, None) == 1
    # shared-memory tiles bound the orbital count
    assert lib.trot_cisd_overlap(ctypes.byref(_cisd(norb=200, nvir=197)), 8, 0x1000, 0x1000, 0x1000, 1 << 40,
                                 None) == 8
    # the step's propagation context must match the CISD sizes and be restricted FP64
    s = _sys(n_walkers=8, norb=10, nchol=12, nocc_a=3)
    st = _lib.TrotState()
    st.walkers_a = st.weights = st.overlaps = st.scalars = st.node_encounters = 0x1000
    assert lib.trot_cisd_prop_step(ctypes.byref(c), ctypes.byref(_sys(n_walkers=8, norb=10, nchol=11, nocc_a=3)),
                                   ctypes.byref(st), 0x1000, None, 0x1000, 1 << 40, None) == 1
    assert lib.trot_cisd_prop_step(ctypes.byref(c), ctypes.byref(s), ctypes.byref(st), 0x1000, None, 0x1000, 16,
                                   None) == 4


def test_tuning_knobs():
    lib = _lib.load()
    assert lib.trot_get_tuning(_lib.TUNE_EXCHANGE_TILES) == 0
    assert lib.trot_set_tuning(_lib.TUNE_EXCHANGE_TILES, 8) == 0
    assert lib.trot_get_tuning(_lib.TUNE_EXCHANGE_TILES) == 8
    assert lib.trot_set_tuning(_lib.TUNE_EXCHANGE_TILES, 0) == 0
    assert lib.trot_set_tuning(7, 1) == 1
    assert b"unknown tuning knob" in lib.trot_last_error()
    assert lib.trot_set_tuning(_lib.TUNE_EXCHANGE_GRID, -3) == 1
    assert lib.trot_get_tuning(99) == 0


def test_ctx_builders_errors():
    """One-time context builders: size query, and argument errors before any launch."""
    lib = _lib.load()
    n1 = lib.trot_prop_ctx_workspace_size(24, 120)
    n2 = lib.trot_prop_ctx_workspace_size(120, 600)
    assert 0 < n1 < n2
    assert lib.trot_prop_ctx_workspace_size(0, 10) == 0
    p = 0x1000
    d = ctypes.c_double
    assert lib.trot_build_prop_ctx(24, 120, d(0.0), d(0.01), p, p, p, p, p, p, None, n1, None) == 3
    assert lib.trot_build_prop_ctx(24, 0, d(0.0), d(0.01), p, p, p, p, p, p, p, n1, None) == 1
    assert lib.trot_build_prop_ctx(24, 120, d(0.0), d(-1.0), p, p, p, p, p, p, p, n1, None) == 1
    assert lib.trot_build_prop_ctx(24, 120, d(0.0), d(0.01), p, p, p, p, p, p, p, n1 - 4096, None) == 4
    assert lib.trot_half_rotate(24, 10, 0, p, p, p, p, p, None) == 1
    assert lib.trot_half_rotate(24, 10, 25, p, p, p, p, p, None) == 1
    assert lib.trot_half_rotate(24, 10, 5, None, p, p, p, p, None) == 3
    assert lib.trot_half_rotate(24, 10, 5, p, p, p, None, p, None) == 3
    assert lib.trot_cisd_lci1(24, 10, 24, p, p, p, None) == 1
    assert lib.trot_cisd_lci1(24, 10, 5, p, None, p, None) == 3


def test_half_green_arguments():
    """trot_half_green: null output or walkers and bad shapes are rejected before any launch."""
    s = _sys()
    assert _status("trot_half_green", ctypes.byref(s), 0x1000, None, None, None, None) == 3
    assert _status("trot_half_green", ctypes.byref(s), None, None, 0x1000, None, None) == 3
    assert _status("trot_half_green", ctypes.byref(_sys(nocc_a=9)), 0x1000, None, 0x1000, None, None) == 1


def test_cisd_packed_contraction_workspace():
    """With chol_symmetric the Cholesky contraction runs on packed copies (extra workspace for
    the packed triangles); the float-float gamma tile is bounded by shared memory too."""
    lib = _lib.load()
    for op in (_lib.OP_FORCE_BIAS, _lib.OP_LOCAL_ENERGY, _lib.OP_PROP_STEP):
        full = lib.trot_cisd_workspace_size(ctypes.byref(_cisd()), 8, op)
        packed = lib.trot_cisd_workspace_size(ctypes.byref(_cisd(chol_symmetric=1)), 8, op)
        # + W N (N + 1) / 2 complex and G N (N + 1) / 2 real values, 256-byte aligned pieces
        assert packed - full >= 8 * 55 * 16 + 12 * 55 * 8, op
    assert lib.trot_cisd_workspace_size(ctypes.byref(_cisd()), 8, _lib.OP_OVERLAP) == \
        lib.trot_cisd_workspace_size(ctypes.byref(_cisd(chol_symmetric=1)), 8, _lib.OP_OVERLAP)
    # float-float gamma tile: N = 48 with 44 occupied orbitals fits the FP64 tiles but not the
    # float-float one (mixed gl)
    big = dict(norb=48, nocc=44, nvir=4)
    assert lib.trot_cisd_workspace_size(ctypes.byref(_cisd(**big)), 8, _lib.OP_LOCAL_ENERGY) > 0
    assert lib.trot_cisd_workspace_size(ctypes.byref(_cisd(gl_precision=_lib.MIXED, **big)), 8,
                                        _lib.OP_LOCAL_ENERGY) == 0
    assert b"exceeds shared memory" in lib.trot_last_error()


def test_packed_vhs_workspace():
    """With chol_packed set, the FP64 step and apply-Trotter workspaces carry the packed VHS
    (W N(N+1)/2 complex values, up to the carver's alignment); the other ops are unchanged."""
    lib = _lib.load()
    W, N = 40, 30
    full, packed = _sys(n_walkers=W, norb=N), _sys(n_walkers=W, norb=N, chol_packed=0x2000)
    extra = W * N * (N + 1) // 2 * 16
    for op in (_lib.OP_PROP_STEP, _lib.OP_APPLY_TROTTER):
        a = lib.trot_workspace_size(ctypes.byref(full), op)
        b = lib.trot_workspace_size(ctypes.byref(packed), op)
        assert extra <= b - a <= extra + 512, (op, a, b)
    for op in (_lib.OP_FORCE_BIAS, _lib.OP_LOCAL_ENERGY):
        assert lib.trot_workspace_size(ctypes.byref(full), op) == lib.trot_workspace_size(ctypes.byref(packed), op)
