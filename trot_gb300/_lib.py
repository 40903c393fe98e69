"""ctypes binding of the C ABI in include/trot_gb300.h.

This is the only way the Python layer reaches the CUDA kernels.  Loading fails
loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

# trot_status
OK = 0
STATUS_NAMES = {
    0: "OK", 1: "BAD_SHAPE", 2: "BAD_DTYPE", 3: "NULL_PTR", 4: "WORKSPACE_TOO_SMALL",
    5: "CUDA_ERROR", 6: "DEVICE_TIMEOUT", 7: "NUMERIC_GUARD", 8: "UNSUPPORTED",
}
# trot_kind
RHF_R, RHF_U, UHF_U = 0, 1, 2
# trot_tune_knob
TUNE_EXCHANGE_TILES, TUNE_EXCHANGE_GRID, TUNE_TEST_TIMEOUT = 0, 1, 2
# trot_precision
FP64, MIXED = 0, 1
# trot_op
OP_FORCE_BIAS, OP_LOCAL_ENERGY, OP_APPLY_TROTTER, OP_PROP_STEP, OP_QR, OP_SR, OP_OVERLAP, OP_RDM1 = range(8)

_p = ctypes.c_void_p
_d = ctypes.c_double
_i = ctypes.c_int


class TrotMixed(ctypes.Structure):
    """trot_mixed (include/trot_gb300.h)."""

    _fields_ = [
        ("slices", _i), ("max_order", _i), ("kpad", _i), ("gammas_per_block", _i * 2), ("n_blocks", _i * 2),
        ("rot_slices", _p * 2), ("rot_exp", _p * 2), ("vhs_slices", _i), ("vhs_order", _i), ("n2pad", _i),
        ("gpad", _i), ("chol_t_slices", _p), ("exp_h1_half_f32", _p),
        ("exp_h1_half_img", _p), ("vhs_packed", _i), ("digit_format", _i),
    ]


class TrotSystem(ctypes.Structure):
    """trot_system (include/trot_gb300.h)."""

    _fields_ = [
        ("kind", _i), ("precision", _i), ("n_walkers", _i), ("norb", _i), ("nchol", _i),
        ("nocc_a", _i), ("nocc_b", _i), ("n_exp_terms", _i),
        ("h0", _d), ("h0_prop", _d), ("dt", _d), ("sqrt_dt", _d),
        ("weight_floor", _d), ("weight_cap", _d), ("pop_control_damping", _d),
        ("mo_a", _p), ("mo_b", _p), ("rot_h1_a", _p), ("rot_h1_b", _p),
        ("rot_chol_a", _p), ("rot_chol_b", _p), ("exp_h1_half", _p), ("chol_flat", _p),
        ("mf_shifts_im", _p), ("mixed", _p), ("chol_packed", _p),
    ]


class TrotState(ctypes.Structure):
    """trot_state (include/trot_gb300.h)."""

    _fields_ = [
        ("walkers_a", _p), ("walkers_b", _p), ("weights", _p), ("overlaps", _p),
        ("scalars", _p), ("node_encounters", _p),
    ]


class TrotCisd(ctypes.Structure):
    """trot_cisd (include/trot_gb300.h)."""

    _fields_ = [
        ("norb", _i), ("nocc", _i), ("nvir", _i), ("nchol", _i), ("h0", _d),
        ("ci1", _p), ("ci2m", _p), ("h1", _p), ("chol", _p), ("lci1", _p), ("mo", _p),
        ("l2ci2_precision", _i), ("gl_precision", _i), ("nvpad", _i), ("ncpad", _i), ("ci2_image", _p),
        ("chol_symmetric", _i),
    ]


class TrotError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        super().__init__(f"trot_gb300 error {STATUS_NAMES.get(status, status)}: {msg}")


_SIGNATURES = {
    "trot_last_error": (ctypes.c_char_p, []),
    "trot_abi_version": (_i, []),
    "trot_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(TrotSystem), _i]),
    "trot_overlap": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p]),
    "trot_half_green": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p]),
    "trot_force_bias": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_local_energy": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_apply_trotter": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_prop_step": (_i, [ctypes.POINTER(TrotSystem), ctypes.POINTER(TrotState), _p, _p, _p,
                            ctypes.c_size_t, _p]),
    "trot_orthonormalize": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p]),
    "trot_sr_resample": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _d, _p, _p, _p, _p, _p, _p, _p,
                              ctypes.c_size_t, _p]),
    "trot_block_energy": (_i, [_i, _p, _p, _p, _d, _d, _p, _p]),
    "trot_block_rdm1": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_sample_normal_fields": (_i, [_p, _i, _i, _p, _p]),
    "trot_sample_uniform": (_i, [_p, _i, _p, _p]),
    "trot_split_key": (_i, [_p, _p]),
    "trot_local_energy_noalloc": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p]),
    "trot_workspace_status": (_i, [_p, _p]),
    "trot_workspace_timeouts": (_i, [_p, _i, _p]),
    "trot_local_energy_noalloc_status": (_i, [_i, _p]),
    "trot_tc_gemm_bf16": (_i, [_p, _p, _p, _i, _i, _i, _p, _p]),
    "trot_cisd_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(TrotCisd), _i, _i]),
    "trot_cisd_overlap": (_i, [ctypes.POINTER(TrotCisd), _i, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_cisd_force_bias": (_i, [ctypes.POINTER(TrotCisd), _i, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_cisd_local_energy": (_i, [ctypes.POINTER(TrotCisd), _i, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_cisd_rdm1": (_i, [ctypes.POINTER(TrotCisd), _i, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_cisd_prop_step": (_i, [ctypes.POINTER(TrotCisd), ctypes.POINTER(TrotSystem), ctypes.POINTER(TrotState),
                                 _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_fp_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(TrotSystem)]),
    "trot_fp_step": (_i, [ctypes.POINTER(TrotSystem), ctypes.POINTER(TrotState), _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_prop_ctx_workspace_size": (ctypes.c_size_t, [_i, _i]),
    "trot_build_prop_ctx": (_i, [_i, _i, _d, _d, _p, _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_half_rotate": (_i, [_i, _i, _i, _p, _p, _p, _p, _p, _p]),
    "trot_cisd_lci1": (_i, [_i, _i, _i, _p, _p, _p, _p]),
    "trot_vjp_workspace_size": (ctypes.c_size_t, [ctypes.POINTER(TrotSystem), _i]),
    "trot_prop_step_vjp": (_i, [ctypes.POINTER(TrotSystem), ctypes.POINTER(TrotState), _p, _p, _p, _p, _p, _p, _p,
                                _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_local_energy_vjp": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_overlap_vjp": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_orthonormalize_vjp": (_i, [ctypes.POINTER(TrotSystem), _p, _p, _p, _p, _p, _p, _p, _p, _p]),
    "trot_prop_ctx_vjp_workspace_size": (ctypes.c_size_t, [_i, _i]),
    "trot_prop_ctx_vjp": (_i, [_i, _i, _d, _p, _p, _p, _p, _p, _p, ctypes.c_size_t, _p]),
    "trot_set_tuning": (_i, [_i, _i]),
    "trot_get_tuning": (_i, [_i]),
    "trot_profile_enable": (_i, [_i]),
    "trot_profile_collect": (_i, [_i, ctypes.c_char_p, _p, _p]),
    "trot_profile_launch_count": (ctypes.c_longlong, []),
}

_lock = threading.Lock()
_lib = None


def exported_symbols():
    return sorted(_SIGNATURES)


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libtrot_gb300.so (building it first when the sources are present)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.lib_path()
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"trot_gb300 CUDA library not found at {path}; run trot_gb300.build")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.trot_abi_version() != 4:
            raise RuntimeError("trot_gb300 ABI version mismatch")
        _lib = lib
        return lib


def check(status: int) -> None:
    if status != OK:
        msg = load(False).trot_last_error().decode(errors="replace")
        raise TrotError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))


def profile_enable(max_launches: int = 4096) -> None:
    check(load().trot_profile_enable(int(max_launches)))


def profile_launch_count() -> int:
    """Kernel launches of the library since the last profile_enable (all of them)."""
    return int(load().trot_profile_launch_count())


def profile_collect(max_names: int = 64) -> dict:
    """{kernel name: (total ms, launches)} since the last collect (synchronises)."""
    import numpy as np

    names = ctypes.create_string_buffer(48 * max_names)
    ms = np.zeros(max_names, dtype=np.float64)
    cnt = np.zeros(max_names, dtype=np.int32)
    n = load().trot_profile_collect(max_names, names, ms.ctypes.data, cnt.ctypes.data)
    if n < 0:
        check(-n)
    raw = names.raw
    out = {}
    for k in range(n):
        nm = raw[48 * k: 48 * k + 48].split(b"\0", 1)[0].decode()
        out[nm] = (float(ms[k]), int(cnt[k]))
    return out
