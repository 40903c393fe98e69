"""CISD trial with restricted walkers (trot/trial/cisd.py, trot/meas/cisd.py)
on the CUDA library.

The trial, meas ops and trial ops keep the reference's names and call
signatures; every kernel takes the whole walker batch and makes one call into
the C ABI (``trot_cisd_*`` in include/trot_gb300.h).  The whole orbital
space is active (``nocc_t_core == nvir_t_outer == 0``).

Precision follows the reference's two switches (trot/meas/cisd.py:823-839):
``testing=True`` keeps every contraction in float64 (the reference's float64
``*_testing`` dtypes); with ``testing=False`` the l2ci2 quadratic forms run on
the tensor cores (3-term BF16 split, FP32 accumulation; the reference uses
float32 there).  ``mixed_precision=True`` computes gl = G L_g and lci2_green
in FP32 (the reference's float32 ``mixed_real_dtype``); overlaps, ci2g, the
Cholesky contractions and every energy sum stay float64.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, native, rng
from . import ctx as ctx_dev
from .core import (HamChol, MeasOps, PropState, System, TrialOps, as_dev, batched, k_energy, k_force_bias,
                   o_rdm1, real_part)


@dataclass(frozen=True)
class CisdTrial:
    """trot/trial/cisd.py:14-88: ci1 (nocc, nvir), ci2 (nocc, nvir, nocc, nvir)
    in the (i, a, j, b) layout, real float64 on the device."""

    ci1: torch.Tensor
    ci2: torch.Tensor
    nocc_t_core: int = 0
    nvir_t_outer: int = 0

    def __post_init__(self):
        object.__setattr__(self, "ci1", as_dev(real_part(self.ci1, "ci1")))
        object.__setattr__(self, "ci2", as_dev(real_part(self.ci2, "ci2")))
        n, v = self.ci1.shape
        if tuple(self.ci2.shape) != (n, v, n, v):
            raise ValueError(f"ci2 shape {tuple(self.ci2.shape)} != {(n, v, n, v)}")

    @property
    def nocc(self) -> int:
        return int(self.ci1.shape[0])

    @property
    def nvir(self) -> int:
        return int(self.ci1.shape[1])

    @property
    def nocc_full(self) -> int:
        return int(self.nocc_t_core + self.nocc)

    @property
    def nvir_full(self) -> int:
        return int(self.nvir + self.nvir_t_outer)

    @property
    def norb(self) -> int:
        return int(self.nocc_full + self.nvir_full)

    @property
    def occ_act_slice(self) -> slice:
        return slice(self.nocc_t_core, self.nocc_full)

    @property
    def vir_act_slice(self) -> slice:
        return slice(self.nocc_full, self.nocc_full + self.nvir)

    @property
    def norb_act(self) -> int:
        return int(self.nocc + self.nvir)

    def coeffs(self):
        """Reference determinant (first nocc columns of the identity) for both spins."""
        mo = _trial_dev(self)["mo"]
        return mo, mo


def _trial_dev(trial: CisdTrial) -> dict:
    """Device operands derived once per trial: ci2m[(i,a),(j,b)] = 2 c_iajb - c_ibja
    as an (nv, nv) matrix, the only combination of the doubles the kernels use."""
    d = trial.__dict__.get("_dev")
    if d is None:
        if trial.nocc_t_core != 0 or trial.nvir_t_outer != 0:
            raise NotImplementedError("CUDA path: CISD trial with a frozen core or outer virtuals")
        n, v = trial.nocc, trial.nvir
        d = {
            "ci1": trial.ci1.contiguous(),
            "ci2m": (2.0 * trial.ci2 - trial.ci2.permute(0, 3, 2, 1)).reshape(n * v, n * v).contiguous(),
            "mo": torch.eye(n + v, dtype=torch.float64, device=trial.ci1.device)[:, :n].contiguous(),
        }
        object.__setattr__(trial, "_dev", d)
    return d


def get_rdm1(trial_data: CisdTrial) -> torch.Tensor:
    """trot/trial/cisd.py:91-96: the reference determinant's 1-RDM for both spins."""
    N, n = trial_data.norb, trial_data.nocc_full
    occ = (torch.arange(N, device=trial_data.ci1.device) < n).to(torch.float64)
    dm = torch.diag(occ)
    return torch.stack([dm, dm])


@dataclass(frozen=True)
class CisdMeasCfg:
    """trot/meas/cisd.py:47-53 (the dtype fields reduce to the two flags)."""

    memory_mode: str = "high"
    mixed_precision: bool = True
    testing: bool = False


@dataclass(frozen=True)
class CisdMeasCtx:
    """trot/meas/cisd.py:63-80: rot_chol (G, nocc, N), lci1 (G, N, nocc), cfg;
    plus the device copies of h1, chol and h0 the kernels read."""

    rot_chol: torch.Tensor
    lci1: torch.Tensor
    cfg: CisdMeasCfg
    h1: torch.Tensor
    chol: torch.Tensor
    h0: float
    ci2_image: torch.Tensor | None = None  # ci2m split-BF16 image (testing=False)
    nvpad: int = 0
    ncpad: int = 0
    chol_symmetric: bool = False  # every chol[g] symmetric: packed-triangle contraction


def build_meas_ctx(ham_data: HamChol, trial_data: CisdTrial, cfg: CisdMeasCfg = CisdMeasCfg()) -> CisdMeasCtx:
    """trot/meas/cisd.py:92-110: lci1[g][i][p] = sum_a chol[g][i][nocc + a] ci1[p][a]."""
    if ham_data.basis != "restricted":
        raise ValueError("CISD MeasOps currently assumes HamChol.basis == 'restricted'.")
    h1 = ctx_dev.real_dev(ham_data.h1, "h1")
    chol = ctx_dev.real_dev(ham_data.chol, "chol")
    if chol.shape[1] != trial_data.norb:
        raise ValueError(f"chol norb {chol.shape[1]} != trial norb {trial_data.norb}")
    n = trial_data.nocc_full
    lci1 = ctx_dev.cisd_lci1(trial_data.ci1, chol)  # whole orbital space active: vir_act_slice = nocc..N
    h0 = ham_data.h0.item() if isinstance(ham_data.h0, torch.Tensor) else ham_data.h0
    img, ncpad, nvpad = None, 0, 0
    if not cfg.testing:
        from . import mixed

        bt = _trial_dev(trial_data)["ci2m"].T.cpu().numpy()  # (nv columns, nv K)
        img, ncpad, nvpad = mixed.split3_image(bt)
        img = img.to(chol.device)
    # Cholesky vectors of real two-electron integrals are symmetric matrices (to rounding after a
    # basis rotation); checked once here: the packed contraction uses (L + L^T) / 2
    amax = float(chol.abs().max()) if chol.numel() else 0.0
    sym = bool(float((chol - chol.transpose(1, 2)).abs().max()) <= 1e-12 * amax) if chol.numel() else False
    return CisdMeasCtx(rot_chol=chol[:, :n, :], lci1=lci1, cfg=cfg, h1=h1, chol=chol,
                       h0=float(np.real(np.asarray(h0))), ci2_image=img, nvpad=nvpad, ncpad=ncpad,
                       chol_symmetric=sym)


def _struct(trial: CisdTrial, meas_ctx: CisdMeasCtx | None) -> _lib.TrotCisd:
    d = _trial_dev(trial)
    c = _lib.TrotCisd()
    c.norb, c.nocc, c.nvir = trial.norb, trial.nocc, trial.nvir
    c.ci1, c.ci2m, c.mo = (native.ptr(d[k]) for k in ("ci1", "ci2m", "mo"))
    c.nchol = 1
    if meas_ctx is not None:
        c.nchol = int(meas_ctx.chol.shape[0])
        c.h0 = meas_ctx.h0
        c.h1, c.chol, c.lci1 = native.ptr(meas_ctx.h1), native.ptr(meas_ctx.chol), native.ptr(meas_ctx.lci1)
        c.gl_precision = _lib.MIXED if meas_ctx.cfg.mixed_precision else _lib.FP64
        c.chol_symmetric = 1 if meas_ctx.chol_symmetric else 0
        if meas_ctx.ci2_image is not None:
            c.l2ci2_precision = _lib.MIXED
            c.ci2_image, c.nvpad, c.ncpad = meas_ctx.ci2_image.data_ptr(), meas_ctx.nvpad, meas_ctx.ncpad
    return c


def _workspace(c: _lib.TrotCisd, W: int, op: int) -> tuple[int, int]:
    n = _lib.load().trot_cisd_workspace_size(ctypes.byref(c), W, op)
    if n == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    buf = native.workspace(n)
    return buf.data_ptr(), buf.numel()


def _check(walkers, trial):
    if isinstance(walkers, tuple):
        raise TypeError("CISD: restricted walkers must be one (W, N, nocc) tensor")
    native.check_walker_tensor(walkers, trial.norb, trial.nocc_full)
    return int(walkers.shape[0])


def _call(name, op, walkers, trial, meas_ctx, out):
    W = _check(walkers, trial)
    c = _struct(trial, meas_ctx)
    ws, nws = _workspace(c, W, op)
    _lib.call(name, ctypes.byref(c), W, walkers.data_ptr(), out.data_ptr(), ws, nws, native.stream_ptr())
    return out


def overlap_batched(walkers, trial_data: CisdTrial) -> torch.Tensor:
    """overlap_r_high (trot/trial/cisd.py:148-186) for a (W, N, nocc) batch."""
    out = torch.empty(_check(walkers, trial_data), dtype=torch.complex128, device=walkers.device)
    return _call("trot_cisd_overlap", _lib.OP_OVERLAP, walkers, trial_data, None, out)


def force_bias_batched(walkers, ham_data, meas_ctx: CisdMeasCtx, trial_data: CisdTrial) -> torch.Tensor:
    """force_bias_kernel_rw_rh (trot/meas/cisd.py:548-605): (W, G) complex128."""
    W = _check(walkers, trial_data)
    out = torch.empty((W, meas_ctx.chol.shape[0]), dtype=torch.complex128, device=walkers.device)
    return _call("trot_cisd_force_bias", _lib.OP_FORCE_BIAS, walkers, trial_data, meas_ctx, out)


def local_energy_batched(walkers, ham_data, meas_ctx: CisdMeasCtx, trial_data: CisdTrial) -> torch.Tensor:
    """energy_kernel_rw_rh (trot/meas/cisd.py:608-769): (W,) complex128."""
    out = torch.empty(_check(walkers, trial_data), dtype=torch.complex128, device=walkers.device)
    return _call("trot_cisd_local_energy", _lib.OP_LOCAL_ENERGY, walkers, trial_data, meas_ctx, out)


def rdm1_batched(walkers, ham_data, meas_ctx: CisdMeasCtx, trial_data: CisdTrial) -> torch.Tensor:
    """rdm1_kernel_rw (trot/meas/cisd.py:772-820): (W, 2, N, N) complex128."""
    N = trial_data.norb
    g = torch.empty((_check(walkers, trial_data), N, N), dtype=torch.complex128, device=walkers.device)
    _call("trot_cisd_rdm1", _lib.OP_FORCE_BIAS, walkers, trial_data, meas_ctx, g)
    return torch.stack([g, g], dim=1)


@batched
def cisd_overlap_r(walkers, trial_data):
    return overlap_batched(walkers, trial_data)


@batched
def _force_bias(walkers, ham_data, meas_ctx, trial_data):
    return force_bias_batched(walkers, ham_data, meas_ctx, trial_data)


@batched
def _energy(walkers, ham_data, meas_ctx, trial_data):
    return local_energy_batched(walkers, ham_data, meas_ctx, trial_data)


@batched
def _rdm1(walkers, ham_data, meas_ctx, trial_data):
    return rdm1_batched(walkers, ham_data, meas_ctx, trial_data)


def make_cisd_trial_data(data: dict, sys: System) -> CisdTrial:
    """trot/trial/cisd.py:203-213."""
    def count(key):
        return int(np.asarray(data[key].cpu() if isinstance(data.get(key), torch.Tensor) else data.get(key, 0)).item())
    return CisdTrial(ci1=data["ci1"], ci2=data["ci2"], nocc_t_core=count("nocc_t_core"),
                     nvir_t_outer=count("nvir_t_outer"))


def make_cisd_trial_ops(sys: System, memory_mode: str = "high") -> TrialOps:
    """trot/trial/cisd.py:189-201."""
    if sys.nup != sys.ndn:
        raise ValueError("Restricted CISD trial requires nup == ndn.")
    if sys.walker_kind.lower() != "restricted":
        raise ValueError(f"CISD trial currently supports only restricted walkers, got: {sys.walker_kind}")
    if memory_mode not in ("high", "low"):
        raise ValueError(f"Unsupported CISD trial memory_mode: {memory_mode!r}")
    return TrialOps(overlap=cisd_overlap_r, get_rdm1=get_rdm1)


def make_cisd_meas_ops(sys: System, memory_mode: str = "high", mixed_precision: bool = True,
                       testing: bool = False) -> MeasOps:
    """trot/meas/cisd.py:823-852.  "high" and "low" memory modes compute the
    same numbers here (the CUDA kernels stream over Cholesky vectors)."""
    if sys.walker_kind.lower() != "restricted":
        raise ValueError(f"CISD MeasOps currently supports only restricted walkers, got: {sys.walker_kind}")
    if memory_mode not in ("high", "low"):
        raise ValueError(f"Unsupported CISD memory_mode: {memory_mode!r}")
    cfg = CisdMeasCfg(memory_mode=memory_mode, mixed_precision=mixed_precision, testing=testing)
    ops = MeasOps(
        overlap=cisd_overlap_r,
        build_meas_ctx=lambda ham_data, trial_data: build_meas_ctx(ham_data, trial_data, cfg),
        kernels={k_force_bias: _force_bias, k_energy: _energy},
        observables={o_rdm1: _rdm1},
    )
    object.__setattr__(ops, "walker_kind", "restricted")
    return ops


def afqmc_step(state: PropState, *, params, ham_data, trial_data: CisdTrial, meas_ctx: CisdMeasCtx, prop_ctx,
               fields=None, energy_out=None, precision: int = _lib.FP64) -> PropState:
    """trot/prop/afqmc.py:79-144 with the CISD meas ops, as one call
    (``trot_cisd_prop_step``); the state's buffers are updated in place.
    ``precision`` = MIXED propagates on the tensor cores (VHS, Taylor action)."""
    w = state.walkers
    W = _check(w, trial_data)
    c = _struct(trial_data, meas_ctx)
    G = c.nchol
    if int(prop_ctx.chol_flat.shape[0]) != G:
        raise ValueError("propagation and measurement contexts disagree on nchol")
    s = _lib.TrotSystem()
    s.kind, s.precision, s.n_walkers = _lib.RHF_R, _lib.FP64, W
    s.norb, s.nchol, s.nocc_a = trial_data.norb, G, trial_data.nocc
    s.mo_a = c.mo
    s.exp_h1_half, s.chol_flat = native.ptr(prop_ctx.exp_h1_half), native.ptr(prop_ctx.chol_flat)
    s.mf_shifts_im = native.ptr(prop_ctx.mf_shifts_im)
    s.h0_prop, s.dt, s.sqrt_dt = float(prop_ctx.h0_prop), float(prop_ctx.dt), float(prop_ctx.sqrt_dt)
    s.n_exp_terms = int(params.n_exp_terms)
    s.weight_floor = float(getattr(params, "weight_floor", 1.0e-3))
    s.weight_cap = float(getattr(params, "weight_cap", 100.0))
    s.pop_control_damping = float(getattr(params, "pop_control_damping", 0.1))
    extra = 0
    if precision == _lib.MIXED:
        from . import mixed

        mx = mixed.context(None, prop_ctx)
        s.precision, s.mixed = _lib.MIXED, mx.data_ptr()
        extra = _lib.load().trot_workspace_size(ctypes.byref(s), _lib.OP_APPLY_TROTTER) + 256
    if fields is None:
        fields = rng.normal_fields(state.rng_key, W, G)
    elif fields.dtype != torch.float64 or not fields.is_cuda or tuple(fields.shape) != (W, G):
        raise ValueError("fields must be a (W, G) float64 CUDA tensor")
    fields = fields.contiguous()
    st = _lib.TrotState()
    st.walkers_a, st.walkers_b = w.data_ptr(), 0
    st.weights, st.overlaps = state.weights.data_ptr(), state.overlaps.data_ptr()
    st.scalars, st.node_encounters = state.scalars.data_ptr(), state.node_encounters.data_ptr()
    n = _lib.load().trot_cisd_workspace_size(ctypes.byref(c), W, _lib.OP_PROP_STEP)
    if n == 0:
        raise _lib.TrotError(1, _lib.load().trot_last_error().decode())
    buf = native.workspace(n + 256 + extra)
    ws, nws = buf.data_ptr(), buf.numel()
    _lib.call("trot_cisd_prop_step", ctypes.byref(c), ctypes.byref(s), ctypes.byref(st), fields.data_ptr(),
              native.ptr(energy_out), ws, nws, native.stream_ptr())
    return state
