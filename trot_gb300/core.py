"""Core types of the hot-path interface, mirroring trot's.

* ``System``      — trot/core/system.py:10-35
* ``HamChol``     — trot/ham/chol.py:14-58
* ``TrialOps``, ``MeasOps`` and kernel names — trot/core/ops.py:49-166
* ``QmcParams*``  — trot/prop/types.py:30-62
* ``PropState``, ``PropOps`` — trot/prop/types.py:20-27,99-103

Arrays are torch tensors on the CUDA device.  Measurement kernels take the
whole walker batch (leading axis W) and are marked ``batched`` so that
``walkers.vmap_chunked`` calls them once instead of mapping them per walker.
"""
from __future__ import annotations

from dataclasses import dataclass, field, fields, replace
from typing import Any, Callable, Mapping, NamedTuple, Tuple

import numpy as np
import torch

k_energy = "energy"
k_force_bias = "force_bias"
o_rdm1 = "rdm1"
o_density_corr = "density_corr"


@dataclass(frozen=True)
class System:
    norb: int
    nelec: Tuple[int, int]
    walker_kind: str

    def __post_init__(self):
        object.__setattr__(self, "walker_kind", self.walker_kind.lower())

    @property
    def nup(self) -> int:
        return self.nelec[0]

    @property
    def ndn(self) -> int:
        return self.nelec[1]

    @property
    def ne(self) -> int:
        return self.nelec[0] + self.nelec[1]


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("trot_gb300 needs a CUDA device (no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def as_dev(x, dtype=torch.float64) -> torch.Tensor:
    """Copy a numpy array / tensor to the current CUDA device, contiguous."""
    if isinstance(x, torch.Tensor):
        return x.to(device=device(), dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(x)).to(device=device(), dtype=dtype).contiguous()


def real_part(x, name: str) -> np.ndarray:
    """Host copy of a real-valued array; complex input must have zero imaginary part."""
    a = x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
    if np.iscomplexobj(a):
        if np.any(np.imag(a) != 0):
            raise NotImplementedError(f"{name}: complex-valued input is not supported by the CUDA path")
        a = np.real(a)
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass(frozen=True)
class HamChol:
    """Cholesky Hamiltonian: h0 scalar, h1 (N, N), chol (G, N, N) (basis "restricted")."""

    h0: Any
    h1: Any
    chol: Any
    basis: str = "restricted"
    nchol: int | None = None

    def __post_init__(self):
        if self.basis not in ("restricted", "generalized"):
            raise ValueError(f"unknown basis: {self.basis}")
        shape = getattr(self.chol, "shape", None)
        if shape is None:
            return
        if self.nchol is None:
            object.__setattr__(self, "nchol", int(shape[0]))
        elif int(shape[0]) not in (0, int(self.nchol)):
            raise ValueError(f"nchol={self.nchol} is inconsistent with chol.shape[0]={shape[0]}")


def batched(fn: Callable) -> Callable:
    """Mark a kernel as taking the whole walker batch."""
    fn.batched = True
    return fn


class TrialOps(NamedTuple):
    overlap: Callable
    get_rdm1: Callable
    calc_green: Callable | None = None
    calc_overlap_ratio: Callable | None = None
    update_green: Callable | None = None


@dataclass(frozen=True)
class MeasOps:
    overlap: Callable
    build_meas_ctx: Callable = lambda ham_data, trial_data: None
    kernels: Mapping[str, Callable] = field(default_factory=dict)
    observables: Mapping[str, Callable] = field(default_factory=dict)

    def has_kernel(self, name: str) -> bool:
        return name in self.kernels

    def has_observable(self, name: str) -> bool:
        return name in self.observables

    def require_kernel(self, name: str) -> Callable:
        try:
            return self.kernels[name]
        except KeyError as e:
            avail = ", ".join(sorted(self.kernels.keys()))
            raise KeyError(f"missing required kernel '{name}'. available: [{avail}]") from e

    def require_observable(self, name: str) -> Callable:
        try:
            return self.observables[name]
        except KeyError as e:
            avail = ", ".join(sorted(self.observables.keys()))
            raise KeyError(f"missing requested observable '{name}'. available: [{avail}]") from e

    def available_kernels(self) -> tuple[str, ...]:
        return tuple(sorted(self.kernels.keys()))

    def available_observables(self) -> tuple[str, ...]:
        return tuple(sorted(self.observables.keys()))


def _random_seed() -> int:
    return int(np.random.randint(0, int(1e6)))


@dataclass(frozen=True)
class QmcParamsBase:
    dt: float = 0.005
    n_chunks: int = 1
    n_exp_terms: int = 6
    n_prop_steps: int = 50
    n_blocks: int = 200
    n_walkers: int = 200
    seed: int = field(default_factory=_random_seed)


@dataclass(frozen=True)
class QmcParams(QmcParamsBase):
    pop_control_damping: float = 0.1
    weight_floor: float = 1.0e-3
    weight_cap: float = 100.0
    shift_ema: float = 0.1
    n_eql_blocks: int = 20


@dataclass(frozen=True)
class QmcParamsFp(QmcParamsBase):
    """Free-projection parameters (trot/prop/types.py:55-62)."""

    dt: float = 0.05
    n_prop_steps: int = 20
    n_qr_blocks: int = 10
    n_blocks: int = 5
    ene0: float | None = None
    n_traj: int = 10


@dataclass
class PropState:
    """Walker population and running scalars.

    Same fields as trot's ``PropState``.  ``pop_control_ene_shift`` and
    ``e_estimate`` are 0-d views into one device buffer ``scalars`` (2,) so the
    CUDA step can update them without a host round trip; ``rng_key`` is an
    int64 (2,) device tensor holding two uint32 words."""

    walkers: Any
    weights: torch.Tensor
    overlaps: torch.Tensor
    rng_key: torch.Tensor
    scalars: torch.Tensor
    node_encounters: torch.Tensor

    @property
    def pop_control_ene_shift(self) -> torch.Tensor:
        return self.scalars[0]

    @property
    def e_estimate(self) -> torch.Tensor:
        return self.scalars[1]

    def _replace(self, **kw) -> "PropState":
        if "pop_control_ene_shift" in kw or "e_estimate" in kw:
            sc = self.scalars.clone()
            if "pop_control_ene_shift" in kw:
                sc[0] = torch.as_tensor(kw.pop("pop_control_ene_shift"), dtype=torch.float64)
            if "e_estimate" in kw:
                sc[1] = torch.as_tensor(kw.pop("e_estimate"), dtype=torch.float64)
            kw["scalars"] = sc
        return replace(self, **kw)

    def clone(self) -> "PropState":
        w = self.walkers
        w = tuple(x.clone() for x in w) if isinstance(w, tuple) else w.clone()
        return PropState(w, self.weights.clone(), self.overlaps.clone(), self.rng_key.clone(),
                         self.scalars.clone(), self.node_encounters.clone())


@dataclass(frozen=True)
class PropOps:
    init_prop_state: Callable
    build_prop_ctx: Callable
    step: Callable
