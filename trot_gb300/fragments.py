"""Batched uneven fragment Hamiltonians (the LNO-style workload: many
independent small systems, each with its own walkers, trial and integrals).

Each fragment is a full hot-path instance (its own contexts, state and
workspace) and runs on its own CUDA stream, so the kernels of small fragments
fill the GPU side by side instead of queueing behind each other.  One step
(phaseless step + local energy) of every fragment is captured once into a
single CUDA graph - fork from the launching stream, one branch per fragment,
join - and replayed: one graph launch per step for the whole batch.
Fragments with N <= 128 orbitals use the tensor-core path when ``mixed`` is
set; larger ones run the FP64 kernels (the exact-slice exchange tiles hold at
most 128 orbitals).  Scheduling is by size: the largest fragments are issued
first so they start before the small ones fill the machine.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np
import torch

from . import synthetic
from .core import HamChol, QmcParams, System
from .meas import make_rhf_meas_ops
from .prop import make_prop_ops
from .trial import RhfTrial, make_rhf_trial_ops

MIXED_MAX_NORB = 128


@dataclass
class Fragment:
    norb: int
    nocc: int
    nchol: int
    n_walkers: int
    mixed: bool
    sys: Any
    ham: Any
    trial: Any
    trial_ops: Any
    meas_ops: Any
    meas_ctx: Any
    prop_ops: Any
    prop_ctx: Any
    params: Any
    state: Any
    energy: torch.Tensor
    stream: torch.cuda.Stream


def lno_fragment_sizes(n_fragments: int = 24, nmin: int = 30, nmax: int = 160, seed: int = 5):
    """Fragment sizes of the uneven-fragment workload: N ~ U[nmin, nmax],
    nocc = round(0.12 N), nchol = 4 N."""
    rng = np.random.default_rng(seed)
    sizes = []
    for n in rng.integers(nmin, nmax + 1, size=n_fragments):
        n = int(n)
        sizes.append((n, max(1, int(round(0.12 * n))), 4 * n))
    return sizes


def make_fragment(norb, nocc, nchol, n_walkers, *, dt=0.005, seed=0, mixed=True, decay=30.0) -> Fragment:
    """RHF trial + restricted walkers on a seeded synthetic fragment Hamiltonian."""
    ss = synthetic.make_system(norb, (nocc, nocc), nchol, decay=decay, seed=seed, h0=0.0)
    use_mixed = bool(mixed and norb <= MIXED_MAX_NORB and nocc <= 16)
    sysm = System(norb=norb, nelec=(nocc, nocc), walker_kind="restricted")
    ham = HamChol(h0=ss.h0, h1=ss.h1, chol=ss.chol)
    trial = RhfTrial(ss.mo_a)
    trial_ops = make_rhf_trial_ops(sysm)
    meas_ops = make_rhf_meas_ops(sysm, mixed_precision=use_mixed)
    meas_ctx = meas_ops.build_meas_ctx(ham, trial)
    params = QmcParams(dt=dt, n_walkers=n_walkers, n_prop_steps=10, seed=1000 + seed)
    prop_ops = make_prop_ops("restricted", "restricted", mixed_precision=use_mixed)
    prop_ctx = prop_ops.build_prop_ctx(ham, trial_ops.get_rdm1(trial), params)
    state = prop_ops.init_prop_state(sys=sysm, ham_data=ham, trial_ops=trial_ops, trial_data=trial,
                                     meas_ops=meas_ops, params=params)
    energy = torch.empty(n_walkers, dtype=torch.complex128, device=state.weights.device)
    return Fragment(norb, nocc, nchol, n_walkers, use_mixed, sysm, ham, trial, trial_ops, meas_ops, meas_ctx,
                    prop_ops, prop_ctx, params, state, energy, torch.cuda.Stream())


class FragmentBatch:
    """Steps every fragment of a batch; ``capture()`` records one batched step as
    a CUDA graph and ``step()`` then replays it."""

    def __init__(self, fragments: list[Fragment]):
        # largest first: the long-running fragments start before the small ones fill the GPU
        self.fragments = sorted(fragments, key=lambda f: -f.norb * f.norb * f.nchol * f.n_walkers)
        self.graph = None

    def _issue(self):
        main = torch.cuda.current_stream()
        for f in self.fragments:
            f.stream.wait_stream(main)
            with torch.cuda.stream(f.stream):
                f.prop_ops.step(f.state, params=f.params, ham_data=f.ham, trial_data=f.trial,
                                trial_ops=f.trial_ops, meas_ops=f.meas_ops, meas_ctx=f.meas_ctx,
                                prop_ctx=f.prop_ctx, energy_out=f.energy)
        for f in self.fragments:
            main.wait_stream(f.stream)

    def step(self):
        """One phaseless step + local energy of every fragment."""
        if self.graph is not None:
            self.graph.replay()
        else:
            self._issue()

    def capture(self):
        """Record one batched step (after at least one eager step, which sizes
        every workspace) as a CUDA graph; later ``step()`` calls replay it."""
        g = torch.cuda.CUDAGraph()
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self._issue()
        self.graph = g
        return g

    @property
    def walker_steps_per_step(self) -> int:
        return sum(f.n_walkers for f in self.fragments)
