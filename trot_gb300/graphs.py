"""A whole AFQMC block as one CUDA graph (trot/prop/blocks.py:195-287 with the
step of trot/prop/afqmc.py:79-144).

``GraphedBlock`` records ``n_prop_steps`` phaseless steps, the QR, overlaps,
local energy, block energy + EMA and the stochastic reconfiguration - fields
and zeta drawn on the device from the state's key - once, then replays the
recording: one graph launch per block, no host work and no host
synchronisation between blocks.  The state's tensors are persistent buffers:
each replay reads them and writes the next block's state back into them, so
successive replays continue the same Markov chain an eager ``block`` loop would
(bit-identical, tested).  Every library call in the block is capturable: the
C ABI issues only kernel launches, memsets and device-to-device copies on the
caller's stream and never synchronises.
"""
from __future__ import annotations

import torch

from .blocks import block
from .core import PropState


def _copy_into(dst, src):
    if isinstance(dst, tuple):
        for d, s in zip(dst, src):
            d.copy_(s)
    else:
        dst.copy_(src)


class GraphedBlock:
    """Capture ``block(state, **kw)`` (``kw``: sys, params, ham_data, trial_data,
    trial_ops, meas_ops, meas_ctx, prop_ops, prop_ctx) into a CUDA graph.

    ``state`` is used as the persistent state: after ``replay()`` it holds the
    state after one more block, and the returned observables (device scalars
    ``energy``, ``weight``) are that block's."""

    def __init__(self, state: PropState, **kw):
        self.state = state
        self.kw = kw
        # eager warm-up on a copy: builds the cached contexts and grows every workspace
        # to its final size, so nothing is allocated or copied from the host under capture
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            block(state.clone(), **kw)
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            out, obs = block(self.state, **kw)
            _copy_into(self.state.walkers, out.walkers)
            self.state.weights.copy_(out.weights)
            self.state.overlaps.copy_(out.overlaps)
            self._energy = obs.scalars["energy"]
            self._weight = obs.scalars["weight"]

    def replay(self, check: bool = False) -> dict:
        """Run one block; returns its device scalars {"energy", "weight"}.  With
        ``check`` the host waits for the block and raises TrotError(DEVICE_TIMEOUT)
        if a tensor-core kernel of it timed out (its results are NaN then)."""
        self.graph.replay()
        if check:
            from . import native

            native.check_device_timeouts("graphed block")
        return {"energy": self._energy, "weight": self._weight}
