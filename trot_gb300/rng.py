"""Device-side random numbers for the step (Philox-4x32-10, see csrc/rng.cu).

A key is an int64 (2,) CUDA tensor holding two uint32 words; ``normal_fields``
and ``uniform`` draw from the key's sub-key and then advance the key in place
(the reference's ``key, subkey = jax.random.split(key)`` pattern)."""
from __future__ import annotations

import torch

from . import _lib, native


def key(seed: int) -> torch.Tensor:
    seed = int(seed)
    from .core import device

    return torch.tensor([seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF], dtype=torch.int64, device=device())


def normal_fields(rng_key: torch.Tensor, n_walkers: int, nchol: int, out: torch.Tensor | None = None):
    if out is None:
        out = torch.empty((n_walkers, nchol), dtype=torch.float64, device=rng_key.device)
    _lib.call("trot_sample_normal_fields", rng_key.data_ptr(), int(n_walkers), int(nchol), out.data_ptr(),
              native.stream_ptr())
    _lib.call("trot_split_key", rng_key.data_ptr(), native.stream_ptr())
    return out


def uniform(rng_key: torch.Tensor, n: int = 1, out: torch.Tensor | None = None):
    if out is None:
        out = torch.empty((n,), dtype=torch.float64, device=rng_key.device)
    _lib.call("trot_sample_uniform", rng_key.data_ptr(), int(n), out.data_ptr(), native.stream_ptr())
    _lib.call("trot_split_key", rng_key.data_ptr(), native.stream_ptr())
    return out
