"""Helpers for GPU tests: build trot_gb300 objects from golden files / synthetic systems."""
from __future__ import annotations

import numpy as np
import torch

import trot_gb300 as tg


def dev(x, dtype=None):
    t = torch.as_tensor(np.ascontiguousarray(x))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda().contiguous()


def cpu(x):
    if isinstance(x, tuple):
        return tuple(cpu(a) for a in x)
    return x.detach().cpu().numpy()


class Setup:
    """trot_gb300 objects for one (trial, walker) kind."""

    def __init__(self, kind, h0, h1, chol, mo_a, mo_b, dt, n_walkers, mixed=False, n_exp_terms=6):
        self.kind = kind
        wk = "restricted" if kind == "rhf_r" else "unrestricted"
        N = h1.shape[0]
        na, nb = mo_a.shape[1], mo_b.shape[1]
        self.sys = tg.System(norb=N, nelec=(na, nb), walker_kind=wk)
        self.ham = tg.HamChol(h0=h0, h1=h1, chol=chol)
        self.params = tg.QmcParams(dt=dt, n_walkers=n_walkers, n_exp_terms=n_exp_terms, seed=7)
        if kind == "uhf_u":
            self.trial = tg.UhfTrial(mo_a, mo_b)
            self.trial_ops = tg.make_uhf_trial_ops(self.sys)
            self.meas_ops = tg.make_uhf_meas_ops(self.sys, mixed_precision=mixed)
        else:
            self.trial = tg.RhfTrial(mo_a)
            self.trial_ops = tg.make_rhf_trial_ops(self.sys)
            self.meas_ops = tg.make_rhf_meas_ops(self.sys, mixed_precision=mixed)
        self.meas_ctx = self.meas_ops.build_meas_ctx(self.ham, self.trial)
        self.prop_ops = tg.make_prop_ops("restricted", wk, mixed_precision=mixed)
        rdm1 = self.trial_ops.get_rdm1(self.trial)
        self.prop_ctx = self.prop_ops.build_prop_ctx(self.ham, rdm1, self.params)
        self.walker_kind = wk

    @classmethod
    def from_golden(cls, g, mixed=False):
        return cls(str(g["kind"]), float(g["h0"]), g["h1"], g["chol"], g["mo_a"], g["mo_b"], float(g["dt"]),
                   int((g["walkers"] if str(g["kind"]) == "rhf_r" else g["walkers_u"]).shape[0]), mixed=mixed)

    def walkers(self, w):
        if isinstance(w, tuple):
            return (dev(w[0]), dev(w[1]))
        return dev(w)

    def force_bias(self, w):
        return self.meas_ops.kernels["force_bias"](w, self.ham, self.meas_ctx, self.trial)

    def energy(self, w):
        return self.meas_ops.kernels["energy"](w, self.ham, self.meas_ctx, self.trial)

    def overlap(self, w):
        return self.meas_ops.overlap(w, self.trial)

    def state(self, walkers, weights, overlaps, shift, e_est):
        W = weights.shape[0]
        return tg.PropState(walkers=walkers, weights=dev(weights), overlaps=dev(overlaps),
                            rng_key=tg.rng.key(3), scalars=dev(np.array([shift, e_est], dtype=np.float64)),
                            node_encounters=torch.zeros(1, dtype=torch.int64, device="cuda"))

    def step(self, state, fields, energy_out=None):
        return self.prop_ops.step(state, params=self.params, ham_data=self.ham, trial_data=self.trial,
                                  trial_ops=self.trial_ops, meas_ops=self.meas_ops, meas_ctx=self.meas_ctx,
                                  prop_ctx=self.prop_ctx, fields=fields, energy_out=energy_out)


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
