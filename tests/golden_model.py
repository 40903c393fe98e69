"""Build oracle models / states from a golden-vector file (test helper)."""
from __future__ import annotations

import numpy as np

from oracle import afqmc_oracle as orc


def model_from_golden(g) -> orc.Model:
    kind = str(g["kind"])
    h0 = float(g["h0"])
    h1, chol = g["h1"], g["chol"]
    mo_a, mo_b = g["mo_a"], g["mo_b"]
    rdm1 = np.stack([mo_a @ mo_a.T, mo_b @ mo_b.T])
    prop = orc.build_prop_ctx(h0, h1, chol, rdm1, float(g["dt"]))
    if kind == "uhf_u":
        meas = orc.build_uhf_meas_ctx(h1, chol, mo_a, mo_b)
        mo = (mo_a, mo_b)
    else:
        meas = orc.build_rhf_meas_ctx(h1, chol, mo_a)
        mo = mo_a
    return orc.Model(kind=kind, h0=h0, mo=mo, meas=meas, prop=prop)


def walkers_from_golden(g, prefix=""):
    if str(g["kind"]) == "rhf_r":
        return g[prefix + "walkers"]
    return (g[prefix + "walkers_u"], g[prefix + "walkers_d"])


def state_from_golden(g) -> orc.State:
    return orc.State(
        walkers=walkers_from_golden(g),
        weights=g["state_weights"].copy(),
        overlaps=g["overlap"].copy(),
        pop_control_ene_shift=float(g["state_shift"]),
        e_estimate=float(g["state_e_estimate"]),
        node_encounters=0,
    )


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
