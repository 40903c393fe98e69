"""Generate the staged-input cache fixtures with the reference's own dump/load.

The reference's trot/staging.py (``dump`` / ``load`` :843-876, ``_dump_h5`` /
``_load_h5`` :1353-1426) runs unmodified; ``h5py`` is replaced by trot_gb300.h5file
(the same File / Group / Dataset / attrs surface) and jax by ``_jaxshim``.  For each
case this writes

    staged_<case>.h5   the file the reference's ``dump`` wrote
    staged_<case>.npz  the inputs it was given (arrays, scalars, JSON metadata)

and checks, here, that the reference's ``load`` reads back a file written by
``trot_gb300.staging.dump`` with the same values.  The tests read only the fixtures.

    python tests/golden/make_staged_golden.py /path/to/trot
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import _jaxshim  # noqa: E402

_jaxshim.install()
from trot_gb300 import h5file, staging  # noqa: E402

sys.modules["h5py"] = h5file
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("TROT_REFERENCE", "")
if not REF or not os.path.isdir(os.path.join(REF, "trot")):
    sys.exit("usage: make_staged_golden.py /path/to/trot  (or set TROT_REFERENCE)")
sys.path.insert(0, REF)

import trot.staging as ref  # noqa: E402


def cases():
    rng = np.random.default_rng(11)

    def sym(n):
        a = rng.normal(size=(n, n))
        return a + a.T

    def chol(g, n):
        c = rng.normal(size=(g, n, n))
        return c + c.transpose(0, 2, 1)

    meta = {"format_version": 1, "timestamp_unix": 1.7e9, "source_kind": "mf", "frozen": 0, "chol_cut": 1e-5,
            "mol": {"nao": 8, "nelectron": 6, "spin": 0, "charge": 0, "basis": "sto-3g"}}
    n, g = 8, 12
    mo = np.linalg.qr(rng.normal(size=(n, n)))[0]
    yield "rhf", dict(h0=-1.25, h1=sym(n), chol=chol(g, n), nelec=(3, 3), norb=n, chol_cut=1e-5, frozen=0,
                      source_kind="mf", basis="restricted"), \
        dict(kind="rhf", data={"mo": mo}, frozen=0, source_kind="mf"), meta
    n, g = 7, 10
    meta_u = dict(meta, frozen=[0, 3], source_kind="cc", mol=dict(meta["mol"], spin=1, nelectron=5))
    fz = np.array([0, 3], np.int64)
    yield "uhf", dict(h0=0.5, h1=sym(n), chol=chol(g, n), nelec=(3, 2), norb=n, chol_cut=2e-6, frozen=fz,
                      source_kind="cc", basis="restricted"), \
        dict(kind="uhf", data={"mo_a": np.linalg.qr(rng.normal(size=(n, n)))[0],
                               "mo_b": np.linalg.qr(rng.normal(size=(n, n)))[0]},
             frozen=fz, source_kind="cc"), meta_u
    n, g, no = 8, 9, 3
    nv = n - no
    c2 = rng.normal(size=(no, nv, no, nv)) * 0.01
    yield "cisd", dict(h0=2.0, h1=sym(n), chol=chol(g, n), nelec=(no, no), norb=n, chol_cut=1e-4, frozen=1,
                       source_kind="cc", basis="restricted"), \
        dict(kind="cisd", data={"ci1": rng.normal(size=(no, nv)) * 0.02, "ci2": c2 + c2.transpose(2, 3, 0, 1),
                                "nocc_t_core": np.array(0, np.int64), "nvir_t_outer": np.array(0, np.int64)},
             frozen=1, source_kind="cc"), dict(meta, frozen=1, source_kind="cc")


def flat(ham, trial, meta):
    out = {"meta_json": np.array(json.dumps(meta))}
    for k, v in ham.items():
        out["ham." + k] = np.asarray(v)
    for k, v in trial.items():
        if k != "data":
            out["trial." + k] = np.asarray(v)
    for k, v in trial["data"].items():
        out["data." + k] = np.asarray(v)
    return out


def same(a, b) -> bool:
    if isinstance(a, dict):
        return a.keys() == b.keys() and all(same(a[k], b[k]) for k in a)
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a, b)


def main():
    for name, ham, trial, meta in cases():
        rs = ref.StagedInputs(ham=ref.HamInput(**ham), trial=ref.TrialInput(**trial), meta=meta)
        path = os.path.join(HERE, f"staged_{name}.h5")
        ref.dump(rs, path)
        np.savez(os.path.join(HERE, f"staged_{name}.npz"), **flat(ham, trial, meta))
        # the reference's loader on a file written by this package
        ours = staging.StagedInputs(ham=staging.HamInput(**ham), trial=staging.TrialInput(**trial), meta=meta)
        with tempfile.TemporaryDirectory() as td:
            p2 = os.path.join(td, "ours.h5")
            staging.dump(ours, p2)
            back = ref.load(p2)
        for k, v in ham.items():
            got = getattr(back.ham, k)
            assert same(got, v) or (k == "nelec" and tuple(got) == tuple(v)), (name, k)
        for k in ("kind", "frozen", "source_kind"):
            assert same(getattr(back.trial, k), trial[k]), (name, k)
        assert same(back.trial.data, trial["data"]), name
        want = dict(meta)
        want["frozen"] = ref._freeze_from_meta_value(meta["frozen"])
        assert json.dumps(back.meta, default=lambda a: a.tolist()) == json.dumps(want, default=lambda a: a.tolist())
        print(f"staged_{name}: reference dump written, reference load of this package's file agrees")


if __name__ == "__main__":
    main()
