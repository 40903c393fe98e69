"""Staged inputs and their HDF5 cache, streamed into HBM.

Mirrors the reference's staged-input containers and cache (trot/staging.py):
``HamInput`` / ``TrialInput`` / ``StagedInputs`` (:470-500), ``dump`` / ``load``
(:843-876) with the file layout of ``_dump_h5`` / ``_load_h5`` (:1353-1426):

    /            attrs: meta_json (JSON text)
    /ham         datasets h0 (scalar), h1 (N, N), chol (G, N, N), nelec (2,) int64,
                 [frozen (k,) int64]; attrs norb, chol_cut, [frozen], source_kind, basis
    /trial       attrs kind, [frozen], source_kind; [frozen dataset]
    /trial/data  one dataset per trial array (mo | mo_a, mo_b | ci1, ci2, ...)

Files written here are read by the reference's loader and the other way round (the
format layer is ``trot_gb300.h5file``; h5py is not needed).  ``load(path, device=...)``
puts the Hamiltonian and trial arrays straight into device memory: each contiguous
payload is read from the file into two pinned host buffers in turn (positioned reads
spread over eight reader threads), and each buffer is copied to HBM on a side stream
while the next one is read, so file reads and the host-to-device copies overlap and no
pageable host copy of the Cholesky tensor is made.

``make_job_inputs`` turns staged inputs into the objects a step needs, as the
reference's setup does (trot/setup.py:148-240 ``_make_trial_bundle``, :365-369 the
``System``; walker kind defaults to the Hamiltonian's basis, trot/setup.py:243-246).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass
from pathlib import Path
from typing import Any, Dict, Tuple, Union

import numpy as np
import torch

from . import h5file
from .core import HamChol, System

STAGE_FORMAT_VERSION = 1
_CHUNK_BYTES = 64 << 20


@dataclass(frozen=True, slots=True)
class HamInput:
    """Hamiltonian in the chosen orthonormal one-particle basis (trot/staging.py:470-483)."""

    h0: float
    h1: Any  # (norb, norb)
    chol: Any  # (nchol, norb, norb)
    nelec: Tuple[int, int]
    norb: int
    chol_cut: float
    frozen: Any  # int or int64 array
    source_kind: str  # "mf" or "cc"
    basis: str  # "restricted" or "generalized"


@dataclass(frozen=True, slots=True)
class TrialInput:
    """Trial inputs (trot/staging.py:486-493)."""

    kind: str
    data: Dict[str, Any]
    frozen: Any
    source_kind: str


@dataclass(frozen=True, slots=True)
class StagedInputs:
    ham: HamInput
    trial: TrialInput
    meta: Dict[str, Any]


# ------------------------------------------------------------------ frozen metadata
def _freeze_meta_value(frozen):
    """trot/staging.py:424-434."""
    if isinstance(frozen, np.ndarray):
        return [int(x) for x in np.asarray(frozen, dtype=np.int64).reshape(-1)]
    if isinstance(frozen, (int, np.integer)):
        return int(frozen)
    if frozen is None:
        return None
    raise TypeError(f"Unsupported frozen metadata type: {type(frozen)}")


def _freeze_from_meta_value(frozen):
    """trot/staging.py:437-446."""
    if frozen is None:
        return None
    if isinstance(frozen, (list, np.ndarray)):
        return np.asarray(frozen, dtype=np.int64)
    if isinstance(frozen, (int, np.integer)):
        return int(frozen)
    raise TypeError(f"Unsupported frozen metadata type: {type(frozen)}")


def _dump_frozen(group, frozen, attr_name: str = "frozen") -> None:
    """trot/staging.py:449-453: an index array is a dataset, a count is an attribute."""
    if isinstance(frozen, np.ndarray):
        group.create_dataset(attr_name, data=np.asarray(frozen, dtype=np.int64))
    else:
        group.attrs[attr_name] = int(frozen)


def _load_frozen(group, attr_name: str = "frozen"):
    """trot/staging.py:456-468."""
    if attr_name in group:
        ds = group[attr_name]
        if not isinstance(ds, h5file.Dataset):
            raise TypeError(f"Expected dataset '{attr_name}', got {type(ds)}")
        return np.asarray(ds[...], dtype=np.int64)
    v = group.attrs[attr_name]
    if isinstance(v, np.ndarray):
        return int(np.asarray(v).item())
    if isinstance(v, (int, np.integer)):
        return int(v)
    raise TypeError(f"Unsupported frozen attribute type: {type(v)}")


def _to_json_str(x) -> str:
    """trot/staging.py:1378-1385."""
    if isinstance(x, np.ndarray):
        x = x.item()
    if isinstance(x, (bytes, bytearray, np.bytes_)):
        return bytes(x).decode("utf-8")
    return str(x)


def _host(x) -> np.ndarray:
    return x.detach().cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)


# ------------------------------------------------------------------ dump / load
def dump(staged: StagedInputs, path: Union[str, Path]) -> None:
    """Write staged inputs to one HDF5 file (trot/staging.py:843-854, 1353-1375)."""
    p = Path(path).expanduser().resolve()
    p.parent.mkdir(parents=True, exist_ok=True)
    ham, tr = staged.ham, staged.trial
    with h5file.File(p, "w") as f:
        f.attrs["meta_json"] = json.dumps(staged.meta)
        g = f.create_group("ham")
        g.create_dataset("h0", data=np.array(ham.h0))
        g.create_dataset("h1", data=_host(ham.h1))
        g.create_dataset("chol", data=_host(ham.chol))
        g.create_dataset("nelec", data=np.array(ham.nelec, dtype=np.int64))
        g.attrs["norb"] = ham.norb
        g.attrs["chol_cut"] = ham.chol_cut
        _dump_frozen(g, ham.frozen)
        g.attrs["source_kind"] = ham.source_kind
        g.attrs["basis"] = ham.basis
        gt = f.create_group("trial")
        gt.attrs["kind"] = tr.kind
        _dump_frozen(gt, tr.frozen)
        gt.attrs["source_kind"] = tr.source_kind
        gd = gt.create_group("data")
        for k, v in tr.data.items():
            gd.create_dataset(k, data=_host(v))


_TORCH = {np.dtype("<f8"): torch.float64, np.dtype("<f4"): torch.float32, np.dtype("<i8"): torch.int64,
          np.dtype("<i4"): torch.int32, np.dtype("<c16"): torch.complex128, np.dtype("<c8"): torch.complex64}


_POOL = None
_PINNED: dict[int, list[torch.Tensor]] = {}
_READERS = 8


def _pool():
    global _POOL
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor
        _POOL = ThreadPoolExecutor(max_workers=_READERS, thread_name_prefix="trot-stage")
    return _POOL


def _pinned(chunk_bytes: int) -> list[torch.Tensor]:
    bufs = _PINNED.get(chunk_bytes)
    if bufs is None:
        bufs = [torch.empty(chunk_bytes, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        _PINNED[chunk_bytes] = bufs
    return bufs


def _pread_parallel(fd: int, view: memoryview, offset: int) -> None:
    """Fill ``view`` from the file at ``offset`` with positioned reads spread over the
    reader threads (each releases the interpreter lock while the kernel copies)."""
    n = len(view)
    piece = max(1 << 20, -(-n // _READERS))
    spans = [(a, min(n, a + piece)) for a in range(0, n, piece)]

    def one(span):
        a, b = span
        while a < b:
            got = os.preadv(fd, [view[a:b]], offset + a)
            if got <= 0:
                raise OSError(f"short read at {offset + a}")
            a += got

    for _ in _pool().map(one, spans):
        pass


def _to_device(ds: h5file.Dataset, device: torch.device, chunk_bytes: int) -> torch.Tensor:
    """One dataset into device memory through two pinned staging buffers: buffer k is
    refilled (parallel positioned reads) while the copy out of buffer 1-k runs."""
    tdt = _TORCH.get(ds.dtype if isinstance(ds.dtype, np.dtype) else None)
    ext = ds.extent()
    if tdt is None or ext is None or ext[1] <= chunk_bytes:
        host = np.asarray(ds[...])
        if tdt is None:
            raise TypeError(f"{ds.name}: dtype {ds.dtype} has no device counterpart")
        return torch.from_numpy(np.array(host, order="C")).to(device)  # a writable copy; keeps 0-d shapes
    off, n = ext
    out = torch.empty(ds.shape, dtype=tdt, device=device)
    flat = out.view(-1).view(torch.uint8)
    bufs = _pinned(chunk_bytes)
    views = [memoryview(b.numpy()) for b in bufs]
    done: list[torch.cuda.Event | None] = [None, None]
    stream = torch.cuda.Stream(device=device)
    fd = ds.file._rd.fh.fileno()
    pos, i = 0, 0
    try:
        while pos < n:
            m = min(chunk_bytes, n - pos)
            k = i & 1
            if done[k] is not None:
                done[k].synchronize()  # the copy out of this buffer has finished
            _pread_parallel(fd, views[k][:m], off + pos)
            with torch.cuda.stream(stream):
                flat[pos:pos + m].copy_(bufs[k][:m], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(stream)
            done[k] = ev
            pos += m
            i += 1
    finally:
        stream.synchronize()  # no copy may still read a buffer the next load refills
    torch.cuda.current_stream(device).wait_stream(stream)
    return out


def load(path: Union[str, Path], device: Union[str, torch.device, None] = None,
         chunk_bytes: int = _CHUNK_BYTES) -> StagedInputs:
    """Read staged inputs written by ``dump`` or by the reference's ``dump``
    (trot/staging.py:857-876, 1388-1423).  With ``device`` the arrays h1, chol and the
    trial data arrive as device tensors; otherwise they are numpy arrays."""
    p = Path(path).expanduser().resolve()
    dev = torch.device(device) if device is not None else None
    if dev is not None and dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())

    def arr(ds):
        if dev is None or dev.type != "cuda":
            return np.asarray(ds[...])
        return _to_device(ds, dev, chunk_bytes)

    with h5file.File(p, "r") as f:
        meta = json.loads(_to_json_str(f.attrs["meta_json"]))
        if "frozen" in meta:
            meta["frozen"] = _freeze_from_meta_value(meta["frozen"])
        g = f["ham"]
        nelec = np.asarray(g["nelec"][...])
        ham = HamInput(h0=float(np.asarray(g["h0"][...]).item()), h1=arr(g["h1"]), chol=arr(g["chol"]),
                       nelec=(int(nelec[0]), int(nelec[1])), norb=int(g.attrs["norb"]),
                       chol_cut=float(g.attrs["chol_cut"]), frozen=_load_frozen(g),
                       source_kind=str(g.attrs["source_kind"]), basis=str(g.attrs["basis"]))
        gt = f["trial"]
        gd = gt["data"]
        data = {k: arr(gd[k]) for k in gd.keys()}
        trial = TrialInput(kind=str(gt.attrs["kind"]), data=data, frozen=_load_frozen(gt),
                           source_kind=str(gt.attrs["source_kind"]))
    return StagedInputs(ham=ham, trial=trial, meta=meta)


# ------------------------------------------------------------------ staged -> step inputs
def make_system(staged: StagedInputs, walker_kind: str | None = None) -> System:
    """trot/setup.py:243-246, 365-369."""
    ham = staged.ham
    return System(norb=int(ham.norb), nelec=tuple(ham.nelec), walker_kind=walker_kind or ham.basis)


def make_ham_data(staged: StagedInputs) -> HamChol:
    ham = staged.ham
    return HamChol(h0=ham.h0, h1=ham.h1, chol=ham.chol, basis=ham.basis)


def make_trial_bundle(sys: System, staged: StagedInputs, mixed_precision: bool = False):
    """(trial_data, trial_ops, meas_ops) for the trial kinds this package covers:
    rhf, rohf / uhf and cisd (trot/setup.py:148-240)."""
    kind = staged.trial.kind.lower()
    data = staged.trial.data
    if kind == "rhf":
        from .meas import make_rhf_meas_ops
        from .trial import make_rhf_trial_data, make_rhf_trial_ops
        return (make_rhf_trial_data(data, sys), make_rhf_trial_ops(sys=sys),
                make_rhf_meas_ops(sys=sys, mixed_precision=mixed_precision))
    if kind in ("rohf", "uhf"):
        from .meas import make_uhf_meas_ops
        from .trial import make_uhf_trial_data, make_uhf_trial_ops
        return (make_uhf_trial_data(data, sys), make_uhf_trial_ops(sys=sys),
                make_uhf_meas_ops(sys=sys, mixed_precision=mixed_precision))
    if kind == "cisd":
        from .cisd import make_cisd_meas_ops, make_cisd_trial_data, make_cisd_trial_ops
        return (make_cisd_trial_data(data, sys), make_cisd_trial_ops(sys=sys),
                make_cisd_meas_ops(sys=sys, mixed_precision=mixed_precision))
    raise NotImplementedError(f"trial kind {staged.trial.kind!r} is not covered by the CUDA path")


def make_job_inputs(staged: StagedInputs, walker_kind: str | None = None, mixed_precision: bool = False):
    """(sys, ham_data, trial_data, trial_ops, meas_ops) from staged inputs."""
    sys = make_system(staged, walker_kind)
    return (sys, make_ham_data(staged)) + make_trial_bundle(sys, staged, mixed_precision)
