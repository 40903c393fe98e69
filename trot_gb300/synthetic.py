"""Seeded synthetic Cholesky Hamiltonians and mean-field trials.

This is the input generator for the benchmark workloads and the tests (there is
no public molecule set for this path and PySCF is not a dependency):

* ``h1``: symmetric, diagonal U(-2, 0), off-diagonal N(0, 0.05);
* ``L_g``: symmetric, entries N(0, 1) * exp(-g / decay) * 0.3, so
  (pq|rs) = sum_g L_g,pq L_g,rs is positive semi-definite by construction;
* trial: RHF or UHF orbitals after a fixed number of SCF iterations on h1 + L.

All draws come from ``numpy.random.default_rng(seed)`` in a fixed order, so a
(seed, sizes) pair names one Hamiltonian on every machine.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class SyntheticSystem:
    h0: float
    h1: np.ndarray  # (N, N)
    chol: np.ndarray  # (G, N, N)
    mo_a: np.ndarray  # (N, na)
    mo_b: np.ndarray  # (N, nb)

    @property
    def norb(self) -> int:
        return self.h1.shape[0]

    @property
    def nchol(self) -> int:
        return self.chol.shape[0]

    @property
    def nelec(self) -> tuple[int, int]:
        return self.mo_a.shape[1], self.mo_b.shape[1]

    def rdm1(self) -> np.ndarray:
        """Trial one-body density, spin blocks (2, N, N)."""
        return np.stack([self.mo_a @ self.mo_a.T, self.mo_b @ self.mo_b.T])


def hamiltonian(norb: int, nchol: int, decay: float = 30.0, seed: int = 0, h0: float = 0.0):
    """Return (h0, h1, chol) for the seeded recipe."""
    rng = np.random.default_rng(seed)
    h1 = rng.normal(0.0, 0.05, (norb, norb))
    h1 = np.triu(h1, 1)
    h1 = h1 + h1.T
    h1[np.diag_indices(norb)] = rng.uniform(-2.0, 0.0, norb)
    chol = rng.normal(0.0, 1.0, (nchol, norb, norb))
    chol = 0.5 * (chol + chol.transpose(0, 2, 1))
    chol *= (np.exp(-np.arange(nchol) / decay) * 0.3)[:, None, None]
    return float(h0), h1, np.ascontiguousarray(chol)


def _coulomb(chol, dm):
    G = chol.shape[0]
    return np.tensordot(chol.reshape(G, -1) @ dm.T.reshape(-1), chol, axes=1)


def _exchange(chol, c):
    """sum_g L_g (c c^T) L_g for occupied orbitals c (N, n): X X^T with X_g = L_g c,
    one (N, G n) x (G n, N) product."""
    G, N, _ = chol.shape
    x = (chol.reshape(G * N, N) @ c).reshape(G, N, c.shape[1]).transpose(1, 0, 2).reshape(N, G * c.shape[1])
    return x @ x.T


def scf(h1, chol, na: int, nb: int, iters: int = 30):
    """Unrestricted SCF with plain Roothaan steps from the core guess.

    With na == nb the alpha and beta orbitals stay identical (RHF)."""
    _, c = np.linalg.eigh(h1)
    ca, cb = c[:, :na], c[:, :nb]
    for _ in range(iters):
        da, db = ca @ ca.T, cb @ cb.T
        j = _coulomb(chol, da + db)
        fa = h1 + j - _exchange(chol, ca)
        fb = h1 + j - _exchange(chol, cb)
        ca = np.linalg.eigh(fa)[1][:, :na]
        cb = np.linalg.eigh(fb)[1][:, :nb]
    return np.ascontiguousarray(ca), np.ascontiguousarray(cb)


def scf_rhf_full(h1, chol, n: int, iters: int = 30):
    """RHF SCF as ``scf`` with na == nb == n; returns all MOs (N, N) and orbital
    energies of the final Fock matrix."""
    _, c = np.linalg.eigh(h1)
    co = c[:, :n]
    for _ in range(iters):
        d = co @ co.T
        f = h1 + 2.0 * _coulomb(chol, d) - _exchange(chol, co)
        eps, c = np.linalg.eigh(f)
        co = c[:, :n]
    return np.ascontiguousarray(c), eps


@dataclass(frozen=True)
class CisdSystem:
    """Hamiltonian in the RHF MO basis (reference determinant = first nocc MOs)
    plus CISD amplitudes in trot's (i, a, j, b) layout."""

    h0: float
    h1: np.ndarray  # (N, N) MO basis
    chol: np.ndarray  # (G, N, N) MO basis
    ci1: np.ndarray  # (n, v)
    ci2: np.ndarray  # (n, v, n, v), symmetric under (i, a) <-> (j, b)

    @property
    def nocc(self) -> int:
        return self.ci1.shape[0]


def make_cisd_system(norb, nocc, nchol, decay=30.0, seed=0, h0=0.0, c1_sigma=0.02, c2_norm=0.2, scf_iters=30):
    """CISD recipe: c1 ~ N(0, c1_sigma); c2_ijab = N(0, 1) / (e_a + e_b - e_i - e_j)
    with e the RHF orbital energies, mapped to ci2[i, a, j, b] = c2_ijab,
    symmetrised under (i, a) <-> (j, b) (the spatial-orbital convention of
    trot/trial/cisd.py) and scaled to ||ci2|| = c2_norm."""
    h0, h1, chol = hamiltonian(norb, nchol, decay, seed, h0)
    c, eps = scf_rhf_full(h1, chol, nocc, scf_iters)
    h1_mo = c.T @ h1 @ c
    chol_mo = np.einsum("pi,gpq,qj->gij", c, chol, c, optimize=True)
    nv = norb - nocc
    rng = np.random.default_rng(seed + 17)
    ci1 = rng.normal(0.0, c1_sigma, (nocc, nv))
    eo, ev = eps[:nocc], eps[nocc:]
    denom = ev[None, None, :, None] + ev[None, None, None, :] - eo[:, None, None, None] - eo[None, :, None, None]
    c2 = rng.normal(size=(nocc, nocc, nv, nv)) / denom
    ci2 = c2.transpose(0, 2, 1, 3)
    ci2 = 0.5 * (ci2 + ci2.transpose(2, 3, 0, 1))
    ci2 *= c2_norm / np.linalg.norm(ci2)
    return CisdSystem(h0=float(h0), h1=np.ascontiguousarray(h1_mo), chol=np.ascontiguousarray(chol_mo),
                      ci1=np.ascontiguousarray(ci1), ci2=np.ascontiguousarray(ci2))


def make_system(norb, nelec, nchol, decay=30.0, seed=0, h0=0.0, scf_iters=30) -> SyntheticSystem:
    h0, h1, chol = hamiltonian(norb, nchol, decay, seed, h0)
    ca, cb = scf(h1, chol, nelec[0], nelec[1], scf_iters)
    return SyntheticSystem(h0=h0, h1=h1, chol=chol, mo_a=ca, mo_b=cb)


def perturbed_walkers(mo: np.ndarray, n_walkers: int, scale: float = 0.1, seed: int = 1) -> np.ndarray:
    """Walkers near the trial: mo + scale * complex Gaussian noise, (W, N, n) c128."""
    rng = np.random.default_rng(seed)
    shape = (n_walkers,) + mo.shape
    noise = rng.normal(size=shape) + 1.0j * rng.normal(size=shape)
    return np.ascontiguousarray(mo[None].astype(np.complex128) + scale * noise)


def fields(n_walkers: int, nchol: int, n_steps: int, seed: int = 2) -> np.ndarray:
    """Seeded N(0, 1) auxiliary fields, (n_steps, W, G) float64."""
    rng = np.random.default_rng(seed)
    return rng.standard_normal((n_steps, n_walkers, nchol))


# Benchmark / test workloads (sizes as quoted for the reference path).
CONFIGS = {
    "cfg1_rhf_n24": dict(norb=24, nelec=(5, 5), nchol=120, decay=30.0, n_walkers=64,
                         dt=0.005, n_steps=50, qr_every=5, kind="rhf_r"),
    "cfg2_uhf_n120": dict(norb=120, nelec=(12, 10), nchol=600, decay=150.0, n_walkers=1024,
                          dt=0.005, n_steps=200, qr_every=10, kind="uhf_u"),
    # the cfg2 system with fewer walkers: small case for profiler captures
    "cfg2_uhf_n120_w256": dict(norb=120, nelec=(12, 10), nchol=600, decay=150.0, n_walkers=256,
                               dt=0.005, n_steps=200, qr_every=10, kind="uhf_u"),
    "cfg4_cisd_n60": dict(norb=60, nelec=(8, 8), nchol=300, decay=30.0, n_walkers=256,
                          dt=0.005, n_steps=100, qr_every=10, kind="cisd"),
    "cfg3_rhf_n80": dict(norb=80, nelec=(10, 10), nchol=400, decay=30.0, n_walkers=512,
                         dt=0.01, n_steps=200, qr_every=20, kind="rhf_r"),
}
