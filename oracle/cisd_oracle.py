"""CPU oracle for the CISD-trial measurements.

TEST INFRASTRUCTURE ONLY (same rules as ``afqmc_oracle``).  numpy complex128
restatement, batched over walkers, of

* ``_overlap_r_with_doubles`` / ``overlap_r_high`` (trot/trial/cisd.py:99-186),
* ``_force_bias_common_terms_high_realimag`` + ``force_bias_kernel_rw_rh_high``
  (trot/meas/cisd.py:455-479, 548-572),
* ``energy_kernel_rw_rh`` in "high" memory mode with float64 contractions
  (``testing=True``) (trot/meas/cisd.py:608-769),

for restricted walkers in the trial's MO basis: the reference determinant
occupies orbitals [0, nocc_full); the CI amplitudes cover the active block
occ [nocc_t_core, nocc_full) x vir [nocc_full, nocc_full + nvir).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class CisdTrial:
    """``CisdTrial`` (trot/trial/cisd.py:14-88)."""

    ci1: np.ndarray  # (n_act, v_act)
    ci2: np.ndarray  # (n_act, v_act, n_act, v_act), (i, a, j, b)
    nocc_t_core: int = 0
    nvir_t_outer: int = 0

    @property
    def nocc(self):
        return self.ci1.shape[0]

    @property
    def nvir(self):
        return self.ci1.shape[1]

    @property
    def nocc_full(self):
        return self.nocc_t_core + self.nocc

    @property
    def norb(self):
        return self.nocc_full + self.nvir + self.nvir_t_outer

    @property
    def occ(self):
        return slice(self.nocc_t_core, self.nocc_full)

    @property
    def vir(self):
        return slice(self.nocc_full, self.nocc_full + self.nvir)


def green(w, nocc_full):
    """``_greens_restricted`` (trot/meas/cisd.py:19-21): solve(wocc^T, w^T), (W, nocc_full, N)."""
    wocc = w[:, :nocc_full, :]
    return np.linalg.solve(np.swapaxes(wocc, -1, -2), np.swapaxes(w, -1, -2))


def overlap(w, tr: CisdTrial):
    """``overlap_r_high`` (trot/trial/cisd.py:148-174):
    (1 + 2 ci1.x + 2 sum ci2_iajb x_ia x_jb - sum ci2_iajb x_ib x_ja) det(w_occ)^2."""
    g = green(w, tr.nocc_full)
    det0 = np.linalg.det(w[:, : tr.nocc_full, :])
    x = g[:, tr.occ, tr.vir]
    o1 = np.einsum("ia,zia->z", tr.ci1, x)
    direct = np.einsum("iajb,zia,zjb->z", tr.ci2, x, x, optimize=True)
    exch = np.einsum("iajb,zib,zja->z", tr.ci2, x, x, optimize=True)
    return (1.0 + 2.0 * o1 + 2.0 * direct - exch) * det0 * det0


def _blocks(g, tr: CisdTrial):
    """``_active_green_blocks`` (trot/meas/cisd.py:24-44)."""
    W = g.shape[0]
    g_act = g[:, tr.occ, :]
    g_occ = g[:, tr.occ, tr.vir]
    gp = np.zeros((W, tr.norb, tr.nvir), dtype=g.dtype)
    gp[:, : tr.nocc_full, :] = g[:, :, tr.vir]
    gp[:, tr.vir, :] = -np.eye(tr.nvir)
    return g_act, g_occ, gp


def _ci2g(ci2, g_occ):
    c = np.einsum("ptqu,bpt->bqu", ci2, g_occ, optimize=True)
    e = np.einsum("ptqu,bpu->bqt", ci2, g_occ, optimize=True)
    return c, e


def force_bias(w, tr: CisdTrial, chol):
    """``force_bias_kernel_rw_rh_high`` (trot/meas/cisd.py:548-572)."""
    g = green(w, tr.nocc_full)
    g_act, g_occ, gp = _blocks(g, tr)
    rot_chol = chol[:, : tr.nocc_full, :]
    lg = np.einsum("gpj,bpj->bg", rot_chol, g, optimize=True)
    ci1g = np.einsum("pt,bpt->b", tr.ci1, g_occ)
    ci1gp = np.einsum("pt,bit->bpi", tr.ci1, gp)
    gci1gp = np.einsum("bpj,bpi->bij", g_act, ci1gp)
    c, e = _ci2g(tr.ci2, g_occ)
    cg_c = (gp @ np.swapaxes(c, -1, -2)) @ g_act
    cg_e = (gp @ np.swapaxes(e, -1, -2)) @ g_act
    cisd_green = -4.0 * cg_c + 2.0 * cg_e
    ci2g = 4.0 * c - 2.0 * e
    gci2g = np.einsum("bqu,bqu->b", ci2g, g_occ)
    ov = 1.0 + 2.0 * ci1g + 0.5 * gci2g
    fb_corr = np.einsum("gij,bij->bg", chol, cisd_green - 2.0 * gci1gp, optimize=True)
    fb = 2.0 * lg + 4.0 * ci1g[:, None] * lg + lg * gci2g[:, None] + fb_corr
    return fb / ov[:, None]



def meas_lci1(chol, ci1, vir):
    """lci1[g][i][p] = sum_t chol[g][i][vir_t] ci1[p][t] (trot/runtime_layout.py:272-281;
    trot/meas/cisd.py:92-110), (G, N, nocc)."""
    return np.einsum("git,pt->gip", np.asarray(chol)[:, :, vir], ci1, optimize=True)


def energy(w, tr: CisdTrial, h0, h1, chol):
    """``energy_kernel_rw_rh`` (trot/meas/cisd.py:608-769), "high" mode, float64."""
    ci1, ci2 = tr.ci1, tr.ci2
    g = green(w, tr.nocc_full)
    g_act, g_occ, gp = _blocks(g, tr)
    rot_chol = chol[:, : tr.nocc_full, :]
    T = lambda x: np.swapaxes(x, -1, -2)

    hg = np.einsum("pj,bpj->b", h1[: tr.nocc_full, :], g)
    e1_0 = 2.0 * hg
    ci1g = np.einsum("pt,bpt->b", ci1, g_occ)
    e1_1_1 = 4.0 * ci1g * hg
    gpci1 = gp @ ci1.T
    ci1_green = gpci1 @ g_act
    e1_1_2 = -2.0 * np.einsum("ij,bij->b", h1, ci1_green)
    c, e = _ci2g(ci2, g_occ)
    ci2_green = 2.0 * ((gp @ T(c)) @ g_act) - 1.0 * ((gp @ T(e)) @ g_act)
    ci2g = 2.0 * c - 1.0 * e
    gci2g = np.einsum("bqu,bqu->b", ci2g, g_occ)
    e1_2 = 2.0 * hg * gci2g - 2.0 * np.einsum("ij,bij->b", h1, ci2_green)
    e1 = e1_0 + e1_1_1 + e1_1_2 + e1_2

    lg = np.einsum("gpj,bpj->bg", rot_chol, g, optimize=True)
    e2_0_1 = 2.0 * np.sum(lg * lg, axis=1)
    lg1 = np.einsum("gpj,bqj->bgpq", rot_chol, g, optimize=True)
    e2_0_2 = -np.einsum("bgpq,bgqp->b", lg1, lg1, optimize=True)
    e2_0 = e2_0_1 + e2_0_2

    e2_1_1 = 2.0 * e2_0 * ci1g
    lci1g = np.einsum("gij,bij->bg", chol, ci1_green, optimize=True)
    e2_1_2 = -2.0 * np.sum(lci1g * lg, axis=1)
    ci1g1 = np.einsum("pt,bqt->bpq", ci1, g[:, :, tr.vir])  # (W, nocc_act, nocc_full)
    e2_1_3_1 = np.einsum("bgpq,bgqa,bap->b", lg1, lg1[:, :, :, tr.occ], ci1g1, optimize=True)
    lci1 = meas_lci1(chol, ci1, tr.vir)  # meas ctx lci1 (G, N, n_act)
    lci1g_mat = np.einsum("gia,bqi->bgaq", lci1, g, optimize=True)
    e2_1_3_2 = -np.einsum("bgaq,bgqa->b", lci1g_mat, lg1[:, :, :, tr.occ], optimize=True)
    e2_1 = e2_1_1 + 2.0 * (e2_1_2 + e2_1_3_1 + e2_1_3_2)

    e2_2_1 = e2_0 * gci2g
    lci2g = np.einsum("gij,bij->bg", chol, ci2_green, optimize=True)
    e2_2_2_1 = -np.sum(lci2g * lg, axis=1)
    lci2_green = np.einsum("gpi,bji->bgpj", rot_chol, ci2_green, optimize=True)
    gl = np.einsum("bpj,gji->bgpi", g, chol, optimize=True)
    e2_2_2_2 = 0.5 * np.einsum("bgpi,bgpi->b", gl, lci2_green, optimize=True)
    glgp = np.einsum("bgpi,bit->bgpt", gl, gp, optimize=True)[:, :, tr.occ, :]
    l2_1 = np.einsum("bgpt,bgqu,ptqu->b", glgp, glgp, ci2, optimize=True)
    l2_2 = np.einsum("bgpu,bgqt,ptqu->b", glgp, glgp, ci2, optimize=True)
    e2_2_3 = 2.0 * l2_1 - l2_2
    e2_2 = e2_2_1 + 4.0 * (e2_2_2_1 + e2_2_2_2) + e2_2_3
    e2 = e2_0 + e2_1 + e2_2
    ov = 1.0 + 2.0 * ci1g + gci2g
    return (e1 + e2) / ov + h0


def rdm1(w, tr: CisdTrial):
    """``rdm1_kernel_rw`` (trot/meas/cisd.py:772-820), one spin: G0 - (ci1_green + ci2_green) / ov,
    G0[:, :nocc_full] = G^T."""
    g = green(w, tr.nocc_full)
    g_act, g_occ, gp = _blocks(g, tr)
    ci1g = np.einsum("pt,bpt->b", tr.ci1, g_occ)
    ci1_green = (gp @ tr.ci1.T) @ g_act
    c, e = _ci2g(tr.ci2, g_occ)
    ci2_green = 2.0 * ((gp @ np.swapaxes(c, -1, -2)) @ g_act) - (gp @ np.swapaxes(e, -1, -2)) @ g_act
    gci2g = np.einsum("bqu,bqu->b", 2.0 * c - e, g_occ)
    ov = 1.0 + 2.0 * ci1g + gci2g
    g0 = np.zeros((w.shape[0], tr.norb, tr.norb), dtype=g.dtype)
    g0[:, :, : tr.nocc_full] = np.swapaxes(g, -1, -2)
    return g0 - (ci1_green + ci2_green) / ov[:, None, None]


@dataclass(frozen=True)
class CisdModel:
    """CISD trial with restricted walkers in the shape ``afqmc_oracle.afqmc_step`` /
    ``afqmc_oracle.block`` expect (overlap, force_bias, energy, trotter, walker_kind):
    trot/prop/afqmc.py:79-144 with the CISD meas ops."""

    trial: CisdTrial
    h0: float
    h1: np.ndarray
    chol: np.ndarray
    prop: object  # afqmc_oracle.PropCtx

    walker_kind = "restricted"

    def overlap(self, w):
        return overlap(w, self.trial)

    def force_bias(self, w):
        return force_bias(w, self.trial, self.chol)

    def energy(self, w):
        return energy(w, self.trial, self.h0, self.h1, self.chol)

    def trotter(self, w, xs, n_terms):
        from oracle import afqmc_oracle

        return afqmc_oracle.apply_trotter_r(w, xs, self.prop, n_terms)
