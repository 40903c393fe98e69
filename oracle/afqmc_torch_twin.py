"""Test infrastructure: a torch complex128 restatement of the phaseless step,
the local energy and the block tail (RHF trial with restricted or unrestricted
walkers, UHF trial with unrestricted walkers),
differentiated by torch's autograd on the CPU.  It stands in for "jax.grad of
the reference" (jax is not available here) as the gradient oracle of the
hand-written adjoint in trot_gb300.adjoint; its forward is checked against the
numpy oracle (oracle/afqmc_oracle.py, itself pinned to the reference's golden
vectors).

Formulas (same citations as the numpy oracle):
* propagation context: trot/prop/chol_afqmc_ops.py:74-127 (exp(-dt/2 h1_eff)
  by torch.linalg.matrix_exp);
* step: trot/prop/afqmc.py:91-144;
* QR with phase-fixed R: trot/walkers.py:137-179;
* local energy: trot/meas/rhf.py:21-60,128-172, trot/meas/uhf.py:205-231; overlaps
  trot/trial/rhf.py:45-54, trot/trial/uhf.py:54-58;
* block tail without SR: trot/prop/blocks.py:228-263.
The objective J = sum_b sum_w wt E~ / sum_b sum_w wt matches trot_gb300.adjoint.
"""
from __future__ import annotations

import math

import torch


def prop_consts(h0, h1, chol, rdm1, dt):
    """(mf_im (G,), h0_prop, exp_h1_half) with h1 a (possibly grad-carrying) tensor."""
    dm = rdm1[0] + rdm1[1] if rdm1.dim() == 3 else rdm1
    t = torch.einsum("gij,ji->g", chol, dm)
    h0_prop = -h0 + 0.5 * torch.sum(t * t)
    v0 = 0.5 * torch.einsum("gik,gkj->ij", chol, chol)
    v1 = torch.einsum("g,gik->ik", -t, chol)
    h1_eff = h1 - v0 - v1
    return t, h0_prop, torch.linalg.matrix_exp(-0.5 * dt * h1_eff)


def half_green(w, mo):
    m = torch.einsum("pi,bpj->bij", mo.to(w.dtype), w)
    return torch.linalg.solve(m.transpose(-1, -2), w.transpose(-1, -2))


def overlap(w, mo):
    d = torch.linalg.det(torch.einsum("pi,bpj->bij", mo.to(w.dtype), w))
    return d * d


def force_bias(w, mo, rot_chol):
    g = half_green(w, mo)
    G = rot_chol.shape[0]
    return 2.0 * g.reshape(g.shape[0], -1) @ rot_chol.reshape(G, -1).T.to(w.dtype)


def local_energy(w, mo, h0, rot_h1, rot_chol):
    g = half_green(w, mo)
    e1 = 2.0 * torch.einsum("bij,ij->b", g, rot_h1.to(w.dtype))
    f = torch.matmul(rot_chol.to(w.dtype)[None], g.transpose(-1, -2)[:, None])
    c = torch.einsum("bgii->bg", f)
    exc = torch.sum(f * f.transpose(-1, -2), dim=(1, 2, 3))
    return h0 + e1 + 2.0 * torch.sum(c * c, dim=1) - exc


def qr_phase_fixed(w):
    q, r = torch.linalg.qr(w)
    d = torch.diagonal(r, dim1=-2, dim2=-1)
    ph = torch.where(d.abs() > 0, d / d.abs(), torch.ones_like(d))
    return q * ph.conj()[:, None, :]


def _overlap_k(w, mo, kind):
    if kind == "rhf_r":
        return overlap(w, mo)
    ma, mb = mo if kind == "uhf_u" else (mo, mo)
    da = torch.linalg.det(torch.einsum("pi,bpj->bij", ma.to(w[0].dtype), w[0]))
    db = torch.linalg.det(torch.einsum("pi,bpj->bij", mb.to(w[1].dtype), w[1]))
    return da * db


def _force_bias_k(w, mo, rot_chol, kind):
    if kind == "rhf_r":
        return force_bias(w, mo, rot_chol)
    ma, mb = mo if kind == "uhf_u" else (mo, mo)
    ra, rb = rot_chol if kind == "uhf_u" else (rot_chol, rot_chol)
    G = ra.shape[0]
    ga, gb = half_green(w[0], ma), half_green(w[1], mb)
    return (ga.reshape(ga.shape[0], -1) @ ra.reshape(G, -1).T.to(ga.dtype)
            + gb.reshape(gb.shape[0], -1) @ rb.reshape(G, -1).T.to(gb.dtype))


def _coul_exch(g, rot_chol):
    f = torch.matmul(rot_chol.to(g.dtype)[None], g.transpose(-1, -2)[:, None])
    return torch.einsum("bgii->bg", f), torch.sum(f * f.transpose(-1, -2), dim=(1, 2, 3))


def _energy_k(w, mo, h0, rot_h1, rot_chol, kind):
    """trot/meas/rhf.py:128-172, trot/meas/uhf.py:205-231 (rot_h1 / rot_chol per spin for uhf_u)."""
    if kind == "rhf_r":
        return local_energy(w, mo, h0, rot_h1, rot_chol)
    ma, mb = mo if kind == "uhf_u" else (mo, mo)
    ha, hb = rot_h1 if kind == "uhf_u" else (rot_h1, rot_h1)
    ra, rb = rot_chol if kind == "uhf_u" else (rot_chol, rot_chol)
    ga, gb = half_green(w[0], ma), half_green(w[1], mb)
    e1 = torch.einsum("bij,ij->b", ga, ha.to(ga.dtype)) + torch.einsum("bij,ij->b", gb, hb.to(gb.dtype))
    ca, xa = _coul_exch(ga, ra)
    cb, xb = _coul_exch(gb, rb)
    e2 = (torch.sum(ca * ca, 1) + torch.sum(cb * cb, 1) + 2.0 * torch.sum(ca * cb, 1) - xa - xb) / 2.0
    return h0 + e1 + e2


def _trotter(w, V, eh, s, n_terms):
    ehc = eh.to(w.dtype)
    w1 = ehc @ w
    term, out = w1, w1
    for k in range(1, n_terms + 1):
        term = (1j * s / k) * (V @ term)
        out = out + term
    return ehc @ out


def step(w, wt, ov, es, ee, x, *, mo, rot_chol, chol, mf_im, h0_prop, eh, dt, n_terms, w_floor=1e-3, w_cap=100.0,
         damping=0.1, kind="rhf_r"):
    """trot/prop/afqmc.py:91-144; w a tensor (rhf_r) or a (wa, wb) tuple; mo / rot_chol
    pairs for uhf_u."""
    s = math.sqrt(dt)
    fb = _force_bias_k(w, mo, rot_chol, kind)
    mf = 1j * mf_im.to(fb.dtype)
    fs = -s * (1j * fb - mf)
    xs = x.to(fb.dtype) - fs
    shift_term = torch.sum(xs * mf, dim=1)
    fb_term = torch.sum(x * fs - 0.5 * fs * fs, dim=1)
    G, N = chol.shape[0], chol.shape[1]
    V = (xs @ chol.reshape(G, N * N).to(xs.dtype)).reshape(-1, N, N)
    wn = _trotter(w, V, eh, s, n_terms) if kind == "rhf_r" else tuple(_trotter(x_, V, eh, s, n_terms) for x_ in w)
    ovn = _overlap_k(wn, mo, kind)
    ratio = ovn / ov
    expo = -s * shift_term + fb_term + dt * (es + h0_prop)
    imp = torch.exp(expo) * ratio
    theta = torch.angle(torch.exp(-s * shift_term) * ratio)
    imp_ph = torch.abs(imp) * torch.cos(theta)
    bad = ~torch.isfinite(imp_ph) | (imp_ph < w_floor) | (imp_ph > w_cap)
    imp_ph = torch.where(bad, torch.zeros_like(imp_ph), imp_ph)
    wtn = wt * imp_ph
    wtn = torch.where(wtn > w_cap, torch.zeros_like(wtn), wtn)
    avg = torch.clamp(torch.mean(wtn), min=1e-300)
    esn = ee - damping * (torch.log(avg) / dt)
    return wn, wtn, ovn, esn


def mixed_energy(h1, *, h0, chol, mo, rdm1, fields, walkers0, e_estimate0, steps_per_block, dt, n_terms,
                 shift_ema=0.1, w_floor=1e-3, w_cap=100.0, damping=0.1, kind="rhf_r"):
    """J(h1) (see module docstring); fields (T, W, G), walkers0 (W, N, n) or a (wa, wb)
    tuple; mo an (N, n) tensor or (mo_a, mo_b) for uhf_u."""
    mf_im, h0_prop, eh = prop_consts(h0, h1, chol, rdm1, dt)
    rot = lambda m: torch.einsum("pi,gpj->gij", m, chol)
    rot_chol = (rot(mo[0]), rot(mo[1])) if kind == "uhf_u" else rot(mo)
    rot_h1 = (mo[0].T @ h1, mo[1].T @ h1) if kind == "uhf_u" else mo.T @ h1
    w = walkers0
    W = (w[0] if isinstance(w, tuple) else w).shape[0]
    wt = torch.ones(W, dtype=torch.float64)
    ov = _overlap_k(w, mo, kind)
    es = torch.tensor(e_estimate0, dtype=torch.float64)
    ee = torch.tensor(e_estimate0, dtype=torch.float64)
    num = torch.zeros((), dtype=torch.float64)
    den = torch.zeros((), dtype=torch.float64)
    thresh = math.sqrt(2.0 / dt)
    for t in range(fields.shape[0]):
        w, wt, ov, es = step(w, wt, ov, es, ee, fields[t], mo=mo, rot_chol=rot_chol, chol=chol, mf_im=mf_im,
                             h0_prop=h0_prop, eh=eh, dt=dt, n_terms=n_terms, w_floor=w_floor, w_cap=w_cap,
                             damping=damping, kind=kind)
        if (t + 1) % steps_per_block == 0:
            w = qr_phase_fixed(w) if kind == "rhf_r" else tuple(qr_phase_fixed(x_) for x_ in w)
            ov = _overlap_k(w, mo, kind)
            e = _energy_k(w, mo, h0, rot_h1, rot_chol, kind).real
            finite = torch.isfinite(e)
            keep = finite & ((e - ee).abs() <= thresh)
            e_t = torch.where(keep, torch.where(finite, e, torch.zeros_like(e)), ee.expand_as(e))
            wt = torch.where(finite, wt, torch.zeros_like(wt))
            nb, db = torch.sum(wt * e_t), torch.sum(wt)
            e_block = torch.where(db == 0, ee, nb / torch.where(db == 0, torch.ones_like(db), db))
            ee = (1.0 - shift_ema) * ee + shift_ema * e_block
            num = num + nb
            den = den + db
    return num / den
