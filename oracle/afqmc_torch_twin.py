"""Test infrastructure: a torch complex128 restatement of the phaseless step,
the local energy and the block tail for an RHF trial with restricted walkers,
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
* local energy: trot/meas/rhf.py:21-60,128-138; overlap trot/trial/rhf.py:45-47;
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


def step(w, wt, ov, es, ee, x, *, mo, rot_chol, chol, mf_im, h0_prop, eh, dt, n_terms, w_floor=1e-3, w_cap=100.0,
         damping=0.1):
    s = math.sqrt(dt)
    fb = force_bias(w, mo, rot_chol)
    mf = 1j * mf_im.to(fb.dtype)
    fs = -s * (1j * fb - mf)
    xs = x.to(fb.dtype) - fs
    shift_term = torch.sum(xs * mf, dim=1)
    fb_term = torch.sum(x * fs - 0.5 * fs * fs, dim=1)
    G, N = chol.shape[0], chol.shape[1]
    V = (xs @ chol.reshape(G, N * N).to(xs.dtype)).reshape(-1, N, N)
    ehc = eh.to(w.dtype)
    w1 = ehc @ w
    term, out = w1, w1
    for k in range(1, n_terms + 1):
        term = (1j * s / k) * (V @ term)
        out = out + term
    wn = ehc @ out
    ovn = overlap(wn, mo)
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
                 shift_ema=0.1, w_floor=1e-3, w_cap=100.0, damping=0.1):
    """J(h1) (see module docstring); fields (T, W, G), walkers0 (W, N, n)."""
    mf_im, h0_prop, eh = prop_consts(h0, h1, chol, rdm1, dt)
    rot_chol = torch.einsum("pi,gpj->gij", mo, chol)
    rot_h1 = mo.T @ h1
    w = walkers0
    W = w.shape[0]
    wt = torch.ones(W, dtype=torch.float64)
    ov = overlap(w, mo)
    es = torch.tensor(e_estimate0, dtype=torch.float64)
    ee = torch.tensor(e_estimate0, dtype=torch.float64)
    num = torch.zeros((), dtype=torch.float64)
    den = torch.zeros((), dtype=torch.float64)
    thresh = math.sqrt(2.0 / dt)
    for t in range(fields.shape[0]):
        w, wt, ov, es = step(w, wt, ov, es, ee, fields[t], mo=mo, rot_chol=rot_chol, chol=chol, mf_im=mf_im,
                             h0_prop=h0_prop, eh=eh, dt=dt, n_terms=n_terms, w_floor=w_floor, w_cap=w_cap,
                             damping=damping)
        if (t + 1) % steps_per_block == 0:
            w = qr_phase_fixed(w)
            ov = overlap(w, mo)
            e = local_energy(w, mo, h0, rot_h1, rot_chol).real
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
