"""The FP64 VHS over the packed upper triangle (``trot_system.chol_packed``, set when every
Cholesky vector is exactly symmetric) against the full product.

Every VHS element is the same dot product over the Cholesky index in both forms, so
apply-Trotter and a whole FP64 step give bit-identical walkers, weights and overlaps.  The
step VJP's transpose contraction sums g_V + g_V^T before the product, so it agrees to
rounding."""
import dataclasses

import numpy as np
import pytest
import torch

from tests.gpu_helpers import Setup, cpu, dev, rel

needs_cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="no CUDA device")


def test_pack_symmetric_cpu():
    from trot_gb300.prop import pack_symmetric

    rng = np.random.default_rng(0)
    c = rng.normal(size=(3, 5, 5))
    c = torch.as_tensor(c + c.transpose(0, 2, 1))
    p = pack_symmetric(c)
    iu = np.triu_indices(5)
    assert p.shape == (3, 15) and np.array_equal(p.numpy(), c.numpy()[:, iu[0], iu[1]])
    # row-major packed index k(p, q) = p N - p (p - 1) / 2 + q - p
    assert p[1, 1 * 5 - 0 + 3 - 1].item() == c[1, 1, 3].item()
    c2 = c.clone()
    c2[2, 0, 1] += 1e-15
    assert pack_symmetric(c2) is None


def _setup(kind, N=24, nelec=(5, 4), G=60, W=9):
    from trot_gb300 import synthetic

    ss = synthetic.make_system(N, nelec if kind == "uhf_u" else (nelec[0], nelec[0]), G, decay=30.0, seed=8, h0=0.1)
    S = Setup(kind, ss.h0, ss.h1, ss.chol, ss.mo_a, ss.mo_b, 0.01, W)
    wa = synthetic.perturbed_walkers(ss.mo_a, W, 0.1, 3)
    wb = synthetic.perturbed_walkers(ss.mo_b, W, 0.1, 4)
    return ss, S, (wa if kind == "rhf_r" else (wa, wb))


@pytest.mark.gpu
@needs_cuda
@pytest.mark.parametrize("kind", ["rhf_r", "rhf_u", "uhf_u"])
def test_apply_trotter_and_step_packed_vs_full(kind):
    import trot_gb300 as tg

    ss, S, w0 = _setup(kind)
    assert S.prop_ctx.chol_packed is not None
    full = dataclasses.replace(S.prop_ctx, chol_packed=None)
    W, G = S.params.n_walkers, ss.nchol
    rng = np.random.default_rng(5)
    xs = dev(rng.normal(size=(W, G)) + 0.3j * rng.normal(size=(W, G)))
    ops = tg.make_trotter_ops("restricted", S.walker_kind)
    a = ops.apply_trotter(S.walkers(w0), xs, S.prop_ctx, 6)
    b = ops.apply_trotter(S.walkers(w0), xs, full, 6)
    for x, y in zip(a if isinstance(a, tuple) else (a,), b if isinstance(b, tuple) else (b,)):
        assert np.array_equal(cpu(x), cpu(y))
    fields = dev(rng.standard_normal((W, G)))
    outs = []
    for ctx in (S.prop_ctx, full):
        w = S.walkers(w0)
        st = S.state(w, np.linspace(0.5, 1.5, W), cpu(S.overlap(w)), -1.0, -1.2)
        S.prop_ctx, keep = ctx, S.prop_ctx
        try:
            st = S.step(st, fields)
        finally:
            S.prop_ctx = keep
        ws = st.walkers if isinstance(st.walkers, tuple) else (st.walkers,)
        outs.append([cpu(x) for x in ws] + [cpu(st.weights), cpu(st.overlaps), cpu(st.scalars)])
    for x, y in zip(*outs):
        assert np.array_equal(x, y)


@pytest.mark.gpu
@needs_cuda
def test_step_vjp_packed_vs_full():
    from tests.test_gpu_adjoint import _c, _problem, _rand_like
    from trot_gb300 import adjoint

    ss, fields, w0, prob = _problem()
    assert prob.chol_packed is not None
    W = w0.shape[0]
    res = []
    for packed in (True, False):
        if not packed:
            prob.chol_packed = None
        w = _c(w0).cuda().requires_grad_(True)
        wb = torch.empty(0, dtype=torch.complex128, device="cuda", requires_grad=True)
        wt = torch.linspace(0.5, 1.5, W, dtype=torch.float64, device="cuda").requires_grad_(True)
        ov = torch.ones(W, dtype=torch.complex128, device="cuda").requires_grad_(True)
        scal = torch.tensor([-1.7, -2.1], dtype=torch.float64, device="cuda").requires_grad_(True)
        eh = adjoint.ExpH1Half.apply(torch.as_tensor(ss.h1).cuda(), prob).detach().requires_grad_(True)
        x = torch.as_tensor(fields[0]).cuda()
        wa_o, _, wt_o, ov_o, sc_o = adjoint.Step.apply(w, wb, wt, ov, scal, eh, x, prob)
        outs = (wa_o, wt_o, ov_o, sc_o)
        gs = [_rand_like(o.detach().cpu(), 20 + i).cuda() for i, o in enumerate(outs)]
        grads = torch.autograd.grad(outs, (w, wt, ov, scal, eh), gs)
        res.append(([cpu(o.detach()) for o in outs], [cpu(g) for g in grads]))
    (f1, g1), (f2, g2) = res
    for a, b in zip(f1, f2):
        assert np.array_equal(a, b)
    for a, b in zip(g1, g2):
        assert rel(a, b) < 1e-12
