"""The PyTorch operator face (torch.ops.trot_gb300.*) without a GPU: every
operator is registered with the dispatcher and its fake implementation gives
the output shapes and dtypes for fake CUDA tensors (what tracing and
FakeTensorMode see)."""
import pytest
import torch
from torch._subclasses.fake_tensor import FakeTensorMode

import trot_gb300.torch_ops  # noqa: F401  (registers the operators)

OPS = ["overlap", "force_bias", "local_energy", "orthonormalize", "sr_resample", "prop_step", "prop_step_functional"]


def test_registered():
    for name in OPS:
        assert hasattr(torch.ops.trot_gb300, name), name


def test_fake_shapes():
    W, N, na, nb, G = 5, 11, 3, 2, 7
    c128, f64 = torch.complex128, torch.float64
    with FakeTensorMode():
        def t(*shape, dtype=f64):
            return torch.empty(*shape, dtype=dtype, device="cuda")

        wa, wb = t(W, N, na, dtype=c128), t(W, N, nb, dtype=c128)
        mo_a, mo_b = t(N, na), t(N, nb)
        ha, hb, ra, rb = t(na, N), t(nb, N), t(G, na, N), t(G, nb, N)
        o = torch.ops.trot_gb300
        assert o.overlap(wa, wb, mo_a, mo_b, 2).shape == (W,)
        fb = o.force_bias(wa, wb, mo_a, mo_b, ra, rb, 2, False)
        assert fb.shape == (W, G) and fb.dtype == c128
        e = o.local_energy(wa, wb, mo_a, mo_b, ha, hb, ra, rb, 0.5, 2, True)
        assert e.shape == (W,) and e.dtype == c128
        qa, qb, nrm = o.orthonormalize(wa, wb, 2)
        assert qa.shape == wa.shape and qb.shape == wb.shape and nrm.shape == (W,)
        sa, sb, sw, idx = o.sr_resample(wa, wb, t(W), 0.3, 2)
        assert sa.shape == wa.shape and sw.shape == (W,) and idx.dtype == torch.int64
        scal, nodes = t(2), torch.empty(1, dtype=torch.int64, device="cuda")
        e2 = o.prop_step(wa, wb, t(W), t(W, dtype=c128), scal, nodes, t(W, G), mo_a, mo_b, ha, hb, ra, rb, t(N, N),
                         t(G, N * N), t(G), 0.1, -0.2, 0.005, 6, 1e-3, 100.0, 0.1, 2, False)
        assert e2.shape == (W,) and e2.dtype == c128
