"""Host-side operand preparation of the mixed-precision path (no GPU)."""
import numpy as np
import pytest
import torch

from trot_gb300 import mixed


def test_digit_slices_reconstruct_rows():
    """Cholesky-row digits: |q_0| <= 512, balanced |q_t| <= 256, all exact in FP16,
    representation error <= 2^-45 of the row's power-of-two scale 2^e, and the sum
    of |q_0| over a row capped at 2^15 (the exponent is raised by one otherwise)."""
    rng = np.random.default_rng(0)
    x = rng.normal(size=(9, 120)) * np.exp(rng.normal(size=(9, 1)) * 5)
    x[3] = 0.0
    x[4, :] = 2.0 ** 5  # exact power of two: every element sits on the digit range boundary
    x[5, :] = 0.3       # constant row: the top digits all share one sign (largest L1 norm)
    q, e = mixed.digit_slices(x)
    assert q.shape == (mixed.SLICES, 9, 120)
    assert np.all(q == np.rint(q))
    assert np.all(np.abs(q[0]) <= 2 ** mixed.ROT_TOP_BITS)
    assert np.all(np.abs(q[1:]) <= 2 ** (mixed.LOW_BITS - 1))
    assert np.all(np.sum(np.abs(q[0]), axis=-1) <= mixed.ROT_L1_CAP)
    # every digit is exactly representable in fp16
    qh = torch.from_numpy(q).to(torch.float16).to(torch.float32).numpy()
    np.testing.assert_array_equal(qh, q)
    sh = [mixed.ROT_TOP_BITS + mixed.LOW_BITS * t for t in range(mixed.SLICES)]
    rec = sum(q[t].astype(np.float64) * np.ldexp(1.0, e - sh[t])[:, None] for t in range(mixed.SLICES))
    err = np.abs(rec - x) / np.ldexp(1.0, e)[:, None]
    assert np.max(err) <= 2.0 ** -(sh[-1] + 1)
    assert np.all(rec[3] == 0.0)
    # the constant row needed the raised exponent: 120 top digits of 0.3 / 0.5 * 512 = 307
    assert int(e[5]) == 0


def test_digit_groups_fit_fp32_exactly():
    """Worst-case partial sums of the two leading digit-product groups against
    Green's-function digits (|q_0| <= 256, |q_t| <= 256) stay within 2^24, so the
    tensor core's FP32 accumulator adds them exactly."""
    rng = np.random.default_rng(7)
    rows = np.concatenate([rng.normal(size=(20, 128)), np.full((2, 128), 0.7), np.abs(rng.normal(size=(2, 128)))])
    q, _ = mixed.digit_slices(rows)
    l1_0 = np.sum(np.abs(q[0]), axis=-1)
    l1_1 = np.sum(np.abs(q[1]), axis=-1)
    g0max = 2.0 ** mixed.GREEN_TOP_BITS
    glow = 2.0 ** (mixed.LOW_BITS - 1)
    assert np.all(l1_0 * g0max <= 2 ** 24)               # group 0: sum |qA_0 qB_0|
    assert np.all(l1_0 * glow + l1_1 * g0max <= 2 ** 24)  # group 1: sum |qA_0 qB_1| + |qA_1 qB_0|


def test_plain_split_is_fp32_accurate():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(50, 64))
    parts = mixed.plain_split(x)
    rec = sum(p.to(torch.float64).numpy() for p in parts)
    assert np.max(np.abs(rec - x) / np.abs(x)) < 2.0 ** -23


def test_rot_tiles_layout():
    rng = np.random.default_rng(2)
    G, n, N = 25, 12, 120
    rc = rng.normal(size=(G, n, N))
    img, e, gb, nblk = mixed.rot_tiles(rc)
    ks = mixed.KPAD // 16
    assert gb == 10 and nblk == 3
    assert tuple(img.shape) == (nblk, ks, mixed.SLICES, 128, 16)
    # undo the core-matrix order: (blk, kstep, plane, rg, kg, ri, ki) -> (plane, blk, row 8 rg + ri, k 16 kstep + 8 kg + ki)
    im = img.to(torch.float64).numpy().reshape(nblk, ks, mixed.SLICES, 16, 2, 8, 8)
    qd = im.transpose(2, 0, 3, 5, 1, 4, 6).reshape(mixed.SLICES, nblk, 128, mixed.KPAD)
    # row (g=13, i=4) lives in block 1, row 3*12+4, orbitals 0..N-1; padding is zero
    sh = [mixed.ROT_TOP_BITS + mixed.LOW_BITS * t for t in range(mixed.SLICES)]
    rec = sum(qd[t, 1, 3 * n + 4, :N] * np.ldexp(1.0, int(e[1, 3 * n + 4]) - sh[t]) for t in range(mixed.SLICES))
    # representation error <= 2^(e - top - low (slices - 1) - 1), e <= log2 max|row| + 2 (the L1 cap)
    bits = mixed.ROT_TOP_BITS + mixed.LOW_BITS * (mixed.SLICES - 1)
    np.testing.assert_allclose(rec, rc[13, 4], rtol=0, atol=2.0 ** (1 - bits) * np.max(np.abs(rc[13, 4])))
    assert img.dtype == torch.float16
    assert np.all(qd[:, :, :, N:] == 0)
    assert np.all(qd[:, 2, 5 * n:, :] == 0)  # last block holds 5 vectors
    # byte offset of element (row 8 rg + ri, k 8 kg + ki) inside a (kstep, plane) block
    flat = img.numpy().reshape(nblk, ks, mixed.SLICES, 128 * 16)
    r, k = 77, 13
    off = (r >> 3) * 128 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7)
    assert flat[1, 2, 3, off] == np.float16(qd[3, 1, r, 2 * 16 + k])


@pytest.mark.parametrize("kchunk", [32, 64])
def test_split3_image_layout(kchunk):
    """Tensor-core operand image of B^T: [ncols/128][K/kchunk][3][128][kchunk] in
    8 x 8 core-matrix order; the three BF16 terms add up to the FP64 value to ~2^-24."""
    rng = np.random.default_rng(3)
    bt = rng.normal(size=(150, 70))
    img, npad, kpad = mixed.split3_image(bt, kchunk=kchunk)
    assert npad == 256 and kpad == (70 + kchunk - 1) // kchunk * kchunk
    assert tuple(img.shape) == (2, kpad // kchunk, 3, 128, kchunk)
    a = img.to(torch.float64).numpy().reshape(2, kpad // kchunk, 3, 16, kchunk // 8, 8, 8)
    # (nt, nk, slice, rg, kg, r, k) -> (slice, nt, rg, r, nk, kg, k)
    m = a.transpose(2, 0, 3, 5, 1, 4, 6).reshape(3, npad, kpad)
    rec = m.sum(axis=0)
    np.testing.assert_allclose(rec[:150, :70], bt, rtol=2.0 ** -23, atol=0)
    assert np.all(rec[150:] == 0) and np.all(rec[:, 70:] == 0)
    # the image's first row of the first chunk is contiguous in 8-element core-matrix rows
    flat = img.to(torch.float64).numpy().reshape(2, kpad // kchunk, 3, -1)
    assert flat[0, 0, 0, 1] == m[0, 0, 1]


def test_packed_vhs_operand_matches_full_product():
    """With symmetric Cholesky matrices the VHS operand is the packed upper triangle, and
    column packed_index(p, q) of x @ B reproduces VHS[p][q] for every (p, q); a general set
    keeps the full (N^2, G) operand."""
    from trot_gb300 import mixed, synthetic

    N, G = 9, 13
    _, _, chol = synthetic.hamiltonian(N, G, 30.0, 3, 0.0)
    x = np.random.default_rng(4).standard_normal((5, G))
    vhs = np.einsum("bg,gpq->bpq", x, chol)
    bt, packed = mixed.vhs_operand(chol.reshape(G, N * N))
    assert packed and bt.shape == (N * (N + 1) // 2, G)
    vp = x @ bt.T
    for p in range(N):
        for q in range(N):
            np.testing.assert_allclose(vp[:, mixed.packed_index(p, q, N)], vhs[:, p, q], rtol=1e-13, atol=1e-13)
    skew = np.random.default_rng(5).standard_normal(chol.shape) * 1e-3
    bt_g, packed_g = mixed.vhs_operand((chol + skew - skew.transpose(0, 2, 1)).reshape(G, N * N))
    assert not packed_g and bt_g.shape == (N * N, G)
