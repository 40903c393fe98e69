"""Numpy restatements of algorithms the CUDA kernels implement, checked on the CPU.

* ``warp_gauss_jordan`` (csrc/common.cuh): in-place Gauss-Jordan with partial pivoting (the
  first largest |A[i][k]| wins), the row interchanges undone as column interchanges in reverse
  order; the LU branch for the determinant alone.
* The tensor-core Trotter kernel's product set (csrc/mixed.cu): 3-term BF16 splits of both
  operands, products A_t [B_0; B_1] for t = 0, 1, 2 plus A_0 B_2 (t + u <= 2 and A_2 B_1).
* The packed upper triangle of the FP64 VHS (csrc/gemm64.cu): index map, mirror, and the
  transpose contraction over the packed triangle of M + M^T.
"""
import numpy as np
import pytest


def warp_gauss_jordan(A, inverse=True):
    A = np.array(A, dtype=np.complex128)
    n = A.shape[0]
    det, perm = 1.0 + 0.0j, []
    for k in range(n):
        col = np.abs(A[k:, k]) ** 2
        bi = k + int(np.argmax(col))  # argmax returns the first maximum
        if bi != k:
            A[[k, bi], :] = A[[bi, k], :]
            det = -det
        perm.append(bi)
        piv = A[k, k]
        det *= piv
        rp = 1.0 / piv
        if inverse:
            A[k, :] = np.where(np.arange(n) == k, rp, A[k, :] * rp)
            rows = [i for i in range(n) if i != k]
            cols = [j for j in range(n) if j != k]
            A[np.ix_(rows, cols)] -= np.outer(A[rows, k], A[k, cols])
            A[rows, k] = -A[rows, k] * rp
        else:
            A[k + 1:, k] *= rp
            A[k + 1:, k + 1:] -= np.outer(A[k + 1:, k], A[k, k + 1:])
    if inverse:
        for k in range(n - 1, -1, -1):
            p = perm[k]
            if p != k:
                A[:, [k, p]] = A[:, [p, k]]
    return A, det


@pytest.mark.parametrize("n", [1, 2, 5, 12, 16])
def test_warp_gauss_jordan(n):
    rng = np.random.default_rng(n)
    M = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    inv, det = warp_gauss_jordan(M)
    _, det_lu = warp_gauss_jordan(M, inverse=False)
    ref_inv, ref_det = np.linalg.inv(M), np.linalg.det(M)
    assert np.abs(inv - ref_inv).max() <= 1e-12 * np.abs(ref_inv).max()
    assert abs(det - ref_det) <= 1e-12 * abs(ref_det) and abs(det_lu - ref_det) <= 1e-12 * abs(ref_det)


def test_warp_gauss_jordan_needs_pivoting():
    M = np.array([[0.0, 2.0, 1.0], [1.0, 0.0, 3.0], [4.0, 1.0, 0.0]], dtype=np.complex128)  # zero leading pivot
    inv, det = warp_gauss_jordan(M)
    assert np.allclose(inv @ M, np.eye(3), atol=1e-14) and np.isclose(det, np.linalg.det(M))


def _bf16(x):
    """Round float64 -> bfloat16 (round to nearest even on the float32 bit pattern)."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _split3(x):
    x = np.asarray(x, dtype=np.float32).astype(np.float64)
    h = _bf16(x)
    m = _bf16(x - h)
    lo = _bf16(x - h - m)
    return h, m, lo


def test_trotter_product_set():
    rng = np.random.default_rng(1)
    A = rng.normal(size=(128, 128)) * np.exp(rng.normal(size=(128, 1)))
    B = rng.normal(size=(128, 48))
    a, b = _split3(A), _split3(B)
    six = sum(a[t] @ b[u] for t in range(3) for u in range(3) if t + u <= 2)
    stacked = sum(a[t] @ (b[0] + b[1]) for t in range(3)) + a[0] @ b[2]  # the kernel's four MMAs
    exact = A.astype(np.float32).astype(np.float64) @ B.astype(np.float32).astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B)
    e6 = np.max(np.abs(six - exact) / scale)
    e7 = np.max(np.abs(stacked - exact) / scale)
    assert e7 <= e6 * 1.0001 + 1e-18  # the extra A_2 B_1 product never hurts
    # the omitted products weigh ~2^-27 of |A| |B| (measured 2^-28.6 here); the FP32 accumulation on
    # the GPU adds ~2^-24 of the accumulated terms, so the product set is not what limits the kernel
    assert e7 < 2.0 ** -26


def test_packed_triangle_vhs_identities():
    rng = np.random.default_rng(2)
    G, N, W = 7, 6, 3
    L = rng.normal(size=(G, N, N))
    L = L + L.transpose(0, 2, 1)
    iu = np.triu_indices(N)
    P = N * (N + 1) // 2
    k = lambda p, q: p * N - p * (p - 1) // 2 + q - p  # noqa: E731
    assert [k(p, q) for p, q in zip(*iu)] == list(range(P))
    lp = L[:, iu[0], iu[1]]  # (G, P)
    x = rng.normal(size=(W, G)) + 1j * rng.normal(size=(W, G))
    vp = x @ lp  # packed VHS
    V = np.empty((W, N, N), dtype=np.complex128)
    for p in range(N):
        for q in range(N):
            V[:, p, q] = vp[:, k(min(p, q), max(p, q))]  # vhs_unpack_kernel
    assert np.allclose(V, np.einsum("wg,gpq->wpq", x, L), rtol=1e-14, atol=1e-13)
    # transpose contraction: sum_pq L[g][pq] M[w][pq] = sum_{p<=q} L[g][pq] (M + M^T - diag M)[pq]
    M = rng.normal(size=(W, N, N)) + 1j * rng.normal(size=(W, N, N))
    mp = (M + M.transpose(0, 2, 1))[:, iu[0], iu[1]]
    diag = iu[0] == iu[1]
    mp[:, diag] = M[:, iu[0][diag], iu[1][diag]]  # pack_sym_kernel: the diagonal once
    assert np.allclose(mp @ lp.T, np.einsum("wpq,gpq->wg", M, L), rtol=1e-13, atol=1e-12)
