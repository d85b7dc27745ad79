"""FP64-accurate Gram blocks on the tensor cores (qpgpu_gram_tc) against exact sums.

X = A^T B for tall A (N x m) and B (N x n) -- the dgemm('T','N') projections of
davidson_diag_hjj_sjj (src/Davidson/diagonalization_hs2.irp.f:232-238) -- is
computed by Ozaki splitting into BF16 digit planes on tcgen05.  Reference
values are exact: every product a_i b_i is split into four exact FP64 parts
(Dekker's splitting into 26-bit halves) and summed with math.fsum (correctly
rounded).  The bar is the FP64 one: the error of an entry stays within
4 eps sqrt(N) sum_i |a_i b_i| (the typical FP64 dot-product error), and a
sum of squares (a Gram diagonal) within 4 eps of its exact value.
"""
import ctypes as C
import math

import numpy as np
import pytest

from quantum_package_gb300 import _lib

pytestmark = pytest.mark.gpu
EPS = np.finfo(np.float64).eps


def _split(a):
    c = a * 134217729.0  # 2^27 + 1
    hi = c - (c - a)
    return hi, a - hi


def _exact_dot(a, b):
    ah, al = _split(a)
    bh, bl = _split(b)
    return math.fsum(np.concatenate([ah * bh, ah * bl, al * bh, al * bl]).tolist())


def _gram_tc(wf, A, B):
    import torch
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B)).cuda()
    m, n = A.shape[1], B.shape[1]
    X = torch.empty((m, n), dtype=torch.float64, device="cuda")
    L = _lib.load()
    rc = L.qpgpu_gram_tc(wf.ctx, C.c_void_p(dA.data_ptr()), m, m, C.c_void_p(dB.data_ptr()), n, n, A.shape[0],
                         C.c_void_p(X.data_ptr()), None)
    _lib.check(rc, wf.ctx)
    return X.cpu().numpy()


@pytest.fixture(scope="module")
def wf():
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.sigma import Wavefunction
    p = G.make_problem(1, n_det=200)
    w = Wavefunction.from_problem(p)
    yield w
    w.close()


@pytest.mark.parametrize("N,m,n", [(100, 8, 8), (4097, 80, 16), (300_001, 128, 16), (1_000_003, 40, 5)])
def test_gram_tc_exact_sums(wf, N, m, n):
    rng = np.random.default_rng(N + m)
    # CI-like columns: a few large entries, a long tail over many decades
    A = rng.normal(size=(N, m)) * np.exp(rng.uniform(-12, 0, size=(N, m)))
    A[0] = rng.normal(size=m)
    B = rng.normal(size=(N, n)) * np.exp(rng.uniform(-8, 2, size=(N, n)))
    X = _gram_tc(wf, A, B)
    Xd = A.T @ B
    scale = np.abs(A).T @ np.abs(B)
    errs = []
    for i, j in zip(rng.choice(m, 4), rng.choice(n, 4)):
        ex = _exact_dot(A[:, i], B[:, j])
        err = abs(X[i, j] - ex)
        assert err <= 4 * EPS * math.sqrt(N) * scale[i, j], (i, j, err)
        errs.append((err / scale[i, j], abs(Xd[i, j] - ex) / scale[i, j]))
    print(f"\nN={N} m={m} n={n}: error / sum|a b| (tensor-core, FP64 dgemm): "
          + ", ".join(f"({a:.1e}, {b:.1e})" for a, b in errs))
    np.testing.assert_allclose(X, Xd, rtol=0, atol=float(16 * EPS * math.sqrt(N) * scale.max()))


def test_gram_tc_orthogonal_columns_and_zeros(wf):
    # Gram-Schmidt case: nearly orthonormal columns, where a diagonal entry is
    # a sum of squares (a one-sided error would pile up) and the off-diagonal
    # ones cancel; exact sums as the reference.  A zero column gives zeros.
    rng = np.random.default_rng(5)
    N = 200_000
    Q, _ = np.linalg.qr(rng.normal(size=(N, 16)))
    Q[:, 15] = 0.0
    X = _gram_tc(wf, Q, Q)
    for i in range(15):
        assert abs(X[i, i] - _exact_dot(Q[:, i], Q[:, i])) <= 4 * EPS, i
    for i, j in [(0, 1), (3, 7), (14, 2)]:
        assert abs(X[i, j] - _exact_dot(Q[:, i], Q[:, j])) <= 4 * EPS, (i, j)
    assert np.all(X[15] == 0.0) and np.all(X[:, 15] == 0.0)


def test_gram_tc_rejects_bad_shapes(wf):
    L = _lib.load()
    assert L.qpgpu_gram_tc(wf.ctx, C.c_void_p(8), 200, 129, C.c_void_p(8), 8, 8, 10, C.c_void_p(8), None) == -1
    assert L.qpgpu_gram_tc(wf.ctx, C.c_void_p(8), 4, 8, C.c_void_p(8), 8, 8, 10, C.c_void_p(8), None) == -1


def _lincomb_tc(wf, blocks, Cm, out_is_last=False):
    import torch
    nb, N, nsd = blocks.shape
    dA = torch.from_numpy(np.ascontiguousarray(blocks)).cuda()
    dC = torch.from_numpy(np.ascontiguousarray(Cm)).cuda()
    dO = dA[nb - 1] if out_is_last else torch.empty((N, nsd), dtype=torch.float64, device="cuda")
    L = _lib.load()
    rc = L.qpgpu_lincomb_tc(wf.ctx, C.c_void_p(dA.data_ptr()), N * nsd, nb * nsd, nsd, C.c_void_p(dC.data_ptr()),
                            C.c_void_p(dO.data_ptr()), nsd, N, None)
    _lib.check(rc, wf.ctx)
    return dO.cpu().numpy()


@pytest.mark.parametrize("N,nb,nsd", [(129, 1, 8), (5000, 10, 8), (300_017, 7, 6), (1_000_000, 10, 8), (4000, 16, 8)])
def test_lincomb_tc_exact_sums(wf, N, nb, nsd):
    # O = [A_0 .. A_nb-1] C (the Davidson's Ritz vectors / Gram-Schmidt
    # updates).  Each row of A and each column of C has one scale (its
    # largest exponent), so the bar is norm-wise: within
    # 4 eps sqrt(m) max|a_r| max|c_j| of the exact value, the size of FP64's
    # rounding of the largest product.  Component-wise bounds of an FP64 dot
    # product are tighter for entries far below that scale.
    rng = np.random.default_rng(N + nb)
    blocks = rng.normal(size=(nb, N, nsd)) * np.exp(rng.uniform(-10, 0, size=(nb, N, nsd)))
    Cm = rng.normal(size=(nb * nsd, nsd)) * np.exp(rng.uniform(-6, 0, size=(nb * nsd, nsd)))
    Cm[:nsd] = np.eye(nsd)  # the identity part of a Gram-Schmidt update
    O = _lincomb_tc(wf, blocks, Cm)
    A = np.concatenate(list(blocks), axis=1)  # (N, m)
    Od = A @ Cm
    m = nb * nsd
    rmax = np.abs(A).max(axis=1)
    cmax = np.abs(Cm).max(axis=0)
    errs = []
    for r in rng.choice(N, 6):
        for j in rng.choice(nsd, 2):
            ex = _exact_dot(A[r], Cm[:, j])
            bar = 4 * EPS * math.sqrt(m) * rmax[r] * cmax[j]
            assert abs(O[r, j] - ex) <= bar, (r, j, O[r, j], ex)
            errs.append(abs(O[r, j] - ex) / (rmax[r] * cmax[j]))
    assert np.all(np.abs(O - Od) <= 16 * EPS * math.sqrt(m) * np.outer(rmax, cmax) + 1e-300)
    print(f"\nN={N} m={m}: error / (max|a_r| max|c_j|) up to {max(errs):.1e}")


def test_lincomb_tc_in_place_and_zeros(wf):
    # the output may be the last block of A (the Gram-Schmidt update writes
    # the new block in place); zero rows and zero columns of C give zeros
    rng = np.random.default_rng(3)
    N, nb, nsd = 70_001, 5, 8
    blocks = rng.normal(size=(nb, N, nsd))
    blocks[:, 17] = 0.0
    Cm = rng.normal(size=(nb * nsd, nsd))
    Cm[:, 3] = 0.0
    ref = np.concatenate(list(blocks), axis=1) @ Cm
    O = _lincomb_tc(wf, blocks, Cm, out_is_last=True)
    np.testing.assert_allclose(O, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    assert np.all(O[17] == 0.0) and np.all(O[:, 3] == 0.0)
    L = _lib.load()
    assert L.qpgpu_lincomb_tc(wf.ctx, None, 0, 0, 8, None, None, 8, 10, None) < 0
