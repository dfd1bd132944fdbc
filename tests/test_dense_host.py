"""Host-side dense linear algebra of the GCRO-DR cycle (vs_dense.cu), called
through the library's test hooks without a GPU: the Schur-form eigensolver
against LAPACK, the least-squares solve against NumPy, and the harmonic Ritz
selections of getHarmVecs1.m / getHarmVecs2.m against the oracle's
restatement (same subspace: eigenvectors are defined up to scale)."""
import ctypes

import numpy as np
import pytest

from oracle import krylov as K

_P = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def lib():
    from voxscatter_gb300 import build, _lib
    build.build()
    return _lib.load()


def _c(a):
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


def _p(a):
    return a.ctypes.data_as(_P)


def _same_span(A, B, tol):
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    s = np.linalg.svd(qa.conj().T @ qb, compute_uv=False)
    assert np.all(s > 1 - tol), s


@pytest.mark.parametrize("n", [1, 2, 7, 40, 75])
def test_eig_matches_lapack(lib, n):
    rng = np.random.default_rng(n)
    A = _c(rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)))
    lam = np.zeros(n, np.complex128)
    X = _c(np.zeros((n, n)))
    assert lib.vsx_dense_eig(n, _p(A), _p(lam), _p(X)) == 0
    assert np.linalg.norm(A @ X - X * lam) <= 1e-12 * np.linalg.norm(A)
    assert np.allclose(np.linalg.norm(X, axis=0), 1.0)
    ref = np.linalg.eigvals(A)
    for v in lam:
        assert np.min(np.abs(ref - v)) <= 1e-11 * np.abs(ref).max()


def test_eig_of_triangular_and_repeated(lib):
    A = _c(np.triu(np.arange(1, 26).reshape(5, 5)) + 0j)
    A[2, 2] = A[1, 1]
    lam = np.zeros(5, np.complex128)
    X = _c(np.zeros((5, 5)))
    assert lib.vsx_dense_eig(5, _p(A), _p(lam), _p(X)) == 0
    assert np.allclose(np.sort(lam.real), np.sort(np.diag(A).real))


def test_lstsq_matches_numpy(lib):
    rng = np.random.default_rng(3)
    r, c = 31, 30
    A = _c(np.triu(rng.normal(size=(r, c)) + 1j * rng.normal(size=(r, c)), -1))  # Hessenberg-shaped
    rhs = rng.normal(size=r) + 1j * rng.normal(size=r)
    y = np.zeros(c, np.complex128)
    assert lib.vsx_dense_lstsq(r, c, _p(A), _p(rhs), _p(y)) == 0
    yo = np.linalg.lstsq(A, rhs, rcond=None)[0]
    assert np.linalg.norm(y - yo) <= 1e-10 * np.linalg.norm(yo)


def _arnoldi(A, v, m):
    n = A.shape[0]
    V = np.zeros((n, m + 1), complex)
    H = np.zeros((m + 1, m), complex)
    V[:, 0] = v / np.linalg.norm(v)
    for k in range(m):
        w = A @ V[:, k]
        for _ in range(2):
            h = V[:, :k + 1].conj().T @ w
            w -= V[:, :k + 1] @ h
            H[:k + 1, k] += h
        H[k + 1, k] = np.linalg.norm(w)
        V[:, k + 1] = w / H[k + 1, k]
    return V, H


@pytest.mark.parametrize("m,k", [(12, 4), (30, 10)])
def test_harm_vecs1_matches_oracle(lib, m, k):
    rng = np.random.default_rng(m)
    n = 200
    A = np.diag(np.concatenate([np.linspace(0.05, 0.3, 6), 1 + rng.random(n - 6)])) + \
        0.05 * (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) / np.sqrt(n)
    _, H = _arnoldi(A, rng.normal(size=n) + 0j, m)
    P = _c(np.zeros((m, k)))
    Hc = _c(H)
    assert lib.vsx_dense_harm_vecs1(m, k, _p(Hc), _p(P)) == 0
    _same_span(P, K.harm_vecs1(m, k, H), 1e-8)


def test_harm_vecs2_matches_oracle(lib):
    rng = np.random.default_rng(9)
    m, k = 25, 6
    H2 = np.triu(rng.normal(size=(m + 1, m)) + 1j * rng.normal(size=(m + 1, m)), -1)
    H2[:k, :k] = np.diag(1 + rng.random(k))
    W = np.zeros((m + 1, m), complex)
    W[:, :k] = rng.normal(size=(m + 1, k)) + 1j * rng.normal(size=(m + 1, k))
    W[k:m, k:m] = np.eye(m - k)
    P = _c(np.zeros((m, k)))
    assert lib.vsx_dense_harm_vecs2(m, k, _p(_c(H2)), _p(_c(W)), _p(P)) == 0
    # the oracle takes U, V (m - k + 1 vectors) and C; build them so that
    # [C V]^H [U V_(m-k)] equals W
    Q, _ = np.linalg.qr(rng.normal(size=(40, m + 1)) + 0j)
    Cq, Vq = Q[:, :k], Q[:, k:]
    Uq = Cq @ W[:k, :k] + Vq @ W[k:, :k]
    _same_span(P, K.harm_vecs2(m, k, H2, Vq, Uq, Cq), 1e-8)
