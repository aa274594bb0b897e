"""The small symmetric eigen-solve (Step 0's X^T X, src/precompute.rs:47; the
randomized SVD's l x l Gram, src/rsvd.rs:162) against numpy's LAPACK eigh:
FP32 one-sided Jacobi sweeps, then FP64 re-orthonormalisation and FP64
two-sided sweeps over the columns still coupled above the rounding level.
Eigenvalues to 1e-10 of the largest, eigenvectors by the projector onto
each cluster of (numerically) equal eigenvalues."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _spd(rng, m, eig):
    q, _ = np.linalg.qr(rng.standard_normal((m, m)))
    return (q * eig) @ q.T


def _check(engine, a, rel=1e-10):
    sig, v = engine.small_eigh(a)
    w, u = np.linalg.eigh(a)
    w, u = w[::-1], u[:, ::-1]
    top = abs(w[0])
    assert np.all(np.diff(sig) <= 1e-12 * top), "not descending"
    assert np.abs(v.T @ v - np.eye(len(w))).max() <= 1e-11
    # clusters of eigenvalues closer than 1e-6 of the largest: the same span,
    # and eigenvalues inside the cluster's range (any basis of a cluster's
    # span is an eigenbasis to that accuracy); isolated ones to 1e-10
    i = 0
    while i < len(w):
        j = i + 1
        while j < len(w) and w[j - 1] - w[j] <= 1e-6 * top:
            j += 1
        width = w[i] - w[j - 1]
        assert np.abs(sig[i:j] - w[i:j]).max() <= rel * top + width, (i, j, np.abs(sig[i:j] - w[i:j]).max())
        assert np.abs(a @ v[:, i:j] - v[:, i:j] * sig[i:j]).max() <= 1e-9 * top + 2 * width
        pa = v[:, i:j] @ v[:, i:j].T
        pb = u[:, i:j] @ u[:, i:j].T
        assert np.abs(pa - pb).max() <= 1e-6, (i, j)
        i = j


@pytest.mark.parametrize("m", [3, 30, 64, 100, 200])
def test_random_gram(engine, m):
    rng = np.random.default_rng(m)
    x = rng.standard_normal((3 * m, m)) * rng.uniform(0.1, 10, m)
    _check(engine, x.T @ x)


def test_near_degenerate_and_rank_deficient(engine):
    """Pairs of equal and nearly equal eigenvalues are not mixed with their
    neighbours; zero eigenvalues (a rank-deficient Gram) stay at zero."""
    rng = np.random.default_rng(1)
    eig = np.array([9.0, 9.0, 9.0 * (1 + 1e-9), 4.0, 2.0, 2.0 + 1e-7, 1.0, 0.5, 1e-6, 0.0, 0.0, 0.0])
    _check(engine, _spd(rng, 12, eig))
    eig = np.concatenate([np.full(20, 3.0), np.linspace(2.0, 1.0, 20), np.zeros(10)])
    _check(engine, _spd(rng, 50, eig))


def test_wide_spectrum(engine):
    """Eigenvalues over twelve decades, as in a Gram of nearly collinear
    covariates: the FP32 sweeps leave the small ones to the FP64 sweeps,
    which then run on those columns alone."""
    rng = np.random.default_rng(2)
    _check(engine, _spd(rng, 50, np.logspace(0, -12, 50)))
    _check(engine, _spd(rng, 30, np.concatenate([np.logspace(2, -1, 20), np.full(10, 1e-9)])))
