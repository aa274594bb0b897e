"""The tcgen05 contraction against exact host arithmetic: genotypes are
exact in BF16, W is split hi + lo BF16, accumulation is FP32."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata

pytestmark = pytest.mark.gpu


def bf16_round(x32: np.ndarray) -> np.ndarray:
    u = x32.astype(np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def split_value(w: np.ndarray) -> np.ndarray:
    w32 = w.astype(np.float32)
    hi = bf16_round(w32)
    lo = bf16_round((w32 - hi).astype(np.float32))
    return hi.astype(np.float64) + lo.astype(np.float64)


def exact_g(c):
    g = np.nan_to_num(c.raw, nan=0.0)       # missing calls contribute 0
    return g                                # (n, p)


@pytest.mark.parametrize("n,p,w", [(300, 1000, 5), (1000, 777, 30), (257, 2000, 70), (4100, 300, 128)])
def test_rows_match_exact(engine, n, p, w):
    c = simdata.simulate(n, p, miss=0.03, seed=n + p)
    geno = engine.upload(c.packed, n)
    W = np.random.default_rng(1).normal(size=(n, w))
    out = geno.contract_raw(W)
    ref = exact_g(c).T @ split_value(W)
    scale = np.abs(exact_g(c)).T @ np.abs(split_value(W))
    assert np.all(np.abs(out - ref) <= 2e-6 * scale + 1e-5), np.abs(out - ref).max()


def test_rows_one_hot_layout(engine):
    """One-hot W columns return single genotype columns exactly (layout check)."""
    n, p = 600, 400
    c = simdata.simulate(n, p, miss=0.05, seed=3)
    geno = engine.upload(c.packed, n)
    pick = np.array([0, 1, 2, 3, 63, 64, 127, 128, 129, 255, 256, 511, 512, 599, 300, 17])
    W = np.zeros((n, len(pick)))
    W[pick, np.arange(len(pick))] = 1.0
    out = geno.contract_raw(W)
    np.testing.assert_array_equal(out, exact_g(c)[pick].T.astype(np.float32))


@pytest.mark.parametrize("n,p,w", [(300, 5000, 30), (1111, 20000, 16)])
def test_transposed_match_exact(engine, n, p, w):
    c = simdata.simulate(n, p, miss=0.02, seed=p)
    geno = engine.upload(c.packed, n)
    Q = np.random.default_rng(2).normal(size=(p, w)) / np.sqrt(p)
    out = geno.contract_raw(Q, transposed=True)
    ref = exact_g(c) @ split_value(Q)
    scale = np.abs(exact_g(c)) @ np.abs(split_value(Q))
    assert np.all(np.abs(out - ref) <= 2e-6 * scale + 1e-6), np.abs(out - ref).max()
