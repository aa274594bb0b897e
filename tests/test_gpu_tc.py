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


def _check(out, g, W, prec):
    """BF16: exact hi+lo model.  FP8: every W element carries an error of at
    most 2^-14 of its column's max |W| (four power-of-two-scaled E4M3 terms)."""
    if prec == "bf16":
        ref = g @ split_value(W)
        scale = np.abs(g) @ np.abs(split_value(W))
        bound = 2e-6 * scale + 1e-5
    else:
        ref = g @ W
        colmax = np.abs(W).max(axis=0)
        bound = (np.abs(g).sum(axis=1)[:, None] * colmax[None, :]) * 2.0 ** -14 + 2e-6 * (np.abs(g) @ np.abs(W)) + 1e-5
    err = np.abs(out - ref)
    assert np.all(err <= bound), float((err / bound).max())
    return ref


PRECS = ["bf16", "fp8"]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,p,w", [(300, 1000, 5), (1000, 777, 30), (257, 2000, 70), (4100, 300, 128)])
def test_rows_match_exact(engines, prec, n, p, w):
    c = simdata.simulate(n, p, miss=0.03, seed=n + p)
    geno = engines[prec].upload(c.packed, n)
    W = np.random.default_rng(1).normal(size=(n, w))
    _check(geno.contract_raw(W), exact_g(c).T, W, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_rows_one_hot_layout(engines, prec):
    """One-hot W columns return single genotype columns exactly (layout check)."""
    n, p = 600, 400
    c = simdata.simulate(n, p, miss=0.05, seed=3)
    geno = engines[prec].upload(c.packed, n)
    pick = np.array([0, 1, 2, 3, 63, 64, 127, 128, 129, 255, 256, 511, 512, 599, 300, 17])
    W = np.zeros((n, len(pick)))
    W[pick, np.arange(len(pick))] = 1.0
    out = geno.contract_raw(W)
    np.testing.assert_array_equal(out, exact_g(c)[pick].T.astype(np.float32))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,p,w", [(300, 5000, 30), (1111, 20000, 16), (700, 3000, 48)])
def test_transposed_match_exact(engines, prec, n, p, w):
    c = simdata.simulate(n, p, miss=0.02, seed=p)
    geno = engines[prec].upload(c.packed, n)
    Q = np.random.default_rng(2).normal(size=(p, w)) / np.sqrt(p)
    _check(geno.contract_raw(Q, transposed=True), exact_g(c), Q, prec)


@pytest.mark.parametrize("transposed", [False, True])
def test_fp8_missing_indicator_operand(engine, transposed):
    """With the indicator operand a missing call contributes W (as if it were 1)."""
    n, p, w = 513, 2100, 30
    c = simdata.simulate(n, p, miss=0.05, seed=77)
    geno = engine.upload(c.packed, n)
    g = exact_g(c) + np.isnan(c.raw)
    rng = np.random.default_rng(5)
    if transposed:
        Q = rng.normal(size=(p, w)) / np.sqrt(p)
        _check(geno.contract_raw(Q, transposed=True, missing_as_one=True), g, Q, "fp8")
    else:
        W = rng.normal(size=(n, w))
        _check(geno.contract_raw(W, missing_as_one=True), g.T, W, "fp8")
