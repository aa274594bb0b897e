"""Batched fits.  Per-trait models on their own sample sets (slfmm_fit_traits)
equal, bit for bit, one fit per trait on an upload restricted to the trait's
samples (the reference's run per trait with --intersect-samples), and the
FP64 oracle on that subset.  Many uneven problems run concurrently
(slfmm_fit_many) equal their one-by-one slfmm_fit_host fits."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_fit import _check
from test_gpu_upload import _same

pytestmark = pytest.mark.gpu


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _traits(n, t_count, seed):
    rng = np.random.default_rng(seed)
    y = rng.normal(size=(n, t_count))
    masks = np.ones((n, t_count), dtype=np.uint8)
    for t in range(t_count):
        frac = rng.uniform(0.0, 0.3)          # 0-30 % of the samples masked per trait
        masks[rng.random(n) < frac, t] = 0
    return y, masks


@pytest.mark.parametrize("prec", ["fp8", "bf16"])
def test_fit_traits_equals_subset_fits(engines, prec):
    sg = _sg()
    eng = engines[prec]
    c = simdata.simulate(400, 6000, k_pop=3, fst=0.08, miss=0.02, d=1, seed=21)
    y, masks = _traits(c.n, 4, 5)
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    geno = eng.upload(c.packed, c.n)
    res = sg.fit_lfmm2_traits(geno, y, masks, cfg, engine=eng)
    assert len(res) == 4
    for t in range(4):
        keep = np.flatnonzero(masks[:, t])
        sub = eng.upload(c.packed, c.n, sample_keep=keep)
        ref = sg.fit_lfmm2(sub, sg.SubsetSpec.all(), sub, y[keep, t:t + 1], cfg, engine=eng)
        assert res[t].u_hat.shape == (keep.size, 3)
        _same(res[t], ref)
    # one trait against the FP64 oracle on its sample subset (engine sketch)
    t = 2
    keep = np.flatnonzero(masks[:, t])
    raw = c.raw[keep]
    omega = O.rng_normal_matrix(cfg.seed, keep.size, 8)
    ora = O.fit_oracle64(raw, raw, y[keep, t:t + 1], k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res[t], ora.assoc, ora.u_hat)


def test_fit_traits_reports_the_trait(engine):
    sg = _sg()
    c = simdata.simulate(120, 800, seed=22)
    y, masks = _traits(c.n, 3, 6)
    masks[:, 1] = 0
    masks[:5, 1] = 1                          # 5 samples: n <= 1 + d + K
    geno = engine.upload(c.packed, c.n)
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.fit_lfmm2_traits(geno, y, masks, sg.Lfmm2Config(k=3, oversampling=1), engine=engine)
    assert "trait 1" in str(e.value)


def _problems(sg, count, seed):
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        n = int(rng.integers(100, 600))
        p = int(rng.integers(5000, 30000))
        k = int(rng.integers(2, 7))
        d = int(rng.integers(1, 4))
        c = simdata.simulate(n, p, k_pop=int(rng.integers(2, 5)), fst=float(rng.uniform(0.02, 0.2)), miss=0.01,
                             d=d, seed=100 + i)
        cfg = sg.Lfmm2Config(k=k, oversampling=5, seed=7 + i, norm=sg.SnpNorm.EIGENSTRAT)
        probs.append((c.packed, n, c.x, cfg))
    return probs


@pytest.mark.parametrize("streams", [1, 3])
def test_fit_many_equals_one_by_one(engine, streams):
    sg = _sg()
    probs = _problems(sg, 6, 31)
    many = sg.fit_lfmm2_many(probs, engine=engine, n_streams=streams)
    for (packed, n, x, cfg), r in zip(probs, many):
        one = sg.fit_lfmm2_host(packed, n, x, cfg, engine=engine)
        _same(r, one)


def test_fit_many_reports_the_problem(engine):
    sg = _sg()
    probs = _problems(sg, 3, 32)
    packed, n, x, cfg = probs[1]
    probs[1] = (packed, n, x, sg.Lfmm2Config(k=n, oversampling=1))   # n <= 1 + d + K
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.fit_lfmm2_many(probs, engine=engine, n_streams=2)
    assert "problem 1" in str(e.value)


@pytest.mark.parametrize("case", ["nmf", "wide"])
def test_fit_traits_row_major_subsets(engine, case):
    """Fits that need the row-major copy (NMF imputation; a sketch too wide
    for the indicator plan) take the re-packed subset: still bit for bit the
    per-trait subset fits."""
    sg = _sg()
    c = simdata.simulate(300, 3000, k_pop=3, fst=0.08, miss=0.05, d=1, seed=23)
    y, masks = _traits(c.n, 2, 8)
    if case == "nmf":
        cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT, impute=sg.ImputeStrategy.NMF,
                             nmf=sg.NmfConfig(k=4, n_iter=3, cv_rate=0.01))
    else:
        cfg = sg.Lfmm2Config(k=40, oversampling=10, norm=sg.SnpNorm.EIGENSTRAT)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2_traits(geno, y, masks, cfg, engine=engine)
    for t in range(2):
        keep = np.flatnonzero(masks[:, t])
        sub = engine.upload(c.packed, c.n, sample_keep=keep)
        ref = sg.fit_lfmm2(sub, sg.SubsetSpec.all(), sub, y[keep, t:t + 1], cfg, engine=engine)
        _same(res[t], ref)
