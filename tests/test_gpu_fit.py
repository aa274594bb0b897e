"""fit_lfmm2 on the GPU against the FP64 oracle with the same sketch Omega:
U_hat by principal angles, max|dt| <= 1e-3, beta / r2 / GIF / p-values."""
from pathlib import Path

import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"
T_TOL = 1e-3          # max |delta t| vs FP64 (the path's stated tolerance)


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _check(res, ref, u_ref, t_tol=T_TOL):
    assert O.principal_angles_sin_max(res.u_hat, u_ref) < 1e-3
    dt = np.abs(res.tstat - ref.tstat).max()
    assert dt <= t_tol, f"max|dt| = {dt}"
    scale = np.abs(ref.beta).max()
    assert np.abs(res.beta - ref.beta).max() <= 1e-3 * scale + 1e-12
    assert np.abs(res.r2 - ref.r2).max() <= 1e-4
    # GIF can move by one histogram bin (0.001 in t^2) at a bin edge
    assert abs(res.gif - ref.gif) <= 0.0023
    # p-values follow from t and GIF.  Calibration evaluates erfc in FP32 (the
    # statistic itself is FP32): relative error ~ 2e-6 (1 + z^2) in the tail
    p_expect = O.calibrate_p(res.tstat, res.gif_per_trait)
    z = np.abs(res.tstat) / np.sqrt(res.gif_per_trait)[None, :]
    rel = np.abs(res.pvalue - p_expect) / np.maximum(p_expect, 1e-300)
    assert np.all(rel <= 2e-6 * (1.0 + z * z)), float((rel / (1 + z * z)).max())
    # top hits keep their order
    top = np.argsort(-np.abs(ref.tstat[:, 0]))[:10]
    top_gpu = np.argsort(-np.abs(res.tstat[:, 0]))[:10]
    assert set(top[:5]) <= set(top_gpu)


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_golden_c1(engines, prec):
    sg = _sg()
    eng = engines[prec]
    g = np.load(GOLD / "golden_c1.npz")
    n = int(g["n"])
    geno = eng.upload(g["packed"], n)
    cfg = sg.Lfmm2Config(k=int(g["k"]), lambda_=float(g["lam"]), oversampling=int(g["oversampling"]),
                         n_power_iter=int(g["power_iter"]), norm=sg.SnpNorm.EIGENSTRAT)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, g["x"], cfg, omega=g["omega"], engine=eng)

    class R:
        pass
    ref = R()
    for k in ("beta", "tstat", "pvalue", "r2"):
        setattr(ref, k, g[k])
    ref.gif = float(g["gif"])
    _check(res, ref, g["u_hat"])


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_multi_covariate_subset_center_only(engines, prec):
    sg = _sg()
    eng = engines[prec]
    c = simdata.simulate(517, 4000, k_pop=4, fst=0.08, miss=0.02, d=3, n_causal=25, seed=21)
    cfg = sg.Lfmm2Config(k=4, lambda_=1e-3, oversampling=6, norm=sg.SnpNorm.CENTER_ONLY, scale_cov=True)
    omega = O.rng_normal_matrix(7, c.n, 10)
    ge = eng.upload(c.packed, c.n, snps=sg.SubsetSpec.from_rate(0.5))
    gf = eng.upload(c.packed, c.n)
    res = sg.fit_lfmm2(ge, sg.SubsetSpec.all(), gf, c.x, cfg, omega=omega, engine=eng)
    idx = O.subset_indices(c.p, rate=0.5)
    ref = O.fit_oracle64(c.raw[:, idx], c.raw, c.x, k=4, lam=1e-3, oversampling=6, norm=O.NORM_CENTER_ONLY,
                         scale_cov=True, omega=omega)
    _check(res, ref.assoc, ref.u_hat)


def test_generated_omega_matches_oracle(engine):
    om = engine.generate_omega(42, 300, 13)
    np.testing.assert_allclose(om, O.rng_normal_matrix(42, 300, 13), rtol=1e-12, atol=1e-12)


def test_center_covariates(engine):
    x = np.random.default_rng(0).normal(size=(101, 4)) * [1, 3, 0, 2] + 5
    for scale in (False, True):
        np.testing.assert_allclose(engine.center_covariates(x, scale), O.center_covariates(x, scale),
                                   rtol=1e-12, atol=1e-12)


def test_engine_rng_fit_statistics(engine):
    """Engine-generated Omega; the reference's validate_results thresholds."""
    sg = _sg()
    c = simdata.simulate(300, 3000, k_pop=3, fst=0.1, miss=0.01, d=1, n_causal=30, effect=0.4, seed=11)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x,
                       sg.Lfmm2Config(k=3, norm=sg.SnpNorm.EIGENSTRAT), engine=engine)
    qa, _ = np.linalg.qr(res.u_hat - res.u_hat.mean(0))
    qt, _ = np.linalg.qr(c.u_true[:, :-1] - c.u_true[:, :-1].mean(0))
    assert np.linalg.svd(qa.T @ qt, compute_uv=False).mean() > 0.5
    assert np.mean(np.sign(res.beta[c.causal, 0]) == np.sign(c.b_true[c.causal, 0])) > 0.6
    null = np.setdiff1d(np.arange(c.p), c.causal)
    assert np.mean(res.pvalue[null, 0] < 0.05) < 0.15
    assert np.mean(res.pvalue[c.causal, 0] < 0.05) > 0.1
    assert 0.5 < res.gif < 2.0


def test_errors(engine):
    sg = _sg()
    c = simdata.simulate(8, 50, seed=3, d=2)
    geno = engine.upload(c.packed, c.n)
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, sg.Lfmm2Config(k=5, oversampling=1), engine=engine)
    assert e.value.code == sg.ERR_DF_NONPOSITIVE and "Insufficient degrees of freedom" in str(e.value)
    c = simdata.simulate(60, 200, seed=3)
    geno = engine.upload(c.packed, c.n)
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, sg.Lfmm2Config(k=2, lambda_=0.0), engine=engine)
    assert e.value.code == sg.ERR_BAD_ARG and "must be positive" in str(e.value)


def test_monomorphic_and_missing_snps(engine):
    sg = _sg()
    c = simdata.simulate(150, 800, miss=0.03, seed=4, monomorphic=5)
    codes = c.codes.copy()
    codes[5, :] = 1                                   # all missing
    packed = O.pack_codes(codes)
    raw = O.DECODE_TABLE[codes].T.copy()
    omega = O.rng_normal_matrix(3, c.n, 12)
    geno = engine.upload(packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, sg.Lfmm2Config(k=2, norm=sg.SnpNorm.EIGENSTRAT),
                       omega=omega, engine=engine)
    ref = O.fit_oracle64(raw, raw, c.x, k=2, norm=O.NORM_EIGENSTRAT, omega=omega)
    assert (res.tstat[:6] == 0).all() and (res.beta[:6] == 0).all() and (res.r2[:6] == 0).all()
    assert (res.pvalue[:6] == 1).all()
    _check(res, ref.assoc, ref.u_hat)


@pytest.mark.parametrize("prec", ["bf16", "fp8"])
def test_joint_many_covariates(engines, prec):
    """Reference-joint shape: many covariates (wide testing operand, 1+d+K = 71)."""
    sg = _sg()
    c = simdata.simulate(1500, 6000, k_pop=5, fst=0.05, miss=0.005, d=50, n_causal=10, seed=8)
    omega = O.rng_normal_matrix(9, c.n, 30)
    geno = engines[prec].upload(c.packed, c.n)
    cfg = sg.Lfmm2Config(k=20, oversampling=10, norm=sg.SnpNorm.EIGENSTRAT)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engines[prec])
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=20, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)


@pytest.mark.parametrize("prec", ["fp32", "fp8"])
def test_high_missingness(engines, prec):
    sg = _sg()
    c = simdata.simulate(800, 3000, k_pop=3, fst=0.1, miss=0.15, d=2, n_causal=20, seed=31)
    omega = O.rng_normal_matrix(4, c.n, 14)
    geno = engines[prec].upload(c.packed, c.n)
    cfg = sg.Lfmm2Config(k=4, norm=sg.SnpNorm.EIGENSTRAT)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engines[prec])
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=4, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)
