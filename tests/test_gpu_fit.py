"""fit_lfmm2 on the GPU against the FP64 oracle with the same sketch Omega:
U_hat by principal angles, max|dt| <= 1e-3, beta / r2 / GIF / p-values."""
from pathlib import Path

import numpy as np
import pytest

from oracle import lfmm_oracle as O
from parity import check_fit
import simdata

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"
T_TOL = 1e-3          # max |delta t| vs FP64 (the path's stated tolerance)


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _check(res, ref, u_ref, t_tol=T_TOL):
    check_fit(res, ref, u_ref, t_tol)


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


def test_singular_design_safe_inv(engine, capfd):
    """A covariate that is constant (zero after centring) makes C^T C and
    X^T X exactly singular whatever the summation order: the reference's
    safe_inv adds eps = 1e-8 max|diag| and warns on stderr
    (src/testing.rs:996-1024), and that covariate gets t = 0.  The other
    covariates are unaffected."""
    sg = _sg()
    c = simdata.simulate(300, 2000, k_pop=3, fst=0.1, miss=0.01, d=3, n_causal=20, seed=12)
    x = 0.5 * c.x
    x[:, 1] = 2.5
    omega = O.rng_normal_matrix(5, c.n, 13)
    geno = engine.upload(c.packed, c.n)
    capfd.readouterr()
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, sg.Lfmm2Config(k=3, norm=sg.SnpNorm.EIGENSTRAT),
                       omega=omega, engine=engine)
    err = capfd.readouterr().err
    ref = O.fit_oracle64(c.raw, c.raw, x, k=3, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)
    assert (res.tstat[:, 1] == 0).all() and (ref.assoc.tstat[:, 1] == 0).all()
    xs = O.center_covariates(x, False)
    cmat = np.hstack([np.ones((c.n, 1)), xs, ref.u_hat])
    ctc = cmat.T @ cmat
    _, reg = O.safe_inv(ctc)
    assert reg
    eps_c = 1e-8 * np.abs(np.diag(ctc)).max()
    eps_x = 1e-8 * np.abs(np.diag(xs.T @ xs)).max()
    assert (f"Warning: C^T C  where C = [1 | X | U_hat] is singular, adding epsilon="
            f"{O.rust_exp(eps_c, 2)} diagonal regularization") in err, err
    assert (f"Warning: X^T X for sequential R^2 is singular, adding epsilon="
            f"{O.rust_exp(eps_x, 2)} diagonal regularization") in err, err


def test_duplicated_covariate(engine):
    """Two identical covariates: C^T C is singular in exact arithmetic, and
    the reference either regularises it (a zero LU pivot) or inverts it as it
    is, depending on the rounding of C^T C; both give the pair near-zero t
    and split beta between the copies.  The GPU fit uses the limit of the
    regularised solve: both copies get |t| < 1e-3, every other covariate the
    least-squares t of the design without the copy."""
    sg = _sg()
    c = simdata.simulate(300, 2000, k_pop=3, fst=0.1, miss=0.01, d=3, n_causal=20, seed=12)
    x = 0.5 * c.x
    x[:, 2] = x[:, 0]
    omega = O.rng_normal_matrix(5, c.n, 13)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, sg.Lfmm2Config(k=3, norm=sg.SnpNorm.EIGENSTRAT),
                       omega=omega, engine=engine)
    ref = O.fit_oracle64(c.raw, c.raw, x[:, :2], k=3, norm=O.NORM_EIGENSTRAT, omega=omega)
    assert O.principal_angles_sin_max(res.u_hat, ref.u_hat) < 1e-3
    assert np.abs(res.tstat[:, [0, 2]]).max() < 1e-3
    # same least-squares fit; t scales with sqrt(df), and df = n - 1 - d - K
    # counts the copy (src/testing.rs:272-279)
    expect = ref.assoc.tstat[:, 1] * np.sqrt((c.n - 1 - 3 - 3) / (c.n - 1 - 2 - 3))
    assert np.abs(res.tstat[:, 1] - expect).max() <= 1e-3
    # ridge effects: the copies share the single-copy effect
    full = O.fit_oracle64(c.raw, c.raw, x, k=3, norm=O.NORM_EIGENSTRAT, omega=omega)
    scale = np.abs(full.assoc.beta).max()
    assert np.abs(res.beta - full.assoc.beta).max() <= 1e-3 * scale


def test_bounded_wait_expiry_leaves_context_usable():
    """Failure detection on the device without a fault: a split-FP8
    contraction whose first wait is on a barrier nothing completes gives
    SLFMM_ERR_DEVICE_TIMEOUT after the bound; the same context then fits
    normally, with the same bits as before."""
    sg = _sg()
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8)
    try:
        c = simdata.simulate(300, 2000, k_pop=3, fst=0.1, miss=0.01, d=2, seed=13)
        omega = O.rng_normal_matrix(6, c.n, 13)
        geno = eng.upload(c.packed, c.n)
        cfg = sg.Lfmm2Config(k=3, norm=sg.SnpNorm.EIGENSTRAT)
        before = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=eng)
        assert eng.lib.slfmm_debug_expire_next_wait(eng.h, 0) == sg.ERR_BAD_ARG
        eng.check(eng.lib.slfmm_debug_expire_next_wait(eng.h, 2_000_000))     # ~1 ms at 2 GHz
        with pytest.raises(sg.SchnelGpuError) as e:
            sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=eng)
        assert e.value.code == sg.ERR_DEVICE_TIMEOUT and "bounded device wait expired (site 30)" in str(e.value)
        after = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=eng)
        for k in ("tstat", "beta", "r2", "u_hat"):
            assert np.array_equal(getattr(after, k), getattr(before, k)), k
        geno.free()
    finally:
        eng.close()


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
def test_wide_design_d100_k30(engines, prec):
    """More covariates than one 64-trait epilogue block and a design wider
    than 128 columns (1 + d + K = 131): the reference puts no limit on d
    (C = [1 | X | U_hat], src/testing.rs:296-304)."""
    sg = _sg()
    c = simdata.simulate(900, 3000, k_pop=4, fst=0.08, miss=0.01, d=100, n_causal=15, seed=19)
    omega = O.rng_normal_matrix(8, c.n, 40)
    geno = engines[prec].upload(c.packed, c.n)
    cfg = sg.Lfmm2Config(k=30, oversampling=10, norm=sg.SnpNorm.EIGENSTRAT)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engines[prec])
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=30, norm=O.NORM_EIGENSTRAT, omega=omega)
    assert res.tstat.shape == (c.p, 100) and res.gif_per_trait.shape == (100,)
    _check(res, ref.assoc, ref.u_hat)
