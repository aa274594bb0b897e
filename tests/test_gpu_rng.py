"""The reference's random streams on the engine (SLFMM_RNG_CHACHA8): every
Gaussian sketch a fit draws -- Omega (src/rsvd.rs:44-46) and the NMF probe
(src/nmf.rs:291-293, seed + 1 000 000) -- is ChaCha8Rng::seed_from_u64 +
Normal(0, 1), and the CV hold-out masks (src/nmf.rs:433-448,
src/testing.rs:437-452) are ChaCha8Rng::seed_from_u64 + Uniform(0, 1).  The
engine's Omega equals the host draw, a fit equals the counter-stream engine's
fit with that Omega passed in, bit for bit, and the NMF fit holds out the
same calls as the FP64 oracle drawing the same streams."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_fit import _check
from test_gpu_upload import _same

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chacha_engine():
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8, rng=sg.SketchRng.CHACHA8)
    yield eng
    eng.close()


def test_generate_omega_streams(engine, chacha_engine):
    import schnellfmm_gb300 as sg
    np.testing.assert_array_equal(chacha_engine.generate_omega(42, 500, 13), sg.reference_normal(42, 500, 13))
    np.testing.assert_array_equal(chacha_engine.generate_omega(42, 500, 13), O.chacha8_normal_matrix(42, 500, 13))
    # the default engine draws the reference's stream; 2 000 x 40 draws take
    # the parallel host path (outputs generated and tested on threads)
    default = sg.Engine(precision=sg.Precision.SPLIT_FP8)
    try:
        np.testing.assert_array_equal(default.generate_omega(7, 2000, 40), O.chacha8_normal_matrix(7, 2000, 40))
    finally:
        default.close()
    # the counter stream: same draws, device log / cos against numpy's (ulps)
    np.testing.assert_allclose(engine.generate_omega(42, 500, 13), O.rng_normal_matrix(42, 500, 13),
                               rtol=0, atol=1e-13)


@pytest.mark.parametrize("host", [False, True])
def test_fit_chacha_equals_injected_omega(engine, chacha_engine, host):
    """Resident fit and slfmm_fit_host (sketch drawn under the upload)."""
    import schnellfmm_gb300 as sg
    c = simdata.simulate(300, 5000, k_pop=3, fst=0.08, miss=0.02, d=2, seed=41)
    cfg = sg.Lfmm2Config(k=3, oversampling=5, seed=123, norm=sg.SnpNorm.EIGENSTRAT)
    omega = sg.reference_normal(cfg.seed, c.n, 8)
    if host:
        got = sg.fit_lfmm2_host(c.packed, c.n, c.x, cfg, engine=chacha_engine)
    else:
        g = chacha_engine.upload(c.packed, c.n)
        got = sg.fit_lfmm2(g, sg.SubsetSpec.all(), g, c.x, cfg, engine=chacha_engine)
    g2 = engine.upload(c.packed, c.n)
    ref = sg.fit_lfmm2(g2, sg.SubsetSpec.all(), g2, c.x, cfg, omega=omega, engine=engine)
    _same(got, ref)
    ora = O.fit_oracle64(c.raw, c.raw, c.x, k=3, oversampling=5, seed=cfg.seed, norm=O.NORM_EIGENSTRAT,
                         rng="chacha8")
    _check(got, ora.assoc, ora.u_hat)


def test_nmf_fit_chacha_matches_oracle(chacha_engine):
    """The NMF probe from seed + 1 000 000 and both CV masks on the
    reference's streams: the held-out calls are the oracle's (count and
    mean-fill error exact), the errors and the fit within tolerance."""
    import schnellfmm_gb300 as sg
    from test_gpu_nmf import _cohort
    raw, packed, x = _cohort()
    n = raw.shape[0]
    k, it, rate, chunk, seed = 4, 6, 0.01, 1000, 42
    nmf = sg.NmfConfig(k=k, n_iter=it, eps=1e-16, cv_rate=rate)
    cfg = sg.Lfmm2Config(k=3, lambda_=1e-5, oversampling=10, norm=sg.SnpNorm.EIGENSTRAT,
                         impute=sg.ImputeStrategy.NMF, nmf=nmf, chunk_size=chunk, seed=seed)
    geno = chacha_engine.upload(packed, n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, cfg, engine=chacha_engine)
    ref = O.fit_oracle64(raw, raw, x, k=3, lam=1e-5, oversampling=10, seed=seed, norm=O.NORM_EIGENSTRAT,
                         nmf=dict(k=k, n_iter=it, eps=1e-16, cv_rate=rate), chunk=chunk, rng="chacha8")
    np.testing.assert_allclose(res.nmf_cv, ref.nmf.cv_mae_per_iter, rtol=2e-3, atol=0)
    assert res.nmf_cv_mean == pytest.approx(ref.nmf.cv_mae_mean_impute, rel=1e-9)
    mae, mmae, cnt = ref.gwas_cv
    assert res.nmf_gwas_cv_count == cnt > 0
    assert res.nmf_gwas_cv_mean_mae == pytest.approx(mmae, rel=1e-9)
    assert res.nmf_gwas_cv_mae == pytest.approx(mae, rel=2e-3)
    # a different stream than the counter one: other calls are held out
    ctr = O.fit_oracle64(raw, raw, x, k=3, lam=1e-5, oversampling=10, seed=seed, norm=O.NORM_EIGENSTRAT,
                         nmf=dict(k=k, n_iter=it, eps=1e-16, cv_rate=rate), chunk=chunk)
    assert ctr.nmf.cv_mae_mean_impute != ref.nmf.cv_mae_mean_impute
    assert O.principal_angles_sin_max(res.u_hat, ref.u_hat) < 2e-3
    dt = np.abs(res.tstat - ref.assoc.tstat).max()
    assert dt <= 1e-3, f"max|dt| = {dt}"
    assert np.abs(res.r2 - ref.assoc.r2).max() <= 1e-4
    geno.free()
