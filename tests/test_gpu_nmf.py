"""NMF imputation on the GPU (src/nmf.rs, src/parallel.rs:219-321,
src/testing.rs:423-487) against the FP64 oracle with the same random streams:
held-out counts exact, CV errors and the fit's statistics within tolerance."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata

pytestmark = pytest.mark.gpu


def _cohort(seed=13):
    c = simdata.simulate(400, 3000, k_pop=3, fst=0.12, miss=0.04, d=2, n_causal=20, effect=0.4, seed=seed)
    # plus contiguous missing blocks per sample, like the NMF benchmark shape
    rng = np.random.default_rng(seed)
    raw = c.raw.copy()
    for i in range(0, c.n, 7):
        s = int(rng.integers(0, c.p - 100))
        raw[i, s:s + 100] = np.nan
    g = np.where(np.isnan(raw), 255, raw).astype(np.int16)
    codes = O.genotypes_to_codes(g.T)
    packed = O.pack_codes(codes)
    return raw, packed, c.x


@pytest.mark.parametrize("prec,k", [("fp8", 4), ("bf16", 4), ("fp32", 4), ("fp8", 20)])
def test_nmf_fit_matches_oracle(engines, prec, k):
    """k = 20: NMF ranks above 16 (NmfConfig.k is any usize in the
    reference, src/nmf.rs:15-35)."""
    import schnellfmm_gb300 as sg
    eng = engines[prec]
    raw, packed, x = _cohort()
    n, p = raw.shape
    it, rate, chunk, seed = 6, 0.01, 1000, 42
    nmf = sg.NmfConfig(k=k, n_iter=it, eps=1e-16, cv_rate=rate)
    cfg = sg.Lfmm2Config(k=3, lambda_=1e-5, oversampling=10, norm=sg.SnpNorm.EIGENSTRAT,
                         impute=sg.ImputeStrategy.NMF, nmf=nmf, chunk_size=chunk, seed=seed)
    omega = O.rng_normal_matrix(9, n, 13)
    geno = eng.upload(packed, n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, cfg, omega=omega, engine=eng)
    ref = O.fit_oracle64(raw, raw, x, k=3, lam=1e-5, oversampling=10, seed=seed, norm=O.NORM_EIGENSTRAT,
                         omega=omega, nmf=dict(k=k, n_iter=it, eps=1e-16, cv_rate=rate), chunk=chunk)
    # estimation-phase CV: same held-out calls, errors within the FP32 products' noise
    assert len(res.nmf_cv) == it
    np.testing.assert_allclose(res.nmf_cv, ref.nmf.cv_mae_per_iter, rtol=2e-3, atol=0)
    assert res.nmf_cv_mean == pytest.approx(ref.nmf.cv_mae_mean_impute, rel=1e-9)
    # GWAS-phase CV: held-out count exact
    mae, mmae, cnt = ref.gwas_cv
    assert res.nmf_gwas_cv_count == cnt > 0
    assert res.nmf_gwas_cv_mean_mae == pytest.approx(mmae, rel=1e-9)
    assert res.nmf_gwas_cv_mae == pytest.approx(mae, rel=2e-3)
    # the imputed fit
    assert O.principal_angles_sin_max(res.u_hat, ref.u_hat) < 2e-3
    dt = np.abs(res.tstat - ref.assoc.tstat).max()
    assert dt <= 1e-3, f"max|dt| = {dt}"
    assert np.abs(res.r2 - ref.assoc.r2).max() <= 1e-4
    assert abs(res.gif - ref.assoc.gif) <= 0.0023
    geno.free()


def test_nmf_rank_limit(engine):
    import schnellfmm_gb300 as sg
    raw, packed, x = _cohort(5)
    geno = engine.upload(packed, raw.shape[0])
    cfg = sg.Lfmm2Config(k=3, impute=sg.ImputeStrategy.NMF, nmf=sg.NmfConfig(k=33, n_iter=1))
    with pytest.raises(sg.SchnelGpuError, match="NMF rank"):
        sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, cfg, engine=engine)
    geno.free()
