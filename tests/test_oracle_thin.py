"""The thin (no n x n) formulation used by the GPU equals the reference's
n x n algorithm: same sketch up to the orthogonal completion Q of X."""
import json
from pathlib import Path

import numpy as np

from oracle import lfmm_oracle as O
import simdata

THRESH = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())[
    "validate_results_thresholds"]


def test_thin_rsvd_and_assoc_match_reference_form():
    c = simdata.simulate(60, 600, k_pop=3, fst=0.1, miss=0.02, d=2, n_causal=10, seed=5)
    xs = O.center_covariates(c.x, False)
    y, _, _ = O.decode_standardized(c.raw, O.NORM_EIGENSTRAT)
    k, l, q = 3, 8, 2
    full = O.precompute_full(xs, 1e-5)
    thin = O.precompute_thin(xs, 1e-5)
    omega = O.rng_normal_matrix(1, 60, l)
    u_ref = O.rsvd_ref(y, full, k, l, q, omega, chunk=128)
    # reference sketch M^T Omega = Q D Omega equals P (Q Omega)
    u_thin = O.rsvd_thin(y, thin, k, l, q, full.q_full @ omega)
    assert O.principal_angles_sin_max(u_ref, u_thin) < 1e-8
    a_ref = O.assoc_ref(y, xs, u_ref, full, chunk=100)
    a_thin = O.assoc_oracle64(y, xs, u_ref, thin.ridge_inv)
    np.testing.assert_allclose(a_thin.tstat, a_ref.tstat, atol=1e-9)
    np.testing.assert_allclose(a_thin.beta, a_ref.beta, atol=1e-9)
    np.testing.assert_allclose(a_thin.r2, a_ref.r2, atol=1e-10)
    assert a_thin.gif == a_ref.gif


def test_fit_oracle_statistical_acceptance():
    """The reference's validate_results thresholds (tests/integration.rs:506-596)."""
    c = simdata.simulate(300, 3000, k_pop=3, fst=0.1, miss=0.01, d=1, n_causal=30, effect=0.4, seed=11)
    fit = O.fit_oracle64(c.raw, c.raw, c.x, k=3, norm=O.NORM_EIGENSTRAT)
    a = fit.assoc
    # canonical correlations of U_hat with the true admixture proportions
    qa, _ = np.linalg.qr(fit.u_hat - fit.u_hat.mean(0))
    qt, _ = np.linalg.qr(c.u_true[:, :-1] - c.u_true[:, :-1].mean(0))
    cc = np.linalg.svd(qa.T @ qt, compute_uv=False)
    assert cc.mean() > THRESH["mean_cancorr_min"]
    sign = np.mean(np.sign(a.beta[c.causal, 0]) == np.sign(c.b_true[c.causal, 0]))
    assert sign > THRESH["sign_agreement_min"]
    null = np.setdiff1d(np.arange(c.p), c.causal)
    assert np.mean(a.pvalue[null, 0] < 0.05) < THRESH["fpr_max"]
    assert np.mean(a.pvalue[c.causal, 0] < 0.05) > THRESH["power_min"]
    lo, hi = THRESH["gif_range"]
    assert lo < a.gif < hi


def test_packed_streamed_oracle_equals_dense():
    """The chunk-streamed oracle (used at n = 20 000) equals the dense one."""
    c = simdata.simulate(90, 700, k_pop=3, fst=0.1, miss=0.03, d=3, n_causal=10, seed=6, monomorphic=2)
    omega = O.rng_normal_matrix(2, c.n, 9)
    est = O.subset_indices(c.p, rate=0.5)
    dense = O.fit_oracle64(c.raw[:, est], c.raw, c.x, k=4, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    packed = O.fit_oracle64_packed(c.packed, c.n, c.x, k=4, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega,
                                   est_snps=est, chunk=64)
    assert O.principal_angles_sin_max(dense.u_hat, packed.u_hat) < 1e-10
    np.testing.assert_allclose(packed.u_hat, dense.u_hat, atol=1e-10)
    np.testing.assert_allclose(packed.assoc.tstat, dense.assoc.tstat, atol=1e-9)
    np.testing.assert_allclose(packed.assoc.beta, dense.assoc.beta, atol=1e-10)
    np.testing.assert_allclose(packed.assoc.r2, dense.assoc.r2, atol=1e-10)
    assert packed.assoc.gif == dense.assoc.gif
    y = O.PackedMatrix(c.packed, c.n, O.NORM_EIGENSTRAT)
    st = O.snp_stats(c.raw, O.NORM_EIGENSTRAT)
    assert (y.counts == st.counts).all() and (y.mean == st.mean).all() and (y.scale == st.scale).all()
