"""Parity at the inbred-plant shape: n = 1 135 samples, 8 admixed
populations, 95 % of calls homozygous (inbreeding 0.9), 2 % missing calls,
K = 12, and factors estimated on the --est-rate 0.01 subset (SubsetSpec::Rate,
every 100th SNP: src/bed.rs:162-171, src/parallel.rs:113-122) while every SNP
is tested.  p = 100 000 SNPs gives 1 000 estimation SNPs."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
from parity import check_fit

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("host", [False, True])
def test_plant_shape_est_rate(engine, host):
    import schnellfmm_gb300 as sg
    n, p, k, l = 1135, 100_000, 12, 22
    rng = np.random.default_rng(77)
    q = rng.dirichlet(np.full(8, 0.5), size=n).astype(np.float32)
    geno = engine.simulate(q, p, fst=0.1, f_lo=0.01, f_hi=0.5, miss=0.02, inbreeding=0.9, seed=11)
    packed = np.empty((p, (n + 3) // 4), dtype=np.uint8)
    geno.download(packed)
    codes = O.unpack_codes(packed[:2000], n)
    het = np.mean(codes == 2) / np.mean(codes != 1)
    assert het < 0.1, f"heterozygous share {het:.3f}: not an inbred cohort"
    pop = q.astype(np.float64) @ rng.normal(size=(8, 1))
    x = 0.4 * pop / pop.std() + rng.normal(size=(n, 1))
    omega = O.rng_normal_matrix(5, n, l)
    cfg = sg.Lfmm2Config(k=k, lambda_=1e-5, oversampling=l - k, n_power_iter=2, norm=sg.SnpNorm.EIGENSTRAT)
    est = sg.SubsetSpec.from_rate(0.01)
    if host:
        res = sg.fit_lfmm2_host(packed, n, x, cfg, est_subset=est, omega=omega, engine=engine)
    else:
        # resident: the estimation rows are their own upload (a subset of the payload)
        ge = engine.upload(packed, n, snps=est)
        res = sg.fit_lfmm2(ge, sg.SubsetSpec.all(), geno, x, cfg, omega=omega, engine=engine)
        ge.free()
    geno.free()
    est_idx = O.subset_indices(p, rate=0.01)
    assert len(est_idx) == 1000
    ref = O.fit_oracle64_packed(packed, n, x, k=k, lam=1e-5, oversampling=l - k, power_iter=2,
                                norm=O.NORM_EIGENSTRAT, omega=omega, est_snps=est_idx)
    check_fit(res, ref.assoc, ref.u_hat)
