"""Generate the committed golden fixtures (run from the repository root):

    python tests/golden/make_golden.py

* ``reference_kats.json`` -- known answers transcribed (as data) from the
  reference crate's own unit and integration tests, with file:line sources.
  The reference (Rust) cannot be built in this environment, so these pin
  the oracle.
* ``golden_c1.npz`` -- the reference's CPU-runnable configuration
  (n=200, p=10000, 2 populations, Fst 0.1, 1 % MCAR, one covariate with 20
  causal SNPs at 0.3 SD, K=3, lambda=1e-5, q=2, oversampling 10, seed 42,
  eigenstrat) generated from a seeded synthetic cohort, with the oracle's
  FP64 outputs for an injected sketch Omega.
* ``golden_edge.npz`` -- ragged/edge decode cases (n=7, monomorphic and
  all-missing SNPs, a sample subset) with oracle counts/means/scales.
"""
import json
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

from oracle import lfmm_oracle as O  # noqa: E402
import simdata  # noqa: E402

OUT = Path(__file__).resolve().parent


def kats():
    s2 = math.sqrt(2.0)
    return {
        "decode_missing_imputation": {
            "source": "src/bed.rs:554-572",
            "packed": [0b11100100], "n": 4, "norm": "eigenstrat",
            "expected": [-s2, 0.0, 0.0, s2], "tol": 1e-10},
        "decode_normalization_center_only": {
            "source": "src/bed.rs:575-597",
            "packed": [0b00111000], "n": 3, "norm": "center_only",
            "expected": [-1.0, 0.0, 1.0], "tol": 1e-10},
        "decode_normalization_eigenstrat": {
            "source": "src/bed.rs:599-609",
            "packed": [0b00111000], "n": 3, "norm": "eigenstrat",
            "expected": [-s2, 0.0, s2], "tol": 1e-10},
        "decode_roundtrip_7x3": {
            "source": "src/bed.rs:516-551",
            "genotypes_sample_major": [[0, 1, 2], [2, 0, 1], [1, 1, 0], [0, 2, 2], [2, 1, 0], [1, 0, 1], [0, 0, 2]],
            "norm": "eigenstrat", "tol": 1e-10},
        "safe_inv_pd": {"source": "src/testing.rs:1078-1093",
                        "a": [[2.0, 1.0], [1.0, 3.0]], "tol": 1e-10},
        "safe_inv_singular": {"source": "src/testing.rs:1095-1113",
                              "a": [[1.0, 2.0], [2.0, 4.0]], "eps": 4e-8, "tol": 1e-6},
        "tsq_histogram_gif": {"source": "src/testing.rs:1116-1126",
                              "t": [1.0, 2.0, 3.0, 4.0, 5.0], "expected_gif": 9.0 / 0.4549, "tol": 0.1},
        "calibrate_monotone": {"source": "src/testing.rs:1129-1159",
                               "t": [3.0, -2.0], "gif": 1.0},
        "precompute_small": {"source": "src/precompute.rs:96-157",
                             "x": [[1.0, 0.5], [0.3, -0.2], [-0.5, 1.0], [0.8, 0.1]], "lambda": 1.0, "tol": 1e-10},
        "subset_indices": {"source": "tests/integration.rs:754-778", "cases": [
            {"kind": "all", "n": 10, "expected": list(range(10))},
            {"kind": "rate", "rate": 0.5, "n": 10, "expected": [0, 2, 4, 6, 8]},
            {"kind": "rate", "rate": 0.25, "n": 10, "expected": [0, 4, 8]},
            {"kind": "rate", "rate": 1.0, "n": 10, "expected": list(range(10))},
            {"kind": "rate", "rate": 0.1, "n": 25, "expected": [0, 10, 20]},
            {"kind": "indices", "indices": [3, 7, 11], "n": 100, "expected": [3, 7, 11]}]},
        "subset_count_consistency": {"source": "tests/integration.rs:781-818",
                                     "n": 1000, "rates": [1.0, 0.5, 0.25, 0.1, 0.01],
                                     "indices": [0, 100, 500, 999], "indices_count": 4},
        "covariate_na_imputation": {"source": "src/main.rs:589-641",
                                    "tsv": "sample_id\tenv_0\tenv_1\nIND0\t.\t0.5\nIND1\t1.0\tNA\nIND2\t4.0\t\nIND3\t5.0\t3.5\nIND4\t6.0\t4.5\n",
                                    "expected": [[4.0, 0.5], [1.0, 8.5 / 3.0], [4.0, 8.5 / 3.0], [5.0, 3.5], [6.0, 4.5]],
                                    "tol": 1e-12},
        "validate_results_thresholds": {"source": "tests/integration.rs:506-596",
                                        "mean_cancorr_min": 0.5, "sign_agreement_min": 0.6,
                                        "fpr_max": 0.15, "power_min": 0.1, "gif_range": [0.5, 2.0]},
    }


def golden_c1():
    c = simdata.simulate(200, 10_000, k_pop=2, fst=0.1, miss=0.01, d=1, n_causal=20, effect=0.3, seed=42,
                         f_lo=0.05, f_hi=0.5)
    k, lam, q, os_ = 3, 1e-5, 2, 10
    omega = O.rng_normal_matrix(42, c.n, k + os_)
    st = O.snp_stats(c.raw, O.NORM_EIGENSTRAT)
    fit = O.fit_oracle64(c.raw, c.raw, c.x, k=k, lam=lam, oversampling=os_, power_iter=q, seed=42,
                         norm=O.NORM_EIGENSTRAT, omega=omega)
    a = fit.assoc
    np.savez_compressed(OUT / "golden_c1.npz", packed=c.packed, n=c.n, x=c.x, omega=omega, k=k, lam=lam,
                        power_iter=q, oversampling=os_, counts=st.counts, mean=st.mean, scale=st.scale,
                        tss=st.tss, u_hat=fit.u_hat, beta=a.beta, tstat=a.tstat, pvalue=a.pvalue, r2=a.r2,
                        gif=a.gif, gif_per_trait=a.gif_per_trait, causal=c.causal, b_true=c.b_true,
                        u_true=c.u_true)


def golden_edge():
    rng = np.random.default_rng(7)
    n, p = 7, 37
    g = rng.integers(0, 3, size=(p, n)).astype(np.int16)
    g[0, :] = 2            # monomorphic hom-alt
    g[1, :] = 1            # all het (CenterOnly keeps scale 1, variance 0)
    g[2, :] = 255          # all missing
    g[3, :] = 0
    g[3, 2] = 255          # monomorphic with one missing
    miss = rng.random((p, n)) < 0.1
    g[5:][miss[5:]] = 255
    codes = O.genotypes_to_codes(g)
    packed = O.pack_codes(codes)
    keep = np.array([6, 0, 3, 5], dtype=np.int64)
    out = {"packed": packed, "n": n, "keep": keep}
    for norm, tag in ((O.NORM_CENTER_ONLY, "co"), (O.NORM_EIGENSTRAT, "es")):
        raw = O.decode_raw(packed, n)
        st = O.snp_stats(raw, norm)
        y, _, _ = O.decode_standardized(raw, norm)
        out.update({f"counts": st.counts, f"mean_{tag}": st.mean, f"scale_{tag}": st.scale,
                    f"tss_{tag}": st.tss, f"y_{tag}": y})
        rawk = O.decode_raw(packed, n, keep)
        stk = O.snp_stats(rawk, norm)
        yk, _, _ = O.decode_standardized(rawk, norm)
        out.update({f"counts_keep": stk.counts, f"mean_keep_{tag}": stk.mean, f"scale_keep_{tag}": stk.scale,
                    f"y_keep_{tag}": yk})
    np.savez_compressed(OUT / "golden_edge.npz", **out)


if __name__ == "__main__":
    (OUT / "reference_kats.json").write_text(json.dumps(kats(), indent=1))
    golden_c1()
    golden_edge()
    for f in sorted(OUT.glob("*")):
        print(f.name, f.stat().st_size)
