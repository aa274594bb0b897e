"""Timed CPU baseline of the reference algorithm -- TEST/BENCH INFRASTRUCTURE.

Runs the faithful n x n restatement of schnelLFMM's CPU path (src/lib.rs
fit_lfmm2: precompute src/precompute.rs:30-88, estimate_factors_streaming
src/rsvd.rs:26-177, test_associations_fused src/testing.rs:252-528) on a
bounded SNP sample of the benchmark workload, timing every stage, and
extrapolates the whole-job wall time to p SNPs:

    T(p) = T_fixed + p * t_snp + ceil(p / chunk) * n_fwd * t_chunk + T_qr(p)

where t_snp is the per-SNP streaming work of all 2q+3 passes, t_chunk the
reference's per-chunk n x n product M (Y Q_z) in each forward pass and T_qr
the Householder QR of the p x l sketches (linear in p).  Only ``bench.py``
calls this, and only for its cpu_baseline leg / reference arm.
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from . import lfmm_oracle as O


def _now():
    return time.perf_counter()


def time_reference_cpu(packed_sample: np.ndarray, n: int, x: np.ndarray, *, k: int, oversampling: int,
                       power_iter: int, lam: float, norm: int, p_total: int, seed: int = 42,
                       chunk: int = 10_000) -> dict:
    t = {}
    s_snps = packed_sample.shape[0]
    t0 = _now()
    raw = O.decode_raw(packed_sample, n)
    y, _, _ = O.decode_standardized(raw, norm)
    t["decode"] = _now() - t0

    t0 = _now()
    xs = O.center_covariates(x, False)
    pre = O.precompute_full(xs, lam)
    t["precompute"] = _now() - t0

    l = k + oversampling
    omega = O.rng_normal_matrix(seed, n, l)
    t0 = _now()
    mt_omega = pre.m.T @ omega
    t["mt_omega"] = _now() - t0

    # streaming passes over the sample (one reference chunk)
    stream = 0.0
    t0 = _now()
    z = y.T @ mt_omega
    stream += _now() - t0
    t0 = _now()
    q_z, _ = np.linalg.qr(z)
    qr_sample = _now() - t0
    t_chunk = 0.0
    for _ in range(power_iter):
        t0 = _now()
        y_qz = y @ q_z
        stream += _now() - t0
        t0 = _now()
        a_qz = pre.m @ y_qz
        t_chunk += _now() - t0
        t0 = _now()
        q_a, _ = np.linalg.qr(a_qz)
        mt_q = pre.m.T @ q_a
        t["mtq"] = t.get("mtq", 0.0) + _now() - t0
        t0 = _now()
        z = y.T @ mt_q
        stream += _now() - t0
        t0 = _now()
        q_z, _ = np.linalg.qr(z)
        qr_sample += _now() - t0
    t0 = _now()
    y_qz = y @ q_z
    stream += _now() - t0
    t0 = _now()
    b = pre.m @ y_qz
    t_chunk += _now() - t0
    t0 = _now()
    u_small, _, _ = np.linalg.svd(b, full_matrices=False)
    u_hat = pre.q_full @ (pre.d_lambda_inv[:, None] * u_small[:, :k])
    t["svd_uhat"] = _now() - t0

    # association pass: n x n OLS-hat precompute, then the per-chunk work
    t0 = _now()
    d = xs.shape[1]
    utu_inv, _ = O.safe_inv(u_hat.T @ u_hat)
    p_u = u_hat @ utu_inv @ u_hat.T
    xtr = pre.ridge_inv @ xs.T
    i_minus_pu = np.eye(n) - p_u
    del p_u
    c = np.hstack([np.ones((n, 1)), xs, u_hat])
    ctc_inv, _ = O.safe_inv(c.T @ c)
    h = ctc_inv @ c.T
    xtx_inv, _ = O.safe_inv(xs.T @ xs)
    hx = xs @ xtx_inv @ xs.T
    t["ols_hat"] = _now() - t0
    t0 = _now()
    bch = xtr @ (i_minus_pu @ y)
    coefs = h @ y
    res = y - c @ coefs
    fx = hx @ y
    rss = np.einsum("ij,ij->j", res, res)
    tss = np.einsum("ij,ij->j", y, y)
    ss_cov = np.einsum("ij,ij->j", fx, fx)
    df = float(n - 1 - d - k)
    tstat, r2 = O._per_snp_stats(y, coefs, rss, ss_cov, tss, np.diag(ctc_inv)[1:1 + d], df, d)
    hist = O.TsqHistogram(d)
    hist.add_chunk(tstat)
    t["test_stream"] = _now() - t0
    t0 = _now()
    gif_pt, _ = hist.compute_gif()
    O.calibrate_p(tstat, gif_pt)
    t["calibrate"] = _now() - t0
    del i_minus_pu, hx

    n_fwd = power_iter + 1
    t_snp = (t["decode"] * (2 * power_iter + 3) + stream + t["test_stream"] + t["calibrate"]) / s_snps
    t_chunk_each = t_chunk / n_fwd
    t_qr = qr_sample / s_snps
    fixed = t["precompute"] + t["mt_omega"] + t.get("mtq", 0.0) + t["svd_uhat"] + t["ols_hat"]
    total = fixed + p_total * (t_snp + t_qr) + math.ceil(p_total / chunk) * n_fwd * t_chunk_each
    return {
        "snps_per_s": p_total / total,
        "extrapolated_total_s": total,
        "sample_snps": s_snps,
        "fixed_s": fixed,
        "per_snp_s": t_snp + t_qr,
        "per_chunk_nxn_s": t_chunk_each,
        "stages_s": {k2: round(v, 4) for k2, v in t.items()},
        "cores": os.cpu_count(),
    }
