"""Parity criteria of a GPU fit against the FP64 oracle, shared by the
GPU tests: U_hat by principal angles, max|dt| <= 1e-3 (the path's stated
tolerance), beta relative to its largest magnitude, r^2, the GIF within one
histogram bin, calibrated p-values and top-hit order."""
import numpy as np

from oracle import lfmm_oracle as O

T_TOL = 1e-3          # max |delta t| vs FP64


def check_fit(res, ref, u_ref, t_tol=T_TOL, top=10):
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
    for j in range(ref.tstat.shape[1]):
        a = np.argsort(-np.abs(ref.tstat[:, j]))[:top]
        b = np.argsort(-np.abs(res.tstat[:, j]))[:top]
        assert set(a[:top // 2]) <= set(b), f"trait {j}: top hits differ"
    return dt
