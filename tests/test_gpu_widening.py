"""The FP64 outputs the association pass forms from FP32 values -- t, beta
and, below |z| = 8, the p-values -- are those FP32 values widened exactly.
The kernels widen by moving the IEEE-754 fields with integer operations
(the conversion instruction runs on the FP64 pipe, a small fraction of the
FP32 rate on this part); a wrong field placement would leave low-order bits
set or scale the value, which the round trip through FP32 catches, and the
oracle comparison bounds the values themselves.  Both the single pass and
the chunked pass with page-locked outputs are covered, with zero-variance
SNPs (beta and t exactly 0)."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_fit import _check
from test_gpu_upload import _pinned_out

pytestmark = pytest.mark.gpu


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _exact_f32(x):
    return np.array_equal(x.astype(np.float32).astype(np.float64), x)


def _check_widened(res):
    assert _exact_f32(res.tstat)
    assert _exact_f32(res.beta)
    z = np.abs(res.tstat) / np.sqrt(res.gif_per_trait)[None, :]
    # below |z| = 8 the p-value is erfcf of the FP32 statistic, widened
    assert _exact_f32(res.pvalue[z < 7.9])
    assert np.all(np.isfinite(res.pvalue)) and np.all((res.pvalue >= 0) & (res.pvalue <= 1))


def _cohort():
    c = simdata.simulate(600, 4000, k_pop=3, fst=0.1, miss=0.03, d=3, n_causal=40, effect=0.8, seed=71,
                         monomorphic=5)
    return c


def test_widening_single_pass(engine):
    sg = _sg()
    c = _cohort()
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(13, c.n, 8)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engine)
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)
    _check_widened(res)
    assert np.all(res.tstat[:5] == 0.0) and np.all(res.beta[:5] == 0.0)   # the monomorphic SNPs
    geno.free()


def test_widening_chunked_pinned(engine):
    sg = _sg()
    c = _cohort()
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(13, c.n, 8)
    out, keep = _pinned_out(sg, c.n, c.p, c.x.shape[1], 3)
    res = sg.fit_lfmm2_host(c.packed, c.n, c.x, cfg, omega=omega, engine=engine, out=out)
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)
    _check_widened(res)
    del keep
