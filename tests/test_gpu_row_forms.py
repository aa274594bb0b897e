"""The two forms of a split-FP8 SNP-row pass: the missing-call indicator
operand inside the tensor-core kernel, and the sparse per-SNP fix over the
missing-call lists after it.  The library picks the form by sample count and
missing-call density (the indicator below 8192 samples, so these small cases
would all take it); SLFMM_TC8_ROW_IND forces either form, and both must
match the FP64 oracle.  The paths that have to give the same bits as the
resident fit -- the sketch pass under the upload and the per-trait subsets
built from the tiles, whose missing-call lists then come from the tiles --
must do so in the sparse form too.  The sparse form is also checked on
ragged sample and SNP counts, on SNPs with most or all of their calls
missing, and on the split-BF16 engine, whose row passes take the same fix."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_fit import _check
from test_gpu_upload import _same
from test_gpu_batch import _traits

pytestmark = pytest.mark.gpu


def _sg():
    import schnellfmm_gb300 as sg
    return sg


@pytest.mark.parametrize("form", ["1", "0"])
def test_row_forms_match_oracle(engine, monkeypatch, form):
    sg = _sg()
    monkeypatch.setenv("SLFMM_TC8_ROW_IND", form)
    c = simdata.simulate(700, 5000, k_pop=3, fst=0.08, miss=0.04, d=3, n_causal=20, seed=61)
    cfg = sg.Lfmm2Config(k=4, oversampling=6, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(9, c.n, 10)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engine)
    ref = O.fit_oracle64(c.raw, c.raw, c.x, k=4, oversampling=6, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)
    geno.free()


def _heavy(c, rows, frac, seed):
    """Packed codes and raw values of cohort c with a share `frac` of the
    calls of SNPs `rows` made missing."""
    rng = np.random.default_rng(seed)
    codes = c.codes.copy()
    for j in rows:
        codes[j, rng.random(c.n) < frac] = 1
    return O.pack_codes(codes), O.DECODE_TABLE[codes].T.copy()


@pytest.mark.parametrize("shape", [(700, 3001), (2000, 2500), (1537, 1800)])
def test_sparse_fix_edges_match_oracle(engines, monkeypatch, shape):
    sg = _sg()
    monkeypatch.setenv("SLFMM_TC8_ROW_IND", "0")
    n, p = shape
    c = simdata.simulate(n, p, k_pop=3, fst=0.08, miss=0.02, d=2, n_causal=15, seed=64)
    # SNPs with 60 % of their calls missing, and one with all of them
    packed, raw = _heavy(c, [0, 5, 767, 768, p - 1], 0.6, 65)
    packed[3] = O.pack_codes(np.ones((1, n), np.uint8))[0]
    raw[:, 3] = np.nan
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(11, n, 8)
    ref = O.fit_oracle64(raw, raw, c.x, k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    for prec in ("fp8", "bf16"):
        eng = engines[prec]
        geno = eng.upload(packed, n)
        res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=eng)
        _check(res, ref.assoc, ref.u_hat)
        geno.free()


def test_sparse_form_fit_host_equals_resident(engine, monkeypatch):
    """The sketch pass under the upload leaves the missing-call fix until the
    upload's lists are complete; the result equals the resident fit bit for bit."""
    sg = _sg()
    monkeypatch.setenv("SLFMM_TC8_ROW_IND", "0")
    c = simdata.simulate(300, 300_000, k_pop=3, fst=0.05, miss=0.02, d=2, n_causal=30, seed=62)
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(5, c.n, 8)
    host = sg.fit_lfmm2_host(c.packed, c.n, c.x, cfg, omega=omega, engine=engine)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=engine)
    _same(host, res)
    geno.free()


def test_sparse_form_traits_equal_subset_fits(engine, monkeypatch):
    """Per-trait matrices held only as tiles take their missing-call lists
    from the tiles (k_miss_fill_tiles): bit for bit the fits on uploads
    restricted to each trait's samples, whose lists come from the packed rows."""
    sg = _sg()
    monkeypatch.setenv("SLFMM_TC8_ROW_IND", "0")
    c = simdata.simulate(400, 6000, k_pop=3, fst=0.08, miss=0.03, d=1, seed=63)
    y, masks = _traits(c.n, 3, 7)
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2_traits(geno, y, masks, cfg, engine=engine)
    for t in range(3):
        keep = np.flatnonzero(masks[:, t])
        sub = engine.upload(c.packed, c.n, sample_keep=keep)
        ref = sg.fit_lfmm2(sub, sg.SubsetSpec.all(), sub, y[keep, t:t + 1], cfg, engine=engine)
        _same(res[t], ref)
        sub.free()
    geno.free()
