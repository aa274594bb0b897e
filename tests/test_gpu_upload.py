"""Chunked ingest: the missing-call lists and tile-major copies built chunk by
chunk during an upload, and the sketch pass that slfmm_fit_host runs under the
upload, give the same fit as the resident path and the FP64 oracle.

Upload chunks hold at most 2^18 SNPs, so p = 300 000 makes two chunks."""
import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_fit import _check

pytestmark = pytest.mark.gpu

N, P = 96, 300_000
CHUNK = 1 << 18


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _fields(r):
    return {k: getattr(r, k) for k in ("u_hat", "beta", "tstat", "pvalue", "r2", "gif_per_trait")}


def _same(a, b):
    fa, fb = _fields(a), _fields(b)
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k
    assert a.gif == b.gif


@pytest.fixture(scope="module")
def cohort():
    # 30 covariates: 1 + d + K = 34 columns leave the split-FP8 association
    # pass without an indicator plan, so it reads the missing-call lists
    return simdata.simulate(N, P, k_pop=3, fst=0.05, miss=0.02, d=30, n_causal=30, seed=77)


@pytest.mark.parametrize("prec", ["fp8", "bf16"])
def test_fit_host_equals_resident(engines, cohort, prec):
    """slfmm_fit_host (sketch pass under the upload) == upload + slfmm_fit, bit for bit."""
    sg = _sg()
    eng = engines[prec]
    c = cohort
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(5, c.n, 8)
    host = sg.fit_lfmm2_host(c.packed, c.n, c.x, cfg, omega=omega, engine=eng)
    geno = eng.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, omega=omega, engine=eng)
    _same(host, res)
    if prec == "fp8":
        ref = O.fit_oracle64(c.raw, c.raw, c.x, k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
        _check(res, ref.assoc, ref.u_hat)


def test_fit_host_generated_omega(engine, cohort):
    """The library's own sketch Omega: the same draw in both paths."""
    sg = _sg()
    c = cohort
    cfg = sg.Lfmm2Config(k=3, oversampling=5, seed=11, norm=sg.SnpNorm.EIGENSTRAT)
    host = sg.fit_lfmm2_host(c.packed, c.n, c.x[:, :2], cfg, engine=engine)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x[:, :2], cfg, engine=engine)
    _same(host, res)


def test_chunked_lists_equal_lazy_lists(engine):
    """A device-simulated matrix builds its lists and tiles on first use; the
    same bytes uploaded build them chunk by chunk: identical fits."""
    sg = _sg()
    rng = np.random.default_rng(4)
    q = rng.dirichlet(np.full(3, 0.5), size=N).astype(np.float32)
    sim = engine.simulate(q, P, fst=0.05, f_lo=0.05, f_hi=0.5, miss=0.03, seed=9)
    packed = sim.download()
    up = engine.upload(packed, N)
    x = rng.normal(size=(N, 30))
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(6, N, 8)
    a = sg.fit_lfmm2(sim, sg.SubsetSpec.all(), sim, x, cfg, omega=omega, engine=engine)
    b = sg.fit_lfmm2(up, sg.SubsetSpec.all(), up, x, cfg, omega=omega, engine=engine)
    _same(a, b)


@pytest.mark.parametrize("prec", ["fp8", "bf16"])
def test_lists_overrun_rebuilt(engines, prec):
    """First chunk without missing calls, later chunks with 30 %: the index
    array sized from the first chunk overruns and the lists are rebuilt."""
    sg = _sg()
    c = simdata.simulate(N, P, k_pop=3, fst=0.05, miss=0.0, d=30, n_causal=30, seed=78)
    rng = np.random.default_rng(12)
    codes = c.codes.copy()
    hole = rng.random(codes[CHUNK:].shape) < 0.3
    codes[CHUNK:][hole] = 1                         # PLINK code 01: missing
    packed = O.pack_codes(codes)
    raw = O.DECODE_TABLE[codes].T.copy()
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(7, N, 8)
    res = sg.fit_lfmm2_host(packed, N, c.x, cfg, omega=omega, engine=engines[prec])
    ref = O.fit_oracle64(raw, raw, c.x, k=3, oversampling=5, norm=O.NORM_EIGENSTRAT, omega=omega)
    _check(res, ref.assoc, ref.u_hat)


def _pinned_out(sg, n, p, d, k):
    out, keep = {}, []
    for name, shape in (("u_hat", (n, k)), ("beta", (p, d)), ("tstat", (p, d)), ("pvalue", (p, d)),
                        ("r2", (p, 3)), ("gif_per_trait", (d,))):
        pa = sg.PinnedArray(shape, np.float64)
        out[name] = pa.array
        keep.append(pa)
    return out, keep


@pytest.mark.parametrize("d", [2, 30])
def test_fit_host_pinned_outputs_chunked(engine, cohort, d):
    """Page-locked outputs: the association pass runs in SNP chunks and copies
    beta and r2 while later chunks compute; bit for bit the resident fit.
    d = 30 takes the association pass without the indicator (missing-call
    lists per chunk), d = 2 the indicator form."""
    sg = _sg()
    c = cohort
    x = c.x[:, :d]
    cfg = sg.Lfmm2Config(k=3, oversampling=5, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(5, c.n, 8)
    out, keep = _pinned_out(sg, c.n, c.p, d, 3)
    host = sg.fit_lfmm2_host(c.packed, c.n, x, cfg, omega=omega, engine=engine, out=out)
    geno = engine.upload(c.packed, c.n)
    res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, x, cfg, omega=omega, engine=engine)
    _same(host, res)
    del keep
