"""The autotuner times the tensor-core ring depths once per shape and keeps
the fastest; it only touches knobs that leave the arithmetic alone, so a
tuned context gives the same bits as the default one."""
import pytest

from oracle import lfmm_oracle as O
import simdata
from test_gpu_upload import _same

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("d", [2, 30])
def test_autotuned_fit_is_bit_identical(engine, d):
    import schnellfmm_gb300 as sg
    c = simdata.simulate(600, 8000, k_pop=3, fst=0.05, miss=0.01, d=d, seed=41)
    cfg = sg.Lfmm2Config(k=4, oversampling=6, norm=sg.SnpNorm.EIGENSTRAT)
    omega = O.rng_normal_matrix(3, c.n, 10)
    tuned = sg.Engine(precision=sg.Precision.SPLIT_FP8, autotune=True)
    try:
        gt = tuned.upload(c.packed, c.n)
        a = sg.fit_lfmm2(gt, sg.SubsetSpec.all(), gt, c.x, cfg, omega=omega, engine=tuned)
        b_geno = engine.upload(c.packed, c.n)
        b = sg.fit_lfmm2(b_geno, sg.SubsetSpec.all(), b_geno, c.x, cfg, omega=omega, engine=engine)
        _same(a, b)
        # a second tuned fit reuses the cached choices
        a2 = sg.fit_lfmm2(gt, sg.SubsetSpec.all(), gt, c.x, cfg, omega=omega, engine=tuned)
        _same(a2, b)
    finally:
        tuned.close()
