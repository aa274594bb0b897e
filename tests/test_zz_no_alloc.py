"""slfmm_gif_noalloc (the allocation-free entry point) against the GIF the
full fit computes from the same FP32 t statistics, on two calls in a row
(the shared static histogram must be re-zeroed by each call)."""
import ctypes as C

import numpy as np
import pytest

import simdata

pytestmark = pytest.mark.gpu


def test_gif_noalloc_matches_fit():
    torch = pytest.importorskip("torch")
    import schnellfmm_gb300 as sg
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8)
    try:
        c = simdata.simulate(400, 3000, k_pop=3, fst=0.1, miss=0.02, d=3, n_causal=20, seed=77)
        geno = eng.upload(c.packed, c.n)
        cfg = sg.Lfmm2Config(k=3, lambda_=1e-5)
        res = sg.fit_lfmm2(geno, sg.SubsetSpec.all(), geno, c.x, cfg, engine=eng)
        p, d = res.tstat.shape
        # the fit's t statistics are FP32 values widened to double: narrowing is exact
        t32 = torch.tensor(np.ascontiguousarray(res.tstat.astype(np.float32)), device="cuda")
        out = torch.empty(d, dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(-1.0)
            torch.cuda.synchronize()
            eng.check(eng.lib.slfmm_gif_noalloc(eng.h, C.c_void_p(t32.data_ptr()), p, d,
                                                C.c_void_p(out.data_ptr())))
            torch.cuda.synchronize()
            raw = out.cpu().numpy()
            np.testing.assert_allclose(np.maximum(raw, 1.0), res.gif_per_trait, rtol=1e-12, atol=0.0)
            assert abs(raw.mean() - res.gif) <= 1e-12 * max(1.0, abs(res.gif))
        # beyond the static histogram's 8 traits: a clear error, nothing launched
        rc = eng.lib.slfmm_gif_noalloc(eng.h, C.c_void_p(t32.data_ptr()), p // 9, 9, C.c_void_p(out.data_ptr()))
        assert rc == sg.ERR_BAD_ARG
        assert b"at most 8 traits" in eng.lib.slfmm_last_error(eng.h)
        geno.free()
    finally:
        eng.close()


def test_gif_noalloc_matches_oracle_histogram():
    """Eight traits (the static histogram's limit) with non-finite t values,
    which the reference's histogram skips (src/testing.rs:135-149), against
    the oracle's TsqHistogram on the same FP32 t; an empty t gives GIF 1."""
    torch = pytest.importorskip("torch")
    import schnellfmm_gb300 as sg
    from oracle import lfmm_oracle as O
    eng = sg.Engine(precision=sg.Precision.SPLIT_FP8)
    try:
        rng = np.random.default_rng(5)
        p, d = 50_001, 8
        t = (rng.standard_normal((p, d)) * rng.uniform(0.8, 1.6, size=d)).astype(np.float32)
        t[rng.integers(0, p, 40), rng.integers(0, d, 40)] = np.nan
        t[rng.integers(0, p, 40), rng.integers(0, d, 40)] = np.inf
        t[rng.integers(0, p, 40), rng.integers(0, d, 40)] = -np.inf
        t[:7, 3] = 1e20                       # t^2 finite in FP64: counted in the last bin
        t[7:200, 5] = np.sqrt(np.float32(1.0005))  # t^2 next to a bin edge
        hist = O.TsqHistogram(d)
        hist.add_chunk(t.astype(np.float64))
        gif_clamped, _ = hist.compute_gif()
        raw_ref = np.array([1.0 if hist.median_for_trait(j) < 1e-10 else hist.median_for_trait(j) / O.GIF_DIVISOR
                            for j in range(d)])
        assert np.all(gif_clamped == np.maximum(raw_ref, 1.0))
        t_dev = torch.tensor(t, device="cuda")
        out = torch.empty(d, dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(-1.0)
            torch.cuda.synchronize()
            eng.check(eng.lib.slfmm_gif_noalloc(eng.h, C.c_void_p(t_dev.data_ptr()), p, d,
                                                C.c_void_p(out.data_ptr())))
            torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), raw_ref, rtol=1e-15, atol=0.0)
        # no SNPs: every median is 0, so every GIF is 1
        eng.check(eng.lib.slfmm_gif_noalloc(eng.h, None, 0, d, C.c_void_p(out.data_ptr())))
        torch.cuda.synchronize()
        assert np.all(out.cpu().numpy() == 1.0)
        # a trait count beyond uint32 -> int narrowing still reports the caller's value
        rc = eng.lib.slfmm_gif_noalloc(eng.h, C.c_void_p(t_dev.data_ptr()), 1, 0xFFFFFFFF,
                                       C.c_void_p(out.data_ptr()))
        assert rc == sg.ERR_BAD_ARG and b"got 4294967295" in eng.lib.slfmm_last_error(eng.h)
    finally:
        eng.close()
