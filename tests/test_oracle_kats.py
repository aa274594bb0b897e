"""Pin the CPU oracle against the reference crate's own known answers
(tests/golden/reference_kats.json, transcribed from its unit tests)."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import lfmm_oracle as O

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())
NORMS = {"eigenstrat": O.NORM_EIGENSTRAT, "center_only": O.NORM_CENTER_ONLY}


@pytest.mark.parametrize("name", ["decode_missing_imputation", "decode_normalization_center_only",
                                  "decode_normalization_eigenstrat"])
def test_decode_kats(name):
    k = KATS[name]
    packed = np.array([k["packed"]], dtype=np.uint8)
    raw = O.decode_raw(packed, k["n"])
    y, _, _ = O.decode_standardized(raw, NORMS[k["norm"]])
    np.testing.assert_allclose(y[:, 0], k["expected"], atol=k["tol"], rtol=0)


def test_decode_roundtrip_7x3():
    k = KATS["decode_roundtrip_7x3"]
    g = np.array(k["genotypes_sample_major"], dtype=np.int16)       # (n, p)
    packed = O.pack_codes(O.genotypes_to_codes(g.T))
    assert packed.shape == (3, 2)                                   # ceil(7/4) bytes, padded
    raw = O.decode_raw(packed, 7)
    np.testing.assert_array_equal(raw, g.astype(float))
    y, mean, scale = O.decode_standardized(raw, O.NORM_EIGENSTRAT)
    for snp in range(3):
        col = g[:, snp].astype(float)
        mu = col.sum() / 7
        af = mu / 2
        sc = 1 / math.sqrt(2 * af * (1 - af))
        np.testing.assert_allclose(y[:, snp], (col - mu) * sc, atol=k["tol"])


def test_snp_stats_match_decode():
    rng = np.random.default_rng(3)
    g = rng.integers(0, 3, size=(50, 33)).astype(np.int16)
    g[rng.random(g.shape) < 0.1] = 255
    packed = O.pack_codes(O.genotypes_to_codes(g))
    raw = O.decode_raw(packed, 33)
    for norm in (O.NORM_CENTER_ONLY, O.NORM_EIGENSTRAT):
        st = O.snp_stats(raw, norm)
        y, mean, scale = O.decode_standardized(raw, norm)
        # the mean of 0/1/2 over observed calls is exact, so bit-identical
        np.testing.assert_array_equal(st.mean, mean)
        np.testing.assert_array_equal(st.scale, scale)
        np.testing.assert_allclose(st.tss, (y * y).sum(axis=0), rtol=1e-12, atol=1e-12)
        assert (st.counts.sum(axis=1) == 33).all()


def test_safe_inv_kats():
    k = KATS["safe_inv_pd"]
    a = np.array(k["a"])
    inv, reg = O.safe_inv(a)
    assert not reg
    np.testing.assert_allclose(a @ inv, np.eye(2), atol=k["tol"])
    k = KATS["safe_inv_singular"]
    a = np.array(k["a"])
    inv, reg = O.safe_inv(a)
    assert reg
    np.testing.assert_allclose((a + k["eps"] * np.eye(2)) @ inv, np.eye(2), atol=k["tol"])


def test_histogram_gif_kat():
    k = KATS["tsq_histogram_gif"]
    h = O.TsqHistogram(1)
    h.add_chunk(np.array(k["t"])[:, None])
    gif, avg = h.compute_gif()
    assert abs(gif[0] - k["expected_gif"]) < k["tol"]
    # exact binned value: t^2 = 9 -> bin floor(9/0.001) = 9000, centre 9.0005
    assert gif[0] == pytest.approx(9.0005 / 0.4549, rel=0, abs=1e-12)


def test_histogram_even_median_walks_empty_bins():
    h = O.TsqHistogram(1)
    h.add_chunk(np.sqrt(np.array([0.0005, 0.0015, 1.0005, 5.0005]))[:, None])
    # middle elements are in bins 1 and 1000 -> mean of centres
    assert h.median_for_trait(0) == pytest.approx(((1 + 0.5) * 0.001 + (1000 + 0.5) * 0.001) / 2)
    h2 = O.TsqHistogram(1)
    h2.add_chunk(np.zeros((4, 1)))
    assert h2.compute_gif()[0][0] == 1.0      # median < 1e-10 -> GIF 1
    h3 = O.TsqHistogram(1)
    h3.add_chunk(np.array([[np.inf], [1e6]]))
    assert h3.total[0] == 1 and h3.counts[0, -1] == 1   # non-finite skipped, clamp to last bin


def test_calibrate_monotone_kat():
    k = KATS["calibrate_monotone"]
    p = O.calibrate_p(np.array(k["t"])[:, None], np.array([k["gif"]]))
    assert p[0, 0] < p[1, 0]
    assert O.calibrate_p(np.zeros((1, 1)), np.array([1.0]))[0, 0] == 1.0


def test_precompute_kat():
    k = KATS["precompute_small"]
    x = np.array(k["x"])
    pre = O.precompute_full(x, k["lambda"])
    np.testing.assert_allclose(pre.q_full.T @ pre.q_full, np.eye(4), atol=k["tol"])
    assert 0 < pre.d_lambda[0] < 1 and 0 < pre.d_lambda[1] < 1
    np.testing.assert_allclose(pre.d_lambda[2:], 1.0, atol=k["tol"])
    s = np.linalg.svd(x, compute_uv=False)
    np.testing.assert_allclose(pre.d_lambda[:2] ** 2, k["lambda"] / (k["lambda"] + s ** 2), atol=k["tol"])
    np.testing.assert_allclose(pre.d_lambda * pre.d_lambda_inv, 1.0, atol=k["tol"])
    np.testing.assert_allclose((x.T @ x + k["lambda"] * np.eye(2)) @ pre.ridge_inv, np.eye(2), atol=k["tol"])
    with pytest.raises(ValueError):
        O.precompute_full(x, 0.0)


def test_subset_kats():
    for case in KATS["subset_indices"]["cases"]:
        if case["kind"] == "all":
            got = O.subset_indices(case["n"])
        elif case["kind"] == "rate":
            got = O.subset_indices(case["n"], rate=case["rate"])
        else:
            got = O.subset_indices(case["n"], indices=case["indices"])
        assert list(got) == case["expected"]
    k = KATS["subset_count_consistency"]
    for r in k["rates"]:
        assert O.subset_snp_count(k["n"], rate=r) == len(O.subset_indices(k["n"], rate=r))
    assert O.subset_snp_count(k["n"], indices=k["indices"]) == k["indices_count"]


def test_center_covariates_scale():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(20, 3)) * [1, 5, 0]
    xs = O.center_covariates(x, False)
    np.testing.assert_allclose(xs.mean(axis=0), 0, atol=1e-12)
    xsc = O.center_covariates(x, True)
    np.testing.assert_allclose(xsc[:, :2].std(axis=0, ddof=1), 1, atol=1e-12)
    np.testing.assert_array_equal(xsc[:, 2], 0.0)      # sd <= 1e-14 left unscaled


def test_df_check():
    with pytest.raises(ValueError, match="Insufficient degrees of freedom"):
        O.check_df(5, 2, 2)
    assert O.check_df(10, 2, 2) == 5.0


def test_rust_exp_format():
    assert O.rust_lower_exp6(1.23456e-4) == "1.234560e-4"
    assert O.rust_lower_exp6(0.0) == "0.000000e0"
    assert O.rust_lower_exp6(-150.0) == "-1.500000e2"
    assert O.rust_lower_exp6(float("nan")) == "NaN"
    assert O.rust_lower_exp6(float("inf")) == "inf"
    assert O.rust_lower_exp6(-float("inf")) == "-inf"
    assert O.rust_lower_exp6(1e300) == "1.000000e300"


def test_rng_stream_definition():
    # SplitMix64 reference values for seed 0: the first outputs of the
    # canonical generator started at state mix(0 + gamma)
    u = O.rng_u64(0, np.arange(3, dtype=np.uint64))
    assert u.dtype == np.uint64 and len(set(u.tolist())) == 3
    z = O.rng_normal_matrix(42, 2000, 5)
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1) < 0.05
    np.testing.assert_array_equal(z, O.rng_normal_matrix(42, 2000, 5))


# RFC 8439 s2.3.2: ChaCha20 block function, key 00 01 .. 1f, nonce
# 00 00 00 09 00 00 00 4a 00 00 00 00, block count 1 -> output state words.
RFC8439_BLOCK_OUT = [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3, 0xC7F4D1C7, 0x0368C033, 0x9AAA2204,
                     0x4E6CD4C3, 0x466482D2, 0x09AA9F07, 0x05D7C214, 0xA2028BD9, 0xD19C12B5, 0xB94E16DE,
                     0xE883D0CB, 0x4E3C50A2]


def test_chacha_block_rfc8439():
    st = np.zeros((2, 16), dtype=np.uint32)
    st[:, :4] = O._CHACHA_CONST
    st[:, 4:12] = np.frombuffer(bytes(range(32)), dtype="<u4")
    st[:, 12] = [1, 2]
    st[:, 13], st[:, 14] = 0x09000000, 0x4A000000
    out = O.chacha_blocks(st, 20)
    assert out[0].tolist() == RFC8439_BLOCK_OUT
    assert out[1].tolist() != RFC8439_BLOCK_OUT


def test_chacha8_stream_layout():
    """Consecutive 64-bit outputs, blocks in counter order: any split of the
    stream at a block boundary concatenates back; the key depends on the seed."""
    a = O.chacha8_u64(42, 40)
    np.testing.assert_array_equal(a, np.concatenate([O.chacha8_u64(42, 16, 0), O.chacha8_u64(42, 24, 2)]))
    assert O.pcg32_seed_words(42) != O.pcg32_seed_words(43)
    assert not np.array_equal(a, O.chacha8_u64(43, 40))
    assert len(set(O.pcg32_seed_words(0))) == 8       # seed 0 still gives a full key


def test_ziggurat_tables_consistent():
    """(R, V) of the 256-strip ziggurat: V is the base strip's area
    R f(R) + int_R^inf f, and the recursion closes at the top strip
    (V / x_255 + f(x_255) = f(0) = 1)."""
    from scipy.special import erfc
    x, f = O.ziggurat_tables()
    r = O.ZIG_R
    tail = math.sqrt(math.pi / 2.0) * erfc(r / math.sqrt(2.0))
    assert r * math.exp(-r * r / 2.0) + tail == pytest.approx(O.ZIG_V, rel=1e-11)
    assert O.ZIG_V / x[255] + f[255] == pytest.approx(1.0, abs=1e-9)
    assert all(x[i] > x[i + 1] for i in range(256)) and x[256] == 0.0 and f[256] == 1.0
    for i in range(1, 255):                           # every strip has area V
        assert x[i] * (f[i + 1] - f[i]) == pytest.approx(O.ZIG_V, rel=1e-9)


def test_chacha8_normal_matrix():
    stats = {}
    z = O.chacha8_normal_matrix(42, 4000, 25, stats)
    assert abs(z.mean()) < 0.02 and abs(z.std() - 1.0) < 0.02
    assert stats["tails"] > 0 and stats["wedges"] > 0   # both fall-back branches taken
    assert np.abs(z).max() > O.ZIG_R                    # tail draws beyond R
    # row-major draw order: fewer rows is a prefix of the same stream
    np.testing.assert_array_equal(O.chacha8_normal_matrix(42, 7, 25), z[:7])
    np.testing.assert_array_equal(O.chacha8_normal_matrix(42, 4000, 25), z)
    assert not np.array_equal(O.chacha8_normal_matrix(43, 7, 25), z[:7])
    np.testing.assert_array_equal(O.sketch_normal("chacha8", 5, 3, 4), O.chacha8_normal_matrix(5, 3, 4))
    np.testing.assert_array_equal(O.sketch_normal("counter", 5, 3, 4), O.rng_normal_matrix(5, 3, 4))


def test_mask_uniform_streams():
    """Hold-out uniforms: the ChaCha8 stream's Uniform(0, 1) is the top 52
    bits of each output (rand_distr's [1, 2) mantissa minus 1); the counter
    stream's the top 53; both hold out about `rate` of the calls."""
    ctr = np.arange(200_000, dtype=np.uint64)
    u = O.mask_uniform("chacha8", 7, ctr)
    np.testing.assert_array_equal(u, (O.chacha8_u64(7, 200_000) >> np.uint64(12)).astype(np.float64) * 2.0 ** -52)
    np.testing.assert_array_equal(O.mask_uniform("chacha8", 7, ctr[[5, 3, 99]]), u[[5, 3, 99]])
    assert abs((u < 0.01).mean() - 0.01) < 1e-3 and u.min() >= 0.0 and u.max() < 1.0
    c = O.mask_uniform("counter", 7, ctr)
    np.testing.assert_array_equal(c, O.rng_uniform(7, ctr))
    assert abs((c < 0.01).mean() - 0.01) < 1e-3
    assert O.mask_uniform("chacha8", 7, np.zeros(0, dtype=np.uint64)).size == 0
