"""Stage (a) on the GPU: allele counts, mean and scale must be bit-exact with
the oracle (src/bed.rs:300-395); the standardised decode too."""
from pathlib import Path

import numpy as np
import pytest

from oracle import lfmm_oracle as O
import simdata

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).parent / "golden"


def _sg():
    import schnellfmm_gb300 as sg
    return sg


@pytest.mark.parametrize("norm,tag", [(0, "co"), (1, "es")])
def test_edge_cases_bit_exact(engine, norm, tag):
    g = np.load(GOLD / "golden_edge.npz")
    geno = engine.upload(g["packed"], int(g["n"]))
    counts, mean, scale, tss = geno.decode_stats(norm)
    np.testing.assert_array_equal(counts, g["counts"])
    np.testing.assert_array_equal(mean, g[f"mean_{tag}"])
    np.testing.assert_array_equal(scale, g[f"scale_{tag}"])
    np.testing.assert_allclose(tss, g[f"tss_{tag}"], rtol=1e-13, atol=1e-13)
    y = geno.decode_chunk(0, geno.n_snps, norm)
    np.testing.assert_array_equal(y, g[f"y_{tag}"])
    gk = engine.upload(g["packed"], int(g["n"]), sample_keep=g["keep"])
    counts, mean, scale, _ = gk.decode_stats(norm)
    np.testing.assert_array_equal(counts, g["counts_keep"])
    np.testing.assert_array_equal(mean, g[f"mean_keep_{tag}"])
    np.testing.assert_array_equal(scale, g[f"scale_keep_{tag}"])
    np.testing.assert_array_equal(gk.decode_chunk(0, gk.n_snps, norm), g[f"y_keep_{tag}"])


@pytest.mark.parametrize("n", [1, 4, 5, 127, 1001, 2049])
def test_counts_random_sizes(engine, n):
    c = simdata.simulate(n, 300, miss=0.05, seed=n)
    geno = engine.upload(c.packed, n)
    counts, mean, scale, tss = geno.decode_stats(1)
    st = O.snp_stats(c.raw, O.NORM_EIGENSTRAT)
    np.testing.assert_array_equal(counts, st.counts)
    np.testing.assert_array_equal(mean, st.mean)
    np.testing.assert_array_equal(scale, st.scale)
    np.testing.assert_allclose(tss, st.tss, rtol=1e-12, atol=1e-12)


def test_snp_subsets_and_sample_keep(engine):
    sg = _sg()
    c = simdata.simulate(333, 1000, miss=0.02, seed=9)
    keep = np.random.default_rng(1).permutation(333)[:200]
    for spec, idx in [(sg.SubsetSpec.from_rate(0.1), O.subset_indices(1000, rate=0.1)),
                      (sg.SubsetSpec.from_rate(0.37), O.subset_indices(1000, rate=0.37)),
                      (sg.SubsetSpec.from_indices([999, 3, 4, 5, 500]), np.array([999, 3, 4, 5, 500]))]:
        geno = engine.upload(c.packed, 333, sample_keep=keep, snps=spec)
        assert geno.n_snps == len(idx) and geno.n_samples == 200
        counts, mean, scale, _ = geno.decode_stats(1)
        raw = O.decode_raw(c.packed[idx], 333, keep)
        st = O.snp_stats(raw, 1)
        np.testing.assert_array_equal(counts, st.counts)
        np.testing.assert_array_equal(mean, st.mean)
        np.testing.assert_array_equal(scale, st.scale)


def test_upload_large_chunked(engine):
    """More rows than one 64 MiB staging chunk: exercises the double-buffered ring."""
    n, p = 4096, 70_000          # 1024 B/SNP -> ~68 MB, two chunks
    rng = np.random.default_rng(2)
    packed = rng.integers(0, 256, size=(p, n // 4), dtype=np.uint8)
    geno = engine.upload(packed, n)
    counts, mean, _, _ = geno.decode_stats(0)
    codes = O.unpack_codes(packed[-50:], n)
    np.testing.assert_array_equal(counts[-50:, 3], (codes == 1).sum(axis=1))
    np.testing.assert_array_equal(counts[:, :3].sum(axis=1) + counts[:, 3], n)


def test_bad_arguments(engine):
    sg = _sg()
    c = simdata.simulate(20, 10, seed=1)
    with pytest.raises(sg.SchnelGpuError):
        engine.upload(c.packed, 20, sample_keep=[0, 25])
    with pytest.raises(sg.SchnelGpuError):
        engine.upload(c.packed, 20, snps=sg.SubsetSpec.from_indices([10]))


def test_decode_chunk_rejects_bad_ranges(engine):
    """A SNP range past the end (also one whose end overflows 64 bits) and an
    unknown normalisation are argument errors, not device accesses."""
    sg = _sg()
    c = simdata.simulate(40, 50, seed=5)
    geno = engine.upload(c.packed, 40)
    np.testing.assert_array_equal(geno.decode_chunk(45, 5, 1), geno.decode_chunk(0, 50, 1)[:, 45:])
    for snp0, ncols in [(45, 6), (51, 0), (2**64 - 2, 3)]:
        with pytest.raises(sg.SchnelGpuError) as e:
            geno.decode_chunk(snp0, ncols, 1)
        assert e.value.code == sg.ERR_BAD_ARG
    with pytest.raises(sg.SchnelGpuError) as e:
        geno.decode_chunk(0, 5, 7)
    assert e.value.code == sg.ERR_BAD_ARG
