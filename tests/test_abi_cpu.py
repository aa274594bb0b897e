"""The C-ABI library on a machine without a GPU: it builds, loads, exports
every entry point the header declares, its host-only entry points (number
formatting, TSV and Parquet writers, .bed validation, the reference's sketch
stream) match the oracle or an independent reader, and every call that needs the device fails loudly instead of
falling back to the CPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from oracle import lfmm_oracle as O

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "schnelgpu.h"


@pytest.fixture(scope="module")
def lib():
    from schnellfmm_gb300 import build
    build.build()
    import schnellfmm_gb300 as sg
    return sg.load_library()


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(slfmm_\w+)\s*\(", text)))


def test_header_entry_points_exported(lib):
    import schnellfmm_gb300 as sg
    names = _declared()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), f"{name} declared in schnelgpu.h but not exported"
    assert sorted(sg.EXPORTED_SYMBOLS) == names


@pytest.mark.parametrize("v", [0.0, -0.0, 1.0, 1.23456e-4, -9.87654321e123, 1e-300, 2.5e-320,
                               123456789.0, 0.1, float("nan"), float("inf"), -float("inf"), 9.9999996e-5])
def test_format_exp6_matches_rust(lib, v):
    import schnellfmm_gb300 as sg
    assert sg.format_exp6(v) == O.rust_lower_exp6(v)


def test_write_tsv_matches_oracle(lib, tmp_path):
    import schnellfmm_gb300 as sg
    rng = np.random.default_rng(5)
    p, d = 57, 3
    res = sg.TestResults(u_hat=np.zeros((4, 2)), gif=1.0, gif_per_trait=np.ones(d),
                         beta=rng.standard_normal((p, d)), tstat=rng.standard_normal((p, d)) * 3,
                         pvalue=rng.uniform(1e-12, 1, (p, d)), r2=rng.uniform(0, 1, (p, 3)))
    res.pvalue[0, 0] = np.nan
    res.beta[1, 1] = 0.0
    bim = [sg.BimRecord(str(1 + i // 20), f"rs{i}", 0.0, 1000 + 7 * i, "A", "G") for i in range(p)]
    names = ["temp", "prec", "alt"]
    out = tmp_path / "res.tsv"
    sg.write_tsv(out, bim, names, res, n_threads=3)
    ref = O.AssocResults(beta=res.beta, tstat=res.tstat, pvalue=res.pvalue, r2=res.r2,
                         gif=res.gif, gif_per_trait=res.gif_per_trait)
    rows = O.tsv_rows([b.chrom for b in bim], [b.pos for b in bim], [b.snp_id for b in bim], ref)
    want = O.tsv_header(names) + "\n" + "".join(r + "\n" for r in rows)
    assert out.read_text() == want


def _results(sg, p, d, seed):
    rng = np.random.default_rng(seed)
    res = sg.TestResults(u_hat=np.zeros((4, 2)), gif=1.0, gif_per_trait=np.ones(d),
                         beta=rng.standard_normal((p, d)), tstat=rng.standard_normal((p, d)) * 3,
                         pvalue=rng.uniform(1e-12, 1, (p, d)), r2=rng.uniform(0, 1, (p, 3)))
    if p and d:
        res.pvalue[0, 0] = np.nan
        res.beta[-1, -1] = -0.0
    bim = [sg.BimRecord(str(1 + i // 20), f"rs{i}_\u00e9", 0.0, 1000 + 7 * i, "A", "G") for i in range(p)]
    return res, bim


@pytest.mark.parametrize("p,d", [(57, 3), (300_000, 2), (0, 1), (9, 0)])
@pytest.mark.parametrize("codec", ["zstd", "none"])
def test_write_parquet_reads_back(lib, tmp_path, p, d, codec):
    """<out>.parquet (coalesce_output_parquet, src/testing.rs:818-983) read
    back by an independent Parquet reader: the calibrated schema
    (src/testing.rs:620-640) with every field required, the values bit for
    bit, row groups of 2^18 rows, the requested codec."""
    pq = pytest.importorskip("pyarrow.parquet")
    import schnellfmm_gb300 as sg
    res, bim = _results(sg, p, d, 11)
    names = [f"cov{j}" for j in range(d)]
    out = tmp_path / "res.parquet"
    sg.write_parquet(out, bim, names, res, compression=sg.PARQUET_ZSTD if codec == "zstd" else sg.PARQUET_UNCOMPRESSED,
                     n_threads=3)
    f = pq.ParquetFile(out)
    tab = f.read()
    want = (["chr", "pos", "snp_id"] + [f"p_{n}" for n in names] + [f"beta_{n}" for n in names]
            + [f"t_{n}" for n in names] + ["r2_cov", "r2_latent", "r2_resid"])
    assert tab.column_names == want and tab.num_rows == p
    assert all(not fld.nullable for fld in tab.schema)
    assert str(tab.schema.field("chr").type) == "string" and str(tab.schema.field("pos").type) == "int64"
    assert f.metadata.num_row_groups == -(-p // (1 << 18))
    if p:
        assert f.metadata.row_group(0).column(3).compression == ("ZSTD" if codec == "zstd" else "UNCOMPRESSED")
    assert tab.column("chr").to_pylist() == [b.chrom for b in bim]
    assert tab.column("pos").to_pylist() == [b.pos for b in bim]
    assert tab.column("snp_id").to_pylist() == [b.snp_id for b in bim]
    bits = lambda a: np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)
    for j, n in enumerate(names):
        for pre, arr in (("p_", res.pvalue), ("beta_", res.beta), ("t_", res.tstat)):
            np.testing.assert_array_equal(bits(tab.column(pre + n).to_numpy()), bits(arr[:, j]))
    for k, n in enumerate(["r2_cov", "r2_latent", "r2_resid"]):
        np.testing.assert_array_equal(bits(tab.column(n).to_numpy()), bits(res.r2[:, k]))


def test_write_parquet_bad_args(lib, tmp_path):
    import schnellfmm_gb300 as sg
    res, bim = _results(sg, 5, 1, 2)
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.write_parquet(tmp_path / "x.parquet", bim, ["a"], res, compression=1)   # SNAPPY: not written
    assert e.value.code == sg.ERR_BAD_ARG
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.write_parquet(tmp_path / "x.parquet", bim[:4], ["a"], res)
    assert e.value.code == sg.ERR_BAD_ARG
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.write_parquet(tmp_path / "no_such_dir" / "x.parquet", bim, ["a"], res)
    assert e.value.code == sg.ERR_IO


def _write_bed(path, payload, magic=bytes([0x6C, 0x1B, 0x01])):
    path.write_bytes(magic + payload.tobytes())


def test_bed_validate(lib, tmp_path):
    n, p = 10, 7
    bps = (n + 3) // 4
    payload = np.random.default_rng(1).integers(0, 256, size=(p, bps), dtype=np.uint8)
    good = tmp_path / "good.bed"
    _write_bed(good, payload)
    out = np.zeros(p * bps, dtype=np.uint8)
    err = C.create_string_buffer(256)
    rc = lib.slfmm_bed_validate(str(good).encode(), n, p, out.ctypes.data_as(C.c_void_p), err, 256)
    assert rc == 0
    assert np.array_equal(out.reshape(p, bps), payload)
    bad_magic = tmp_path / "bad_magic.bed"
    _write_bed(bad_magic, payload, magic=bytes([0x6C, 0x1B, 0x00]))
    assert lib.slfmm_bed_validate(str(bad_magic).encode(), n, p, None, err, 256) == -2
    assert b"magic" in err.value.lower() or b"snp-major" in err.value.lower()
    short = tmp_path / "short.bed"
    _write_bed(short, payload[:-1])
    assert lib.slfmm_bed_validate(str(short).encode(), n, p, None, err, 256) == -2
    missing = tmp_path / "nope.bed"
    assert lib.slfmm_bed_validate(str(missing).encode(), n, p, None, err, 256) in (-2, -7)


@pytest.mark.parametrize("seed,rows,cols", [(42, 2000, 30), (1_000_042, 300, 14), (0, 7, 3),
                                             (2**64 - 1, 1, 1), (9, 5, 0)])
def test_reference_normal_matches_oracle(lib, seed, rows, cols):
    """slfmm_reference_normal (ChaCha8Rng::seed_from_u64 + Normal(0, 1), the
    SLFMM_RNG_CHACHA8 stream) equals the oracle's restatement bit for bit;
    the (2000, 30) case takes the tail and wedge branches."""
    import schnellfmm_gb300 as sg
    stats = {}
    ref = O.chacha8_normal_matrix(seed, rows, cols, stats)
    got = sg.reference_normal(seed, rows, cols)
    assert got.shape == (rows, cols)
    np.testing.assert_array_equal(got, ref)
    if rows * cols >= 60_000:
        assert stats["tails"] > 0 and stats["wedges"] > 0


def test_reference_normal_bad_args(lib):
    assert lib.slfmm_reference_normal(1, 4, 4, None) == -1
    assert lib.slfmm_reference_normal(1, 0, 4, None) == 0
    assert lib.slfmm_reference_normal(1, 2**63, 4, C.c_void_p(8)) == -1   # rows x cols overflows


def test_host_array_shapes_checked():
    """Host matrices whose shape does not match the call are argument errors
    before the library is called (it would read them with the implied shape)."""
    import schnellfmm_gb300 as sg
    sg._check_shape("x", np.zeros((5, 2)), 5)
    sg._check_shape("omega", None, 5, 13)
    for a, rows, cols in [(np.zeros(5), 5, None), (np.zeros((4, 2)), 5, None), (np.zeros((5, 12)), 5, 13)]:
        with pytest.raises(sg.SchnelGpuError) as e:
            sg._check_shape("x", a, rows, cols)
        assert e.value.code == sg.ERR_BAD_ARG and "expected" in str(e.value)
    packed, p = sg._payload(np.zeros((7, 3), dtype=np.uint8), 10)
    assert p == 7 and packed.flags.c_contiguous and packed.dtype == np.uint8
    pinned = np.zeros(12, dtype=np.uint8)
    assert sg._payload(pinned, 4)[0].ctypes.data == pinned.ctypes.data   # no copy of a usable payload
    with pytest.raises(sg.SchnelGpuError) as e:
        sg._payload(np.zeros(10, dtype=np.uint8), 10)
    assert e.value.code == sg.ERR_BAD_BED


def test_create_rejects_unknown_rng(lib):
    import schnellfmm_gb300 as sg
    opts = sg._Opts(int(sg.Precision.SPLIT_FP8), 0, None, 0, 7)
    h = C.c_void_p()
    assert lib.slfmm_create(0, C.byref(opts), C.byref(h)) == -1 and not h.value


def test_no_gpu_fails_loudly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import schnellfmm_gb300 as sg
    with pytest.raises(sg.SchnelGpuError):
        sg.Engine()
