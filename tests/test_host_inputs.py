"""Host-side input logic: the covariate loader (load_covariates,
src/main.rs:339-571) on the reference's own known answer (its test at
src/main.rs:589-641, restated in tests/golden/reference_kats.json) plus the
delimiter, matching, intersection and error rules of the same function; the
--est-bed sample alignment (src/main.rs:282-331); the PLINK triplet reader
(BedFile::open, src/bed.rs:60-135) and SNP subset counts."""
import json
from pathlib import Path

import numpy as np
import pytest

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _sg():
    import schnellfmm_gb300 as sg
    return sg


def _fam(sg, iids):
    return [sg.FamRecord("FAM", iid, "0", "0", 0, "-9") for iid in iids]


def test_covariate_na_imputation_kat(tmp_path):
    sg = _sg()
    k = KATS["covariate_na_imputation"]
    path = tmp_path / "cov.tsv"
    path.write_text(k["tsv"])
    names, x, kept = sg.load_covariates(path, _fam(sg, [f"IND{i}" for i in range(5)]))
    assert names == ["env_0", "env_1"] and kept == [0, 1, 2, 3, 4]
    np.testing.assert_allclose(x, np.array(k["expected"]), rtol=0, atol=k["tol"])
    assert x[1, 1] == (0.5 + 3.5 + 4.5) / 3.0 and x[0, 0] == 4.0


def test_csv_fam_order_and_extra_samples(tmp_path):
    sg = _sg()
    path = tmp_path / "cov.csv"
    path.write_text(",a,b\r\nS3,3,30\r\n\r\nS1,1,10\r\nS9,9,90\r\nS2,2,nan\r\n")
    names, x, kept = sg.load_covariates(path, _fam(sg, ["S1", "S2", "S3"]))
    assert names == ["a", "b"] and kept == [0, 1, 2]
    np.testing.assert_array_equal(x, [[1, 10], [2, 20], [3, 30]])   # 'nan' is missing: mean of 10 and 30


def test_intersect_samples(tmp_path):
    sg = _sg()
    path = tmp_path / "cov.tsv"
    path.write_text("id\tv\nB\t2\nD\t4\n")
    fam = _fam(sg, ["A", "B", "C", "D"])
    with pytest.raises(sg.SchnelGpuError, match="--intersect-samples"):
        sg.load_covariates(path, fam)
    names, x, kept = sg.load_covariates(path, fam, intersect=True)
    assert kept == [1, 3] and x[:, 0].tolist() == [2.0, 4.0]
    with pytest.raises(sg.SchnelGpuError, match="No samples in common"):
        sg.load_covariates(path, _fam(sg, ["X", "Y"]), intersect=True)


@pytest.mark.parametrize("text,match", [
    ("", "empty"),
    ("id\n", "header has only 1 field"),
    ("id\tv\n\n", "no data rows"),
    ("id\tv\nA\t1\nA\t2\n", "Duplicate sample ID 'A'"),
    ("id\tv\nA\t1\n\nB\t1\t2\n", "Line 4 has 3 fields"),
    ("id\tv\nA\tinf\n", "Infinite value"),
    # the message shows the parsed value as Rust displays it (src/main.rs:436-443)
    ("id\tv\nA\t1e999\n", r"Infinite value \(inf\) for covariate 'v' on line 2 \(sample 'A'\)"),
    ("id\tv\nA\t-Infinity\n", r"Infinite value \(-inf\)"),
    ("id\tv\nA\t1_0\n", "Failed to parse value '1_0'"),
    ("id\tv\nA\tabc\n", "Failed to parse value 'abc' for covariate 'v' on line 2"),
])
def test_errors(tmp_path, text, match):
    sg = _sg()
    path = tmp_path / "cov.tsv"
    path.write_text(text)
    with pytest.raises(sg.SchnelGpuError, match=match) as e:
        sg.load_covariates(path, _fam(sg, ["A", "B"]))
    assert e.value.code == sg.ERR_BAD_ARG


def test_all_missing_column_and_missing_file(tmp_path):
    sg = _sg()
    path = tmp_path / "cov.tsv"
    path.write_text("id\tv\tw\nA\tNA\t1\nB\t.\t\n")
    names, x, _ = sg.load_covariates(path, _fam(sg, ["A", "B"]))
    np.testing.assert_array_equal(x, [[0.0, 1.0], [0.0, 1.0]])     # no observed value: 0
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.load_covariates(tmp_path / "none.tsv", _fam(sg, ["A"]))
    assert e.value.code == sg.ERR_IO


def _bed(sg, iids):
    return sg.BedFile(Path("x.bed"), _fam(sg, iids), [], np.zeros(0, np.uint8))


def test_align_est_bed_samples():
    """--est-bed alignment (src/main.rs:282-331): the estimation .bed follows
    the main .bed's samples and order; a missing sample is an error."""
    sg = _sg()
    est = _bed(sg, ["A", "B", "C"])
    sg.align_est_bed_samples(est, _bed(sg, ["A", "B", "C"]))
    assert est.sample_keep is None and est.n_samples == 3            # already aligned: untouched
    est = _bed(sg, ["A", "B", "C", "D"])
    sg.align_est_bed_samples(est, _bed(sg, ["C", "A", "D"]))
    assert est.sample_keep.tolist() == [2, 0, 3] and [r.iid for r in est.fam_records] == ["C", "A", "D"]
    assert est.n_samples == 3 and est.n_physical_samples == 4
    est = _bed(sg, ["A", "B"])
    with pytest.raises(sg.SchnelGpuError, match=r"missing 6 sample\(s\) .*\[C, D, E, F, G\], \.\.\.") as e:
        sg.align_est_bed_samples(est, _bed(sg, ["A", "C", "D", "E", "F", "G", "H"]))
    assert e.value.code == sg.ERR_BAD_ARG


def _triplet(tmp_path, n, p, fam_lines=None, bim_lines=None, payload=None):
    from oracle import lfmm_oracle as O
    rng = np.random.default_rng(n * 1000 + p)
    codes = rng.integers(0, 4, size=(p, n), dtype=np.uint8)
    packed = O.pack_codes(codes) if payload is None else payload
    (tmp_path / "t.bed").write_bytes(bytes([0x6C, 0x1B, 0x01]) + packed.tobytes())
    (tmp_path / "t.fam").write_text("".join(fam_lines if fam_lines is not None else
                                            [f"F{i} I{i} 0 0 {i % 3} -9\n" for i in range(n)]))
    (tmp_path / "t.bim").write_text("".join(bim_lines if bim_lines is not None else
                                            [f"{1 + i // 4}\trs{i}\t0.5\t{100 + i}\tA\tG\n" for i in range(p)]))
    return tmp_path / "t.bed", packed


def test_bed_file_open(tmp_path):
    """BedFile::open (src/bed.rs:60-135): .fam / .bim parsed, the .bed's magic
    and size checked, the payload mapped; subset_samples (:155-159) keeps the
    physical layout."""
    sg = _sg()
    path, packed = _triplet(tmp_path, 10, 7)
    bed = sg.BedFile.open(path)
    assert bed.n_samples == bed.n_physical_samples == 10 and bed.n_snps == 7 and bed.bytes_per_snp() == 3
    assert bed.fam_records[3] == sg.FamRecord("F3", "I3", "0", "0", 0, "-9")
    assert bed.bim_records[5] == sg.BimRecord("2", "rs5", 0.5, 105, "A", "G")
    np.testing.assert_array_equal(np.asarray(bed.payload).reshape(7, 3), packed)
    bed.subset_samples([9, 0, 4])
    assert bed.n_samples == 3 and bed.n_physical_samples == 10 and bed.bytes_per_snp() == 3
    assert [r.iid for r in bed.fam_records] == ["I9", "I0", "I4"] and bed.sample_keep.tolist() == [9, 0, 4]


def test_bed_file_open_errors(tmp_path):
    sg = _sg()
    path, _ = _triplet(tmp_path, 10, 7, payload=np.zeros((6, 3), np.uint8))   # one SNP short
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.BedFile.open(path)
    assert e.value.code == sg.ERR_BAD_BED
    path, _ = _triplet(tmp_path, 4, 2, fam_lines=["F0 I0 0 0 1\n"] * 4)
    with pytest.raises(sg.SchnelGpuError, match="FAM line 1 has 5 fields"):
        sg.BedFile.open(path)
    path, _ = _triplet(tmp_path, 4, 2, bim_lines=["1 rs0 0 x A G\n", "1 rs1 0 5 A G\n"])
    with pytest.raises(sg.SchnelGpuError, match="BIM line 1: invalid position 'x'"):
        sg.BedFile.open(path)
    with pytest.raises(sg.SchnelGpuError) as e:
        sg.BedFile.open(tmp_path / "absent.bed")
    assert e.value.code == sg.ERR_IO


def test_subset_spec_counts():
    """SubsetSpec counts (src/bed.rs:162-171) against the oracle's index lists
    and the reference's subset known answers."""
    sg = _sg()
    from oracle import lfmm_oracle as O
    for n_snps in (0, 1, 99, 100, 101, 10_000):
        assert sg.SubsetSpec.all().count(n_snps) == n_snps
        for rate in (0.01, 0.1, 0.37, 0.5, 1.0):
            assert sg.SubsetSpec.from_rate(rate).count(n_snps) == len(O.subset_indices(n_snps, rate=rate))
    k = KATS["subset_count_consistency"]
    assert sg.SubsetSpec.from_indices(k["indices"]).count(k["n"]) == k["indices_count"]
    for bad in (0.0, -0.1, 5.0, float("nan")):
        with pytest.raises(sg.SchnelGpuError, match="est-rate must be in"):
            sg.SubsetSpec.from_rate(bad)


def test_imputation_warnings_and_na_case(tmp_path, capsys):
    """NA tokens in any case count as missing, and the warning names each
    covariate with its missing count (the expectations of the reference's
    tests/integration.rs:278-350)."""
    sg = _sg()
    path = tmp_path / "cov.tsv"
    rows = ["IND0\t.\t0.5", "IND1\t1.0\tNA", "IND2\t2.0\tna", "IND3\t3.0\tNa", "IND4\t\t1.5", "IND5\t4.0\t2.5"]
    path.write_text("sample_id\tenv_0\tenv_1\n" + "\n".join(rows) + "\n")
    names, x, _ = sg.load_covariates(path, _fam(sg, [f"IND{i}" for i in range(6)]))
    err = capsys.readouterr().err
    assert "imputed to column mean" in err
    assert "covariate 'env_0' has 2 missing value(s)" in err and "covariate 'env_1' has 3 missing value(s)" in err
    assert x[0, 0] == x[4, 0] == (1.0 + 2.0 + 3.0 + 4.0) / 4.0
    assert x[1, 1] == x[2, 1] == x[3, 1] == (0.5 + 1.5 + 2.5) / 3.0
