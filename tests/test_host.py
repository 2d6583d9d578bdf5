"""Host-side tests (no GPU): the C-ABI library loads and exports every symbol
include/gepi.h declares, the synthetic generator is byte-reproducible, the
host reader matches the oracle's restatement of BinPlinkReader, the host
Fisher test matches the oracle, and argument errors are reported before any
device work."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

import helpers as H

HEADER = os.path.join(H.ROOT, "include", "gepi.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gepi_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_header_symbol(gepi):
    lib = ctypes.CDLL(gepi.library_path())
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings(gepi):
    L = gepi.lib()
    assert L.gepi_abi_version() == 2
    assert L.gepi_status_string(0) == b"ok"
    assert L.gepi_status_string(6) == b"phenotype class 1 or 2 is empty"


def test_counting_variants_and_struct_layouts(gepi):
    """The counting-variant table (names, shapes) and the ctypes mirrors of the
    structs that carry a variant match the header's layout."""
    import ctypes

    names = [gepi.variant_name(v) for v in range(1, gepi.NUM_VARIANTS + 1)]
    assert names == ["popc_32x32_w32", "popc_32x32_w16", "popc_64x32_w32", "tensor_80x64_w12"]
    assert gepi.variant_name(0) == "" and gepi.variant_name(gepi.NUM_VARIANTS + 1) == ""
    assert gepi.variant_shape(3) == {"method": 1, "tile_a": 64, "tile_b": 32, "stage_words": 32}
    assert gepi.variant_shape(4) == {"method": 2, "tile_a": 80, "tile_b": 64, "stage_words": 12}
    assert ctypes.sizeof(gepi._Params) == 48 and gepi._Params.variant.offset == 20
    assert ctypes.sizeof(gepi._ScanReq) == 40 and gepi._ScanReq.variant.offset == 36
    assert gepi._ScanStats.variant.offset == 80 and ctypes.sizeof(gepi._ScanStats) == 88


def test_result_layout_matches_interaction_result(gepi):
    dt = gepi.RESULT_DTYPE
    assert dt.itemsize == 48
    assert dt.fields["sA"][1] == 0 and dt.fields["sB"][1] == 4
    assert dt.fields["n"][1] == 16 and dt.fields["ent"][1] == 32 and dt.fields["fun"][1] == 36


@pytest.mark.parametrize("name", [n for n in H.golden_names()])
def test_generator_reproduces_golden_inputs(name, gepi, tmp_path):
    doc = H.load_golden(name)
    # synthetic cases are regenerated, the reference's demo filesets read from
    # tests/golden/data; either way the sha256 of .bed/.bim/.fam must be the
    # one the golden output was made from
    H.golden_input(doc, str(tmp_path))


def test_synth_bed_matches_written_file(gepi, tmp_path):
    spec = gepi.SynthSpec(n_snps=100, n_cases=70, n_controls=61, missing=0.03, n_planted=2,
                          seed=5)
    base = str(tmp_path / "s")
    gepi.synth_write(spec, base)
    bed, ph, planted = gepi.synth_bed(spec)
    assert bed.tobytes() == open(base + ".bed", "rb").read()
    assert (ph == 2).sum() == 70 and (ph == 1).sum() == 61
    assert planted.shape == (2, 2) and len(set(planted.ravel().tolist())) == 4


def test_reader_matches_oracle_decode(gepi, tmp_path):
    spec = gepi.SynthSpec(n_snps=77, n_cases=65, n_controls=70, missing=0.05, seed=9)
    base = str(tmp_path / "r")
    gepi.synth_write(spec, base)
    r = gepi.BinPlinkReader(base)
    assert r.checkConsistency() and r.readData()
    bits, valid, m1, m2 = H.decode_rows(H.read_fileset(base))
    assert r.numSNPs() == 154 and r.numSamples() == 135 and r.elementsSNP() == 3
    assert np.array_equal(r.BitData(), bits) and np.array_equal(r.ValidData(), valid)
    assert np.array_equal(r.classMask(1), m1) and np.array_equal(r.classMask(2), m2)
    sid, allele, chrom, pos = r.getSnp(5)
    assert sid == "rs3" and allele in "ACGT" and chrom >= 1 and pos == 1200
    r.close()


def test_reader_on_reference_demo_data(gepi):
    base = os.path.join(H.GOLDEN_DATA_DIR, "thinhap1")
    r = gepi.BinPlinkReader(base)
    assert r.checkConsistency() and r.readData()
    bits, valid, m1, m2 = H.decode_rows(H.read_fileset(base))
    assert np.array_equal(r.BitData(), bits) and np.array_equal(r.ValidData(), valid)
    assert r.numSNPs() == 2040 and r.numSamples() == 89


def test_reader_errors(gepi, tmp_path):
    spec = gepi.SynthSpec(n_snps=10, n_cases=5, n_controls=5, seed=3)
    base = str(tmp_path / "e")
    gepi.synth_write(spec, base)
    data = bytearray(open(base + ".bed", "rb").read())
    open(base + ".bed", "wb").write(bytes(data[:-1]))
    r = gepi.BinPlinkReader(base)
    assert not r.checkConsistency() and "different than expected" in r.error
    data[0] = 0
    open(base + ".bed", "wb").write(bytes(data))
    r = gepi.BinPlinkReader(base)
    assert not r.checkConsistency() and "Magic" in r.error
    r = gepi.BinPlinkReader(str(tmp_path / "missing"))
    assert not r.checkConsistency()


def test_planes_argument_errors_before_device(gepi):
    """Format and class errors are detected on the host (no GPU touched)."""
    spec = gepi.SynthSpec(n_snps=8, n_cases=6, n_controls=6, seed=4)
    bed, ph, _ = gepi.synth_bed(spec)
    bad = bed.copy()
    bad[1] = 0
    with pytest.raises(gepi.GepiError) as e:
        gepi.Planes.from_bed(bad, 8, ph)
    assert e.value.status == 3
    with pytest.raises(gepi.GepiError) as e:
        gepi.Planes.from_bed(bed[:-1], 8, ph)
    assert e.value.status == 3
    with pytest.raises(gepi.GepiError) as e:
        gepi.Planes.from_bed(bed, 8, np.full_like(ph, 2))
    assert e.value.status == 6
    with pytest.raises(gepi.GepiError) as e:
        gepi.Planes.from_bed(bed, 8, np.where(ph == 1, -9, ph))
    assert e.value.status == 6


def test_host_fisher_matches_oracle(gepi):
    """p within 1e-9 relative of the oracle's FP64 restatement of fisher_p.c
    (R tie rule), i.e. |d log10 p| <= 1e-9 / ln 10."""
    lib = H.oracle()
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(3000):
        n = int(rng.integers(2, 3000))
        y = int(rng.integers(1, n))
        z = n - y
        w = int(rng.integers(0, y + 1))
        x = int(rng.integers(0, z + 1))
        ref = lib.orc_fisher_log10p(w, y - w, x, z - x, 0)
        got = gepi.fisher_log10p(w, y - w, x, z - x)
        if math.isnan(ref):
            continue
        if ref < -300:
            # the oracle's linear-space FP64 sum is subnormal or zero there
            assert got < -295
            continue
        d = abs(got - ref) * math.log(10.0)
        worst = max(worst, d)
        assert d <= 1e-9, (w, x, y, z, got, ref)
    print(f"host Fisher worst |rel p err| {worst:.3e}")


def test_host_fisher_known_values(gepi):
    assert abs(gepi.fisher_log10p(2, 1, 0, 3) - math.log10(0.4)) < 1e-12
    assert gepi.fisher_pval(0, 0, 0, 0) == 0.0
    assert gepi.fisher_log10p(5, 5, 5, 5) == 0.0
