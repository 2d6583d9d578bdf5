"""GPU tests of the scan's scheduling choices, which must never change a result.

- Hot tiles first: large scans visit the tiles of the strongest marginal SNPs
  before the rest.  The ranked list must equal the band-order scan's (a scan
  with progress callbacks keeps band order) and the other counting kernel's.
- Arbitrary allele rows: rows handed in directly may leave a valid sample with
  neither allele set (a .bed never does); the bounds assume nothing about the
  rows, so the scan must still equal the oracle.
- Class size: the tensor-core kernel passes counts as 16-bit values, so it
  refuses classes above 65,535 samples; AUTO then picks the popcount kernel.
"""
import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def test_hot_order_matches_band_order_and_other_kernel(gepi):
    # 8,000 SNPs: ~6,300 tensor-core tiles and ~31,000 popcount tiles, both
    # above the size at which the scan reorders its tiles
    spec = gepi.SynthSpec(n_snps=8000, n_cases=300, n_controls=320, maf_lo=0.02, maf_hi=0.5,
                          missing=0.01, n_planted=3, odds_ratio=4.0, seed=808)
    bed, ph, _ = gepi.synth_bed(spec)
    k = 2000
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        hot_tc = pl.scan(k, method=2)
        hot_popc = pl.scan(k, method=1)
        seen = []
        band_tc = pl.scan_progress(k, seen.append, points=0, with_tops=False, method=2)
    assert seen, "band-order scan reported no progress"
    assert hot_tc.tobytes() == band_tc.tobytes()
    assert hot_tc.tobytes() == hot_popc.tobytes()
    assert np.count_nonzero(hot_tc["n"].reshape(-1)) > 0


@pytest.mark.parametrize("method", [1, 2], ids=["popc", "tensor"])
def test_rows_without_allele_cover_match_oracle(gepi, tmp_path, method):
    spec = gepi.SynthSpec(n_snps=120, n_cases=150, n_controls=170, maf_lo=0.05, maf_hi=0.5,
                          missing=0.02, n_planted=2, odds_ratio=3.0, seed=1212)
    base = str(tmp_path / "u")
    gepi.synth_write(spec, base)
    fs = H.read_fileset(base)
    bits, valid, m1, m2 = H.decode_rows(fs)
    # clear both allele rows of a third of the valid samples of every other SNP:
    # valid samples carrying neither allele (never produced by a .bed)
    rng = np.random.default_rng(5)
    bits = bits.copy()
    for s in range(0, spec.n_snps, 2):
        drop = rng.integers(0, 2**63, size=bits.shape[1], dtype=np.int64).astype(np.uint64)
        drop &= rng.integers(0, 2**63, size=bits.shape[1], dtype=np.int64).astype(np.uint64)
        bits[2 * s] &= ~drop
        bits[2 * s + 1] &= ~drop
    rows = (bits, valid, m1, m2)
    k = 800
    with gepi.Planes.from_rows(bits, valid, m1, m2) as pl:
        got = pl.scan(k, method=method)
    want, _, _ = H.oracle_topk(rows, k)
    assert got.tobytes() == want.tobytes()


def test_tensor_kernel_refuses_classes_above_16_bits(gepi):
    spec = gepi.SynthSpec(n_snps=150, n_cases=65600, n_controls=64, maf_lo=0.05, maf_hi=0.5,
                          missing=0.01, n_planted=0, seed=65600)
    bed, ph, _ = gepi.synth_bed(spec)
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        with pytest.raises(gepi.GepiError):
            pl.scan(100, method=2)
        auto = pl.scan(100, method=0)
        popc = pl.scan(100, method=1)
        assert auto.tobytes() == popc.tobytes()
        assert pl.last_stats()["method"] == 1


def test_fisher_auto_choice_matches_both_kernels(gepi):
    # AUTO times the two kernels on a short Fisher scan for Fisher requests;
    # whichever it picks, the ranked list is the same
    spec = gepi.SynthSpec(n_snps=700, n_cases=260, n_controls=240, maf_lo=0.05, maf_hi=0.5,
                          missing=0.02, n_planted=2, odds_ratio=3.0, seed=4242)
    bed, ph, _ = gepi.synth_bed(spec)
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        auto = pl.scan(300, objective=1, method=0)
        chosen = pl.last_stats()["method"]
        popc = pl.scan(300, objective=1, method=1)
        tc = pl.scan(300, objective=1, method=2)
    assert chosen in (1, 2)
    assert auto.tobytes() == popc.tobytes() == tc.tobytes()
