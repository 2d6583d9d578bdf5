"""GPU parity: the CUDA scan through the C ABI against the CPU oracle.

Integer work (Gram counts, contingency counts, row/function indices, the
ranked order) must be bit-exact.  Entropy scores are bit-exact too: both sides
rank by the same fixed-point key and round it to float the same way.  Fisher
p-values must agree within 1e-9 relative (|d ln p| <= 1e-9).
"""
import math
import os

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu

FISHER_RTOL = 1e-9  # on p: |d ln p| <= 1e-9


def make_planes(gepi, spec_kw, tmp_path, name="c"):
    spec = gepi.SynthSpec(**spec_kw)
    base = str(tmp_path / name)
    gepi.synth_write(spec, base)
    fs = H.read_fileset(base)
    rows = H.decode_rows(fs)
    pl = gepi.Planes.from_bed(fs.bed, fs.n_lines, fs.pheno)
    return pl, rows, fs, base


def items_of(tops):
    return [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in tops]


def assert_same_topk(got, want):
    assert got.shape == want.shape
    for i in range(got.size):
        g, w = got[i], want[i]
        gi = (int(g["sA"]), int(g["sB"]), int(g["fun"]), tuple(int(v) for v in g["n"]))
        wi = (int(w["sA"]), int(w["sB"]), int(w["fun"]), tuple(int(v) for v in w["n"]))
        assert gi == wi, f"rank {i}: gpu {gi} oracle {wi}"
        assert np.float32(g["ent"]).tobytes() == np.float32(w["ent"]).tobytes(), (
            f"rank {i}: ent {g['ent']!r} vs {w['ent']!r}")


SHAPES = [
    dict(n_snps=33, n_cases=31, n_controls=32, missing=0.02, seed=63),     # 63 samples
    dict(n_snps=64, n_cases=32, n_controls=32, missing=0.02, seed=64),     # 64
    dict(n_snps=65, n_cases=33, n_controls=32, missing=0.10, seed=65),     # 65
    dict(n_snps=70, n_cases=100, n_controls=29, missing=0.05, seed=129),   # class pad
    dict(n_snps=40, n_cases=1, n_controls=1, missing=0.0, seed=2),         # 1 + 1 samples
    dict(n_snps=45, n_cases=700, n_controls=1500, missing=0.3, seed=7),    # >1 K chunk
]


METHODS = {"popc": 1, "tensor": 2}
VARIANTS = [1, 2, 3, 4]  # popc 32x32 w32, popc 32x32 w16, popc 64x32 w32, tensor 80x64 w12


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("kw", SHAPES, ids=[f"s{k['n_cases'] + k['n_controls']}" for k in SHAPES])
def test_pair_counts_bit_exact(gepi, tmp_path, kw, variant):
    """Every counting variant (kernel, tile shape, words per stage) gives the
    oracle's Gram counts bit for bit."""
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    N = fs.n_lines
    m = gepi.variant_method(variant)
    got = pl.pair_counts(0, N, 0, N, method=m)
    want = H.oracle_pair_gram(rows, 0, N, 0, N)
    assert np.array_equal(got, want)
    # an unaligned sub-rectangle crossing tile boundaries
    a0, na, b0, nb = 3, min(N - 3, 37), 1, min(N - 1, 33)
    got = pl.pair_counts(a0, na, b0, nb, method=m)
    assert np.array_equal(got, H.oracle_pair_gram(rows, a0, na, b0, nb))
    pl.close()


@pytest.mark.parametrize("kw", [
    dict(n_snps=300, n_cases=400, n_controls=350, missing=0.02, seed=77),
    dict(n_snps=130, n_cases=1300, n_controls=900, missing=0.03, n_planted=2, seed=78),
])
def test_every_variant_returns_the_same_list(gepi, tmp_path, kw):
    """The autotuner's candidates are interchangeable: each variant's ranked
    list (and range list) is byte-identical and equals the oracle's."""
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 400
    want, _, _ = H.oracle_topk(rows, k)
    lists = []
    for v in VARIANTS:
        got = pl.scan(k, variant=v)
        st = pl.last_stats()
        assert st["variant"] == v and st["tile_snps"] == gepi.variant_shape(v)["tile_a"]
        assert_same_topk(got, want)
        lists.append(got.tobytes())
    assert len(set(lists)) == 1
    ranges = {pl.scan_range(40, 70, 5, 60, 150, method=0).tobytes()}
    for v in VARIANTS:
        r = gepi.ScanRequest(pl, 150, a0=40, na=70, b0=5, nb=60, variant=v)
        (got,) = gepi.scan_batch([r])
        ranges.add(got.tobytes())
    assert len(ranges) == 1
    pl.close()


def test_tensor_counts_exact_at_large_counts(gepi):
    """FP8 products summed in FP32 stay exact up to the largest counts: all-set
    and half-set planes over 40,000 samples per class, tensor == popcount."""
    n_snps, n_samples = 40, 80000
    nw = n_samples // 64
    rng = np.random.default_rng(9)
    bits = np.zeros((2 * n_snps, nw), dtype=np.uint64)
    valid = np.full((2 * n_snps, nw), np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
    for s in range(n_snps):
        kind = s % 4
        if kind == 0:      # every sample carries both alleles (all three planes set)
            bits[2 * s] = bits[2 * s + 1] = np.uint64(0xFFFFFFFFFFFFFFFF)
        elif kind == 1:    # column-5 allele everywhere
            bits[2 * s] = np.uint64(0xFFFFFFFFFFFFFFFF)
        else:              # random
            bits[2 * s] = rng.integers(0, 2**63, size=nw, dtype=np.uint64)
            bits[2 * s + 1] = ~bits[2 * s] | rng.integers(0, 2**63, size=nw, dtype=np.uint64)
    m1 = np.zeros(nw, dtype=np.uint64)
    m2 = np.zeros(nw, dtype=np.uint64)
    m1[: nw // 2] = np.uint64(0xFFFFFFFFFFFFFFFF)
    m2[nw // 2:] = np.uint64(0xFFFFFFFFFFFFFFFF)
    with gepi.Planes.from_rows(bits, valid, m1, m2) as pl:
        assert pl.class_sizes() == (40000, 40000)
        p = pl.pair_counts(0, n_snps, 0, n_snps, method=1)
        t = pl.pair_counts(0, n_snps, 0, n_snps, method=2)
    assert p.max() == 40000
    assert np.array_equal(p, t)


def test_rows_path_matches_bed_path(gepi, tmp_path):
    kw = dict(n_snps=50, n_cases=90, n_controls=77, missing=0.04, seed=21)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    bits, valid, m1, m2 = rows
    pr = gepi.Planes.from_rows(bits, valid, m1, m2)
    assert pr.class_sizes() == pl.class_sizes() == (77, 90)
    assert np.array_equal(pr.pair_counts(0, 50, 0, 50), pl.pair_counts(0, 50, 0, 50))
    pr.close()
    pl.close()


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("name", ["test", "thinhap1", "cfg1", "s63", "s64", "s65", "s129", "miss50",
                                  "cfg2_small"])
def test_scan_entropy_matches_oracle_and_gold(gepi, tmp_path, name, method):
    doc = H.load_golden(name)
    base = H.golden_input(doc, str(tmp_path))
    fs = H.read_fileset(base)
    rows = H.decode_rows(fs)
    k = doc["k"]
    with gepi.Planes.from_bed(fs.bed, fs.n_lines, fs.pheno) as pl:
        got = pl.scan(k, method=METHODS[method])
    want, keys, nranked = H.oracle_topk(rows, k)
    assert_same_topk(got, want)
    if nranked >= k:
        gold = doc["rows"]
        gold_items = [(r["sA"], r["sB"], r["fun"]) for r in gold]
        gold_keys = [k_ for k_, _ in H.exact_keys(rows, gold_items)]
        probs = H.compare_ranked(items_of(got), [-float(v) for v in keys], gold_items, gold_keys,
                                 k, rtol=2e-5)
        assert not probs, probs[:5]


def test_scan_is_deterministic_and_method_independent(gepi, tmp_path):
    kw = dict(n_snps=300, n_cases=400, n_controls=350, missing=0.02, seed=77)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    a = pl.scan(500, method=1)
    b = pl.scan(500, method=1)
    c = pl.scan(500, method=2)
    assert a.tobytes() == b.tobytes() == c.tobytes()
    # the plane set keeps its last scan tile list: repeats reuse it, other
    # ranges, tile shapes and uploads (pair counts, autotuning) replace it
    N = fs.n_lines
    r1 = pl.scan_range(40, 200, 10, 150, 300, method=2)
    assert_same_topk(r1, H.oracle_topk_range(rows, 80, 480, 20, 320, 300)[0])
    assert pl.scan(500, method=2).tobytes() == a.tobytes()
    assert np.array_equal(pl.pair_counts(0, N, 0, N, method=2), H.oracle_pair_gram(rows, 0, N, 0, N))
    assert pl.scan(500, method=2).tobytes() == a.tobytes()
    assert pl.scan_range(40, 200, 10, 150, 300, method=2).tobytes() == r1.tobytes()
    assert pl.scan(500, method=1).tobytes() == a.tobytes()
    pl.close()


def test_autotune_choice_drives_auto(gepi, tmp_path):
    """METHOD_AUTO uses the autotuner's pick -- the fastest timed variant --
    and every method gives the same list."""
    kw = dict(n_snps=400, n_cases=600, n_controls=700, missing=0.02, seed=91)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    rep_ = pl.autotune_variants()
    ms = rep_["ms"]
    assert all(v > 0 for v in ms.values()), ms
    assert rep_["name"] == min(ms, key=ms.get)
    t = pl.autotune()
    assert t["method"] in (METHODS["popc"], METHODS["tensor"])
    assert t["popc_ms"] > 0 and t["tensor_ms"] > 0
    assert (t["tensor_ms"] < t["popc_ms"]) == (t["method"] == METHODS["tensor"])
    assert pl.autotune() == t  # cached per plane set
    a = pl.scan(300)
    assert pl.last_stats()["method"] == t["method"]
    assert pl.last_stats()["variant"] == rep_["variant"]
    b = pl.scan(300, method=METHODS["popc"] + METHODS["tensor"] - t["method"])
    assert a.tobytes() == b.tobytes()
    want, _, _ = H.oracle_topk(rows, 300)
    assert_same_topk(a, want)
    pl.close()
    small, _, _, _ = make_planes(gepi, dict(n_snps=100, n_cases=50, n_controls=60, seed=92),
                                 tmp_path, "s")
    assert small.autotune() == {"method": METHODS["popc"], "popc_ms": 0.0, "tensor_ms": 0.0}
    small.close()


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("cap", ["4096", "20000"])
def test_scan_exact_under_candidate_overflow(gepi, tmp_path, cap, monkeypatch, method):
    """A tiny candidate buffer forces overflow, select, compaction and batch
    retries; the result must stay exact."""
    kw = dict(n_snps=200, n_cases=150, n_controls=170, missing=0.03, seed=31)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    monkeypatch.setenv("GEPI_DEBUG_CAP", cap)
    got = pl.scan(300, method=METHODS[method])
    monkeypatch.delenv("GEPI_DEBUG_CAP")
    want, _, _ = H.oracle_topk(rows, 300)
    assert_same_topk(got, want)
    pl.close()


def test_k_beyond_ranked_tests_zero_pads(gepi, tmp_path):
    kw = dict(n_snps=3, n_cases=4, n_controls=3, missing=0.0, seed=12)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 100  # 5 * 6 * 7 / 2 = 105 tests, many with zero association
    got = pl.scan(k)
    want, _, nranked = H.oracle_topk(rows, k)
    assert nranked < k
    assert_same_topk(got, want)
    assert all(int(t["sA"]) == 0 and int(t["n"][2]) == 0 for t in got[nranked:])
    pl.close()


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("rng_", [(0, 40, 0, 40), (40, 60, 5, 50), (90, 30, 0, 120), (7, 1, 7, 1)])
def test_scan_range_matches_oracle(gepi, tmp_path, rng_, method):
    kw = dict(n_snps=120, n_cases=160, n_controls=140, missing=0.02, seed=41)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    a0, na, b0, nb = rng_
    got = pl.scan_range(a0, na, b0, nb, 200, method=METHODS[method])
    want, _, _ = H.oracle_topk_range(rows, 2 * a0, 2 * (a0 + na), 2 * b0, 2 * (b0 + nb), 200)
    assert_same_topk(got, want)
    pl.close()


def test_process_gpu_1_dropin(gepi, tmp_path):
    """process_gpu_1 with the reference reader's host arrays."""
    spec = gepi.SynthSpec(n_snps=150, n_cases=120, n_controls=130, missing=0.02, seed=55)
    base = str(tmp_path / "p")
    gepi.synth_write(spec, base)
    r = gepi.BinPlinkReader(base)
    assert r.checkConsistency() and r.readData()
    par = gepi.Params(topmost=250)
    tops = np.zeros(250, dtype=gepi.RESULT_DTYPE)
    gepi.process_gpu_1(r, tops, par)
    want, _, _ = H.oracle_topk((r.BitData(), r.ValidData(), r.classMask(1), r.classMask(2)), 250)
    assert_same_topk(tops, want)


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("kw", [
    dict(n_snps=60, n_cases=70, n_controls=65, missing=0.02, seed=81),
    dict(n_snps=40, n_cases=300, n_controls=420, missing=0.05, n_planted=2, seed=82),
])
def test_scan_fisher_matches_oracle(gepi, tmp_path, kw, method):
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 150
    got = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    want, keys, nranked = H.oracle_topk(rows, k, objective=1)
    assert nranked >= k
    # values: every returned test re-scored by the oracle within tolerance
    items = items_of(got)
    ex = H.exact_keys(rows, items, objective=1)
    worst = 0.0
    for t, (key, n) in zip(got, ex):
        assert tuple(int(v) for v in t["n"]) == n
        want_l10 = -key
        d = abs(float(t["ent"]) - want_l10)
        assert d <= 2e-7 * abs(want_l10) + 1e-30  # float rounding of the output
    # ranked lists identical up to near-ties within the Fisher tolerance
    got_keys = [k_ for k_, _ in ex]
    probs = H.compare_ranked(items, got_keys, items_of(want), [-float(v) for v in keys], k,
                             rtol=FISHER_RTOL * 10)
    assert not probs, probs[:5]
    pl.close()


def _device_value_errors(gepi, rows, got, values, objective):
    """Largest |d ln p| (Fisher) or relative error of I (entropy) of the
    device's FP64 values against the oracle's FP64 restatements
    (fisher_p.c:52-76 with R's tie rule; entropyDelta4, entropy_inline.h:30-80)."""
    lib = H.oracle()
    worst = 0.0
    for t, v in zip(got, values):
        w, x, y, z = (int(q) for q in t["n"])
        if w * z == x * y:  # zero-filled slot
            assert v == 0.0
            continue
        if objective == 1:
            ref = lib.orc_fisher_log10p(w, y - w, x, z - x, 0)
            assert math.isfinite(ref)
            worst = max(worst, abs(v - ref) * math.log(10.0))
        else:
            ref = lib.orc_entropy_f64(w, x, y, z)  # entropyDelta4: -I bits, the sign of `ent`
            worst = max(worst, abs(v - ref) / abs(ref))
        assert np.float32(v) == np.float32(t["ent"])
    return worst


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("kw", [
    dict(n_snps=60, n_cases=70, n_controls=65, missing=0.02, seed=81),
    dict(n_snps=40, n_cases=300, n_controls=420, missing=0.05, n_planted=2, seed=82),
    dict(n_snps=120, n_cases=1500, n_controls=1700, missing=0.01, n_planted=2, seed=83),
])
def test_device_fp64_values_within_tolerance(gepi, tmp_path, kw, method):
    """The device's FP64 objective of every returned test, before the float
    rounding of the output field: Fisher p within 1e-9 relative
    (|d ln p| <= 1e-9) of the oracle's FP64 Fisher, entropy within 1e-6
    relative of the FP64 entropyDelta4 restatement."""
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 150
    got = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    err_f = _device_value_errors(gepi, rows, got, pl.last_values(k), 1)
    assert err_f <= FISHER_RTOL, err_f
    got = pl.scan(k, objective=gepi.ENTROPY, method=METHODS[method])
    err_e = _device_value_errors(gepi, rows, got, pl.last_values(k), 0)
    assert err_e <= 1e-6, err_e
    print(f"max device error: Fisher |d ln p| {err_f:.3e}, entropy rel {err_e:.3e}")
    pl.close()


@pytest.mark.parametrize("method", sorted(METHODS))
@pytest.mark.parametrize("kw", [
    dict(n_snps=40, n_cases=300, n_controls=420, missing=0.05, n_planted=2, seed=82),
    dict(n_snps=120, n_cases=1500, n_controls=1700, missing=0.01, n_planted=2, seed=83),
])
def test_device_fisher_fp64_walks_within_tolerance(gepi, tmp_path, monkeypatch, kw, method):
    """The FP64 tail walks that tables of 2^24 samples and more take, forced
    at these sizes with GEPI_DEBUG_FISHER_FP64=1: every returned p within
    1e-9 relative of the oracle's FP64 Fisher, like the float-float walks
    that run by default."""
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 150
    monkeypatch.setenv("GEPI_DEBUG_FISHER_FP64", "1")
    got = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    err64 = _device_value_errors(gepi, rows, got, pl.last_values(k), 1)
    monkeypatch.delenv("GEPI_DEBUG_FISHER_FP64")
    got = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    err_ff = _device_value_errors(gepi, rows, got, pl.last_values(k), 1)
    assert err64 <= FISHER_RTOL, err64
    assert err_ff <= FISHER_RTOL, err_ff
    print(f"max device error: Fisher |d ln p| FP64 walks {err64:.3e}, float-float {err_ff:.3e}")
    pl.close()


@pytest.mark.parametrize("method", sorted(METHODS))
def test_fisher_pending_list_overflow(gepi, tmp_path, monkeypatch, method):
    """Fisher tests that pass the bounds go to a pending list evaluated by a
    launch across the GPU; those past its capacity are evaluated inside the
    counting launch.  With the list shrunk to 7 entries (GEPI_DEBUG_PEND_CAP)
    most tests take that path: the same ranked tests with the same counts,
    FP64 values equal to 1e-12 (the two evaluations are one function, built
    into different kernels), and within 1e-9 of the oracle."""
    kw = dict(n_snps=120, n_cases=1500, n_controls=1700, missing=0.01, n_planted=2, seed=83)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 150
    want = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    want_v = pl.last_values(k)
    monkeypatch.setenv("GEPI_DEBUG_PEND_CAP", "7")
    got = pl.scan(k, objective=gepi.FISHER, method=METHODS[method])
    got_v = pl.last_values(k)
    monkeypatch.delenv("GEPI_DEBUG_PEND_CAP")
    for f in ("sA", "sB", "n", "fun"):
        assert np.array_equal(got[f], want[f]), f
    assert np.allclose(got_v, want_v, rtol=1e-12, atol=0.0)
    err = _device_value_errors(gepi, rows, got, got_v, 1)
    assert err <= FISHER_RTOL, err
    pl.close()


def test_device_fisher_fp64_config2_full_size(gepi):
    """Config 2 at full size (20,000 SNPs x 4,000 samples, 3 planted pairs),
    Fisher top-1,000 through both counting kernels: the same list, and every
    returned p within 1e-9 relative of the oracle's FP64 Fisher."""
    spec = gepi.SynthSpec(n_snps=20000, n_cases=2000, n_controls=2000, maf_lo=0.01, maf_hi=0.5,
                          missing=0.01, n_planted=3, odds_ratio=2.0, seed=1002)
    bed, ph, _ = gepi.synth_bed(spec)
    fs = H.Fileset(bed=bed, pheno=ph, n_lines=spec.n_snps, bim=[])
    rows = H.decode_rows(fs)
    k = 1000
    worst = 0.0
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        lists = []
        for method in (2, 1):
            got = pl.scan(k, objective=gepi.FISHER, method=method)
            worst = max(worst, _device_value_errors(gepi, rows, got, pl.last_values(k), 1))
            lists.append(got)
    assert lists[0].tobytes() == lists[1].tobytes()
    assert worst <= FISHER_RTOL, worst
    print(f"config 2 Fisher top-{k}: max |d ln p| {worst:.3e}")


def test_config2_scale_properties(gepi):
    """Config 2 (20,000 SNPs x 4,000 samples, 3 planted pairs, top
    1,000): size-independent checks -- every returned count and key is the
    oracle's, the list is sorted under the tie-break, and no sampled test beats
    the k-th entry without being listed."""
    spec = gepi.SynthSpec(n_snps=20000, n_cases=2000, n_controls=2000, maf_lo=0.01, maf_hi=0.5,
                          missing=0.01, n_planted=3, odds_ratio=2.0, seed=1002)
    bed, ph, planted = gepi.synth_bed(spec)
    fs = H.Fileset(bed=bed, pheno=ph, n_lines=spec.n_snps, bim=[])
    rows = H.decode_rows(fs)
    k = 1000
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        got = pl.scan(k, method=2)
        plain = pl.scan(k, method=1)
    assert got.tobytes() == plain.tobytes()
    items = items_of(got)
    ex = H.exact_keys(rows, items)
    keys = []
    for t, (key, n) in zip(got, ex):
        assert tuple(int(v) for v in t["n"]) == n
        assert np.float32(-key) == np.float32(t["ent"])
        keys.append(key)
    order = sorted(range(k), key=lambda i: (-keys[i], items[i]))
    assert order == list(range(k))
    kth = keys[-1]
    listed = set(items)
    rs = np.random.default_rng(5)
    R = 2 * spec.n_snps
    sample = []
    for _ in range(20000):
        a, b = sorted(int(v) for v in rs.integers(0, R, size=2))
        sample.append((b, a, int(rs.integers(0, 5))))
    for (key, _), it in zip(H.exact_keys(rows, sample), sample):
        assert key < kth or it in listed or key == kth


def test_config3_full_size_properties(gepi):
    """The headline workload at full size (100,000 SNPs x 10,000 samples, 10
    planted pairs, top-10,000), by size-independent properties: the tensor-core
    and popcount kernels return the same list bit for bit; every returned count
    and key is the oracle's; the list is sorted under the tie-break; no sampled
    test beats the k-th entry without being listed; two shards merged on the
    host equal the whole scan."""
    spec = gepi.SynthSpec(n_snps=100000, n_cases=5000, n_controls=5000, maf_lo=0.01, maf_hi=0.5,
                          missing=0.01, n_planted=10, odds_ratio=2.0, seed=1003)
    bed, ph, planted = gepi.synth_bed(spec)
    fs = H.Fileset(bed=bed, pheno=ph, n_lines=spec.n_snps, bim=[])
    rows = H.decode_rows(fs)
    k = 10000
    with gepi.Planes.from_bed(bed, spec.n_snps, ph) as pl:
        got = pl.scan(k, method=2)
        assert pl.last_stats()["method"] == 2
        plain = pl.scan(k, method=1)
        parts = [pl.scan_range(*gepi.shard_range(spec.n_snps, 2, s), k, method=2) for s in range(2)]
    assert got.tobytes() == plain.tobytes()
    assert gepi.merge_results(parts, k, 10000).tobytes() == got.tobytes()
    items = items_of(got)
    ex = H.exact_keys(rows, items)
    keys = []
    for t, (key, n) in zip(got, ex):
        assert tuple(int(v) for v in t["n"]) == n
        assert np.float32(-key) == np.float32(t["ent"])
        keys.append(key)
    order = sorted(range(k), key=lambda i: (-keys[i], items[i]))
    assert order == list(range(k))
    kth = keys[-1]
    listed = set(items)
    rs = np.random.default_rng(6)
    R = 2 * spec.n_snps
    sample = []
    for _ in range(50000):
        a, b = sorted(int(v) for v in rs.integers(0, R, size=2))
        sample.append((b, a, int(rs.integers(0, 5))))
    for (key, _), it in zip(H.exact_keys(rows, sample), sample):
        assert key < kth or it in listed or key == kth
