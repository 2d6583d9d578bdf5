"""gepi_process_gpu_1_noalloc: the scan for callers that cannot allocate
device memory (hosts whose GPU memory belongs to their own pool or framework).
It must return what gepi_process_gpu_1 returns for the same inputs -- the same
bytes for either objective, since both build their scoring tables from the
same host values -- and what the oracle returns (identical indices and counts,
entropy scores bit for bit, Fisher within 1e-9 on p), on consecutive calls
that reuse its fixed scratch array; it must allocate no device memory, take
its candidate-overflow retry path like the allocating scan, and refuse inputs
beyond that array with GEPI_ERR_LIMIT.  Kept in a file pytest collects last."""
import ctypes
import ctypes.util
import math
import os

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _call(gepi, fn, rows, k, objective, verbose=0):
    bits, valid, m1, m2 = rows
    par = gepi.Params(topmost=k, ffun=objective)._c()
    par.verbose = verbose
    tops = np.zeros(k, dtype=gepi.RESULT_DTYPE)
    st = fn(H.ptr(bits), H.ptr(valid), bits.shape[0], bits.shape[1], H.ptr(m1), H.ptr(m2),
            H.ptr(tops), ctypes.byref(par))
    assert st == 0, gepi.lib().gepi_last_error()
    return tops


def _rows(gepi, tmp_path, name, **kw):
    base = str(tmp_path / name)
    gepi.synth_write(gepi.SynthSpec(**kw), base)
    return H.decode_rows(H.read_fileset(base))


def _same_as_oracle(got, rows, k, objective):
    want, keys, _ = H.oracle_topk(rows, k, objective=objective)
    if objective == 0:
        # entropy: exact keys on both sides, so the same list bit for bit
        for i in range(k):
            g, w = got[i], want[i]
            assert (int(g["sA"]), int(g["sB"]), int(g["fun"]), tuple(g["n"])) == \
                   (int(w["sA"]), int(w["sB"]), int(w["fun"]), tuple(w["n"])), i
            assert np.float32(g["ent"]).tobytes() == np.float32(w["ent"]).tobytes(), i
        return
    # Fisher: every returned test's counts are the oracle's and its p within
    # 1e-9 relative; the lists agree up to the order of tests whose p-values
    # tie within that tolerance
    items = [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in got]
    ex = H.exact_keys(rows, items, objective=1)
    for t, (key, n) in zip(got, ex):
        assert tuple(int(v) for v in t["n"]) == n
        assert abs(float(t["ent"]) + key) <= 2e-7 * abs(key) + 1e-9 / math.log(10.0)
    want_items = [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in want]
    probs = H.compare_ranked(items, [k_ for k_, _ in ex], want_items, [-float(v) for v in keys],
                             k, rtol=1e-8)
    assert not probs, probs[:5]


def _cudart():
    """The CUDA runtime, for cudaMemGetInfo (device-wide free memory)."""
    cands = [ctypes.util.find_library("cudart")]
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        if os.path.isdir(d):
            cands += [os.path.join(d, f) for f in sorted(os.listdir(d)) if f.startswith("libcudart.so")]
    for c in cands:
        if c:
            try:
                return ctypes.CDLL(c)
            except OSError:
                pass
    pytest.skip("no CUDA runtime library to read free device memory")


def _free_bytes(rt):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_noalloc_matches_process_gpu_1_and_oracle_on_consecutive_calls(gepi, tmp_path):
    L = gepi.lib()
    cases = [
        (dict(n_snps=150, n_cases=120, n_controls=130, missing=0.02, seed=55), 250, 0),
        (dict(n_snps=90, n_cases=400, n_controls=333, missing=0.05, n_planted=1, seed=56), 300, 0),
        (dict(n_snps=60, n_cases=70, n_controls=65, missing=0.02, seed=57), 120, 1),
        (dict(n_snps=45, n_cases=300, n_controls=420, missing=0.05, n_planted=2, seed=58), 150, 1),
    ]
    for i, (kw, k, obj) in enumerate(cases):
        rows = _rows(gepi, tmp_path, f"c{i}", **kw)
        want = _call(gepi, L.gepi_process_gpu_1, rows, k, obj)
        got = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, k, obj)
        assert got.tobytes() == want.tobytes()
        again = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, k, obj)
        assert again.tobytes() == got.tobytes()
        _same_as_oracle(got, rows, k, obj)


def test_noalloc_allocates_no_device_memory(gepi, tmp_path):
    """After a first call (which loads the library's kernels), further calls
    leave the device's free memory unchanged to the byte."""
    L = gepi.lib()
    rows = _rows(gepi, tmp_path, "m", n_snps=200, n_cases=300, n_controls=280, missing=0.02,
                 n_planted=1, seed=61)
    rt = _cudart()
    first = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, 400, 0)
    before = _free_bytes(rt)
    for obj in (0, 1, 0):
        got = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, 400, obj)
    assert _free_bytes(rt) == before
    assert got.tobytes() == first.tobytes()


def _overflow_rows(n_weak=1984, n_strong=64, n_samples=256, seed=71):
    """Rows whose last 64 SNPs carry the class almost perfectly: their tiles
    come last in the tile list, after the threshold has settled on the weak
    SNPs and the batches have grown, so one batch appends far more than the
    65,536-record candidate buffer holds."""
    rng = np.random.default_rng(seed)
    n_snps = n_weak + n_strong
    nw = n_samples // 64
    case = np.zeros(n_samples, dtype=bool)
    case[rng.permutation(n_samples)[: n_samples // 2]] = True
    g = np.empty((n_snps, n_samples), dtype=np.int8)  # minor-allele count 0/1/2
    maf = rng.uniform(0.05, 0.5, size=n_weak)
    g[:n_weak] = rng.binomial(2, maf[:, None], size=(n_weak, n_samples))
    p = np.where(case, 0.9, 0.1)
    g[n_weak:] = rng.binomial(2, p[None, :], size=(n_strong, n_samples))
    miss = rng.random((n_snps, n_samples)) < 0.01

    def pack(b):
        b = b.reshape(b.shape[0], nw, 64).astype(np.uint64)
        return (b << np.arange(64, dtype=np.uint64)).sum(axis=2, dtype=np.uint64)

    # row 2s: carriers of the first allele (count >= 1), row 2s+1: of the other (count <= 1)
    a = (g >= 1) & ~miss
    b = (g <= 1) & ~miss
    bits = np.empty((2 * n_snps, nw), dtype=np.uint64)
    bits[0::2] = pack(a)
    bits[1::2] = pack(b)
    v = pack(~miss)
    valid = np.repeat(v, 2, axis=0)
    m1 = pack(~case[None, :])[0]
    m2 = pack(case[None, :])[0]
    return bits, valid, m1, m2


def test_noalloc_candidate_overflow_retry(gepi, capfd):
    """A burst of strong tests overflows the fixed candidate buffer inside one
    batch; the retry (threshold from what was captured, compaction, the batch
    again in halves) runs and the list still equals gepi_process_gpu_1's and
    the oracle's."""
    L = gepi.lib()
    rows = _overflow_rows()
    k = 16384
    got = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, k, 0, verbose=1)
    err = capfd.readouterr().err
    assert "candidate overflow" in err, err[-2000:]
    want = _call(gepi, L.gepi_process_gpu_1, rows, k, 0)
    assert got.tobytes() == want.tobytes()
    _same_as_oracle(got, rows, k, 0)


def test_noalloc_rejects_requests_beyond_its_scratch(gepi, tmp_path):
    L = gepi.lib()
    rows = _rows(gepi, tmp_path, "small", n_snps=20, n_cases=10, n_controls=10, seed=3)
    bits, valid, m1, m2 = rows
    tops = np.zeros(20000, dtype=gepi.RESULT_DTYPE)
    par = gepi.Params(topmost=20000)._c()  # k beyond the 16,384 limit
    st = L.gepi_process_gpu_1_noalloc(H.ptr(bits), H.ptr(valid), bits.shape[0], bits.shape[1],
                                      H.ptr(m1), H.ptr(m2), H.ptr(tops), ctypes.byref(par))
    assert st == 9
    big = np.zeros((2 * 20000, 64), dtype=np.uint64)  # 40,000 rows x 4,096 samples: too large
    m = np.zeros(64, dtype=np.uint64)
    m[0], m[1] = 1, 2
    par = gepi.Params(topmost=10)._c()
    st = L.gepi_process_gpu_1_noalloc(H.ptr(big), H.ptr(big), big.shape[0], big.shape[1],
                                      H.ptr(m), H.ptr(m[::-1].copy()), H.ptr(tops),
                                      ctypes.byref(par))
    assert st == 9, gepi.lib().gepi_last_error()
