"""gepi_process_gpu_1_noalloc: the scan for callers that cannot allocate
device memory (hosts whose GPU memory belongs to their own pool or framework).
It must return what gepi_process_gpu_1 returns for the same inputs -- the
same tolerance as every other parity test: identical indices and counts, and
for entropy the float score bit for bit -- on consecutive calls that reuse its
fixed scratch array, and refuse inputs beyond that array with GEPI_ERR_LIMIT.
Kept in a file pytest collects last."""
import ctypes

import numpy as np
import pytest

import helpers as H

pytestmark = pytest.mark.gpu


def _call(gepi, fn, rows, k, objective):
    bits, valid, m1, m2 = rows
    par = gepi.Params(topmost=k, ffun=objective)._c()
    tops = np.zeros(k, dtype=gepi.RESULT_DTYPE)
    st = fn(H.ptr(bits), H.ptr(valid), bits.shape[0], bits.shape[1], H.ptr(m1), H.ptr(m2),
            H.ptr(tops), ctypes.byref(par))
    assert st == 0, gepi.lib().gepi_last_error()
    return tops


def _rows(gepi, tmp_path, name, **kw):
    base = str(tmp_path / name)
    gepi.synth_write(gepi.SynthSpec(**kw), base)
    return H.decode_rows(H.read_fileset(base))


def _same(got, want, objective):
    for i in range(want.size):
        g, w = got[i], want[i]
        assert (int(g["sA"]), int(g["sB"]), int(g["fun"]), tuple(g["n"])) == \
               (int(w["sA"]), int(w["sB"]), int(w["fun"]), tuple(w["n"])), i
        if objective == 0:
            assert np.float32(g["ent"]).tobytes() == np.float32(w["ent"]).tobytes(), i
        else:
            # Fisher: log-factorial tables built by device lgamma vs host lgamma
            assert abs(float(g["ent"]) - float(w["ent"])) <= 2e-7 * abs(float(w["ent"])) + 1e-30, i


def test_noalloc_matches_process_gpu_1_on_consecutive_calls(gepi, tmp_path):
    L = gepi.lib()
    cases = [
        (dict(n_snps=150, n_cases=120, n_controls=130, missing=0.02, seed=55), 250, 0),
        (dict(n_snps=90, n_cases=400, n_controls=333, missing=0.05, n_planted=1, seed=56), 300, 0),
        (dict(n_snps=60, n_cases=70, n_controls=65, missing=0.02, seed=57), 120, 1),
    ]
    for i, (kw, k, obj) in enumerate(cases):
        rows = _rows(gepi, tmp_path, f"c{i}", **kw)
        want = _call(gepi, L.gepi_process_gpu_1, rows, k, obj)
        got = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, k, obj)
        _same(got, want, obj)
        again = _call(gepi, L.gepi_process_gpu_1_noalloc, rows, k, obj)
        assert again.tobytes() == got.tobytes()


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
