"""Failure detection on the GPU without a GPU fault: the tensor-core counting
kernel's bounded waits.

The kernel's roles (bulk copies, producers, the MMA thread, the scoring warps)
wait on one another through mbarriers, each wait bounded by a clock budget; on
expiry the CTA pair records an error code, drains its own copies and MMAs,
meets at the final cluster barrier, frees its tensor memory and returns, and
the host turns the code into GEPI_ERR_TIMEOUT.  GEPI_DEBUG_STALL=<cycles>
(tests only) makes the producers withhold their arrivals on the first chunk's
full barrier -- a flag nothing else sets -- with a short budget, so the MMA
thread's wait runs out on any shape.  The test checks the status on every
entry point that launches the kernel, and that the next scan on the same plane
set, with the normal budget, equals the oracle.  (The reference prints CUDA
errors and carries on, inc/gEpiCount.h:37-38.)"""
import numpy as np
import pytest

import helpers as H
from test_gpu_parity import assert_same_topk, make_planes

pytestmark = pytest.mark.gpu

TIMEOUT = 7  # GEPI_ERR_TIMEOUT
STALL_CYCLES = "2000000"  # ~1 ms at 2 GHz


def test_tensor_kernel_wait_timeout_reports_and_recovers(gepi, tmp_path, monkeypatch):
    kw = dict(n_snps=90, n_cases=70, n_controls=64, missing=0.02, n_planted=1, seed=17)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    N, k = fs.n_lines, 120
    want, _, _ = H.oracle_topk(rows, k)
    assert_same_topk(pl.scan(k, method=2), want)  # the kernel is loaded and healthy

    monkeypatch.setenv("GEPI_DEBUG_STALL", STALL_CYCLES)
    for attempt in range(2):  # the error path leaves nothing behind for the next call
        with pytest.raises(gepi.GepiError) as e:
            pl.scan(k, method=2)
        assert e.value.status == TIMEOUT, str(e.value)
        assert "bounded wait" in str(e.value)
    with pytest.raises(gepi.GepiError) as e:
        pl.pair_counts(0, N, 0, N, method=2)
    assert e.value.status == TIMEOUT, str(e.value)
    with pytest.raises(gepi.GepiError) as e:
        gepi.scan_batch([gepi.ScanRequest(pl, k, method=2)])
    assert e.value.status == TIMEOUT, str(e.value)
    monkeypatch.delenv("GEPI_DEBUG_STALL")

    # same plane set, normal budget: exact again, on every entry point
    assert_same_topk(pl.scan(k, method=2), want)
    assert np.array_equal(pl.pair_counts(0, N, 0, N, method=2), H.oracle_pair_gram(rows, 0, N, 0, N))
    (got,) = gepi.scan_batch([gepi.ScanRequest(pl, k, method=2)])
    assert_same_topk(got, want)
    pl.close()
