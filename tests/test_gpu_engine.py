"""The scan engine: many requests at once (gepi_scan_batch) and the serving
loop (gepi_server_*).  Every request's results must equal, bit for bit, the
direct gepi_scan_range call with the same arguments, and the oracle's."""
import threading
import time

import numpy as np
import pytest

import helpers as H
from test_gpu_parity import assert_same_topk, make_planes

pytestmark = pytest.mark.gpu

COHORTS = [
    dict(n_snps=120, n_cases=160, n_controls=140, missing=0.02, seed=41),
    dict(n_snps=75, n_cases=33, n_controls=31, missing=0.10, seed=42),
    dict(n_snps=200, n_cases=150, n_controls=170, missing=0.03, n_planted=2, seed=43),
]


def _cohorts(gepi, tmp_path):
    out = []
    for i, kw in enumerate(COHORTS):
        pl, rows, fs, _ = make_planes(gepi, kw, tmp_path, f"c{i}")
        out.append((pl, rows))
    return out


def _requests(gepi, cohorts):
    """Whole sets and ranges, both objectives, both counting methods."""
    (p0, _), (p1, _), (p2, _) = cohorts
    R = gepi.ScanRequest
    return [
        R(p0, 200),
        R(p1, 90, method=1),
        R(p2, 300, method=2),
        R(p0, 150, a0=40, na=60, b0=5, nb=50, method=2),
        R(p2, 120, objective=gepi.FISHER, method=1),
        R(p1, 64, a0=7, na=1, b0=7, nb=1),
        R(p2, 250, a0=90, na=30, b0=0, nb=120, method=1),
        R(p0, 10, a0=10, na=0, b0=0, nb=10),  # empty range
    ]


def _direct(r):
    if r.na < 0:
        return r.planes.scan_range(0, r.planes.n_snps, 0, r.planes.n_snps, r.k,
                                   objective=r.objective, method=r.method, variant=r.variant)
    return r.planes.scan_range(r.a0, r.na, r.b0, r.nb, r.k, objective=r.objective,
                               method=r.method, variant=r.variant)


def _oracle(r, rows):
    n = r.planes.n_snps
    a0, na, b0, nb = (0, n, 0, n) if r.na < 0 else (r.a0, r.na, r.b0, r.nb)
    want, _, _ = H.oracle_topk_range(rows, 2 * a0, 2 * (a0 + na), 2 * b0, 2 * (b0 + nb), r.k,
                                     objective=r.objective)
    return want


def test_batch_matches_direct_and_oracle(gepi, tmp_path):
    cohorts = _cohorts(gepi, tmp_path)
    rows_of = {id(pl): rows for pl, rows in cohorts}
    reqs = _requests(gepi, cohorts)
    got, stats = gepi.scan_batch(reqs, with_stats=True)
    for r, g, st in zip(reqs, got, stats):
        d = _direct(r)
        assert g.tobytes() == d.tobytes()
        ds = r.planes.last_stats()
        assert st["snp_pairs"] == ds["snp_pairs"] and st["tiles"] == ds["tiles"]
        assert st["method"] == ds["method"]
        if r.objective == gepi.ENTROPY:
            assert_same_topk(g, _oracle(r, rows_of[id(r.planes)]))
    assert not np.frombuffer(got[-1].tobytes(), np.uint8).any()  # empty range: zero-filled
    for pl, _ in cohorts:
        pl.close()


@pytest.mark.parametrize("cap", ["4096", "20000"])
def test_batch_exact_under_candidate_overflow(gepi, tmp_path, cap, monkeypatch):
    cohorts = _cohorts(gepi, tmp_path)
    rows_of = {id(pl): rows for pl, rows in cohorts}
    R = gepi.ScanRequest
    reqs = [R(cohorts[2][0], 300, method=1), R(cohorts[2][0], 300, method=2),
            R(cohorts[0][0], 300, method=2), R(cohorts[1][0], 200, method=1)]
    monkeypatch.setenv("GEPI_DEBUG_CAP", cap)
    got, stats = gepi.scan_batch(reqs, with_stats=True)
    monkeypatch.delenv("GEPI_DEBUG_CAP")
    assert sum(s["overflows"] for s in stats) > 0
    for r, g in zip(reqs, got):
        assert_same_topk(g, _oracle(r, rows_of[id(r.planes)]))
    for pl, _ in cohorts:
        pl.close()


@pytest.mark.parametrize("policy", ["deadline", "short", "oldest"])
@pytest.mark.parametrize("budget", [0, 1])
def test_server_same_result_alone_and_mixed(gepi, tmp_path, budget, policy, monkeypatch):
    """A request gives the same results served alone as among others
    submitted concurrently from several threads (budget 1 byte: one request
    admitted at a time; 0: the default budget, all together), under every
    scheduling policy and a 1 ms batch quantum; the server's counters add up."""
    monkeypatch.setenv("GEPI_SERVE_POLICY", policy)
    monkeypatch.setenv("GEPI_QUANTUM_MS", "1")
    cohorts = _cohorts(gepi, tmp_path)
    reqs = _requests(gepi, cohorts)
    with gepi.Server(0, budget) as srv:
        alone = []
        for r in reqs:
            tops, info = srv.wait(srv.submit(r))
            assert info["latency_ms"] >= info["queue_ms"] >= 0.0
            alone.append(tops)
        mixed = [None] * len(reqs)
        infos = [None] * len(reqs)

        def client(idx):
            for i in idx:
                t = srv.submit(reqs[i])
                mixed[i], infos[i] = srv.wait(t)

        order = list(range(len(reqs)))
        threads = [threading.Thread(target=client, args=(order[j::3],)) for j in range(3)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        # and all at once from one thread
        tickets = [srv.submit(r) for r in reversed(reqs)]
        burst = [srv.wait(t)[0] for t in tickets][::-1]
        time.sleep(0.05)  # the loop copies its counters before it next sleeps
        st = srv.stats()
    assert st["steps"] >= len(reqs) // 2
    assert st["graph_launches"] == st["steps"]
    assert st["select_launches"] == 20 * st["steps"]
    assert 0.0 < st["device_ms"] <= st["wall_ms"]
    for r, a, m, b in zip(reqs, alone, mixed, burst):
        d = _direct(r)
        assert a.tobytes() == d.tobytes()
        assert m.tobytes() == d.tobytes()
        assert b.tobytes() == d.tobytes()
    _, stats = gepi.scan_batch(reqs, with_stats=True)
    for info, st in zip(infos, stats):
        assert info["snp_pairs"] == st["snp_pairs"] and info["method"] == st["method"]
    for pl, _ in cohorts:
        pl.close()


def test_server_and_batch_reject_bad_requests(gepi, tmp_path):
    pl, _, _, _ = make_planes(gepi, COHORTS[1], tmp_path)
    R = gepi.ScanRequest
    with gepi.Server(0) as srv:
        for bad in (R(pl, 0), R(pl, 10, objective=7), R(pl, 10, method=9),
                    R(pl, 10, a0=70, na=10, b0=0, nb=5)):
            with pytest.raises(gepi.GepiError) as e:
                srv.submit(bad)
            assert e.value.status == 1
            with pytest.raises(gepi.GepiError):
                gepi.scan_batch([R(pl, 5), bad])
        with pytest.raises(gepi.GepiError):
            srv.wait(12345)
        # the server still serves after the rejections
        tops, _ = srv.wait(srv.submit(R(pl, 20)))
        assert tops.tobytes() == pl.scan(20).tobytes()
    pl.close()


def test_batch_of_many_cohorts(gepi):
    """Sixteen seeded cohorts of uneven sizes in one call, each equal to its
    direct scan."""
    pls = []
    for i in range(16):
        spec = gepi.SynthSpec(n_snps=100 + 37 * i, n_cases=60 + 11 * i, n_controls=90 + 5 * i,
                              missing=0.02, n_planted=1, seed=500 + i)
        bed, ph, _ = gepi.synth_bed(spec)
        pls.append(gepi.Planes.from_bed(bed, spec.n_snps, ph))
    reqs = [gepi.ScanRequest(p, 100, method=1 + (i % 2)) for i, p in enumerate(pls)]
    got = gepi.scan_batch(reqs)
    for r, g in zip(reqs, got):
        assert g.tobytes() == _direct(r).tobytes()
    for p in pls:
        p.close()


@pytest.mark.parametrize("shards", [2, 3, 5])
@pytest.mark.parametrize("objective", [0, 1], ids=["entropy", "fisher"])
def test_sharded_scan_merges_to_whole_scan(gepi, tmp_path, shards, objective):
    """Shard scans on the device (gepi_shard_range + scan_range), merged on the
    host, equal the whole-triangle scan."""
    pl, rows, fs, _ = make_planes(gepi, COHORTS[2], tmp_path)
    k = 300
    parts = []
    for s in range(shards):
        a0, na, b0, nb = gepi.shard_range(pl.n_snps, shards, s)
        parts.append(pl.scan_range(a0, na, b0, nb, k, objective=objective))
    n0, n1 = pl.class_sizes()
    merged = gepi.merge_results(parts, k, n0 + n1, objective)
    whole = pl.scan(k, objective=objective)
    if objective == 0:
        assert merged.tobytes() == whole.tobytes()
    else:
        items = lambda t: [(int(r["sA"]), int(r["sB"]), int(r["fun"])) for r in t]
        gk = [-float(r["ent"]) for r in merged]
        wk = [-float(r["ent"]) for r in whole]
        probs = H.compare_ranked(items(merged), gk, items(whole), wk, k, rtol=1e-6)
        assert not probs, probs[:5]
    pl.close()


def test_batch_runs_one_counting_launch_per_step(gepi):
    """Many cohorts of one kernel group: every engine step is one graph replay
    holding ONE persistent counting launch over all of them (tiles claimed from
    one work list with an atomic counter) and one chain of 20 batched select
    launches; every list equals its direct scan."""
    pls = []
    for i in range(12):
        spec = gepi.SynthSpec(n_snps=300 + 53 * i, n_cases=200 + 97 * i, n_controls=300 + 31 * i,
                              missing=0.02, n_planted=1, seed=700 + i)
        bed, ph, _ = gepi.synth_bed(spec)
        pls.append(gepi.Planes.from_bed(bed, spec.n_snps, ph))
    reqs = [gepi.ScanRequest(p, 150, variant=4) for p in pls]
    got, stats = gepi.scan_batch(reqs, with_stats=True)
    bs = gepi.scan_batch_stats(0)
    assert bs["steps"] >= max(s["batches"] for s in stats)
    assert 1 <= bs["count_launches"] <= bs["steps"]
    assert bs["select_launches"] == 20 * bs["steps"]
    assert bs["graph_launches"] == bs["steps"]
    for r, g, st in zip(reqs, got, stats):
        assert g.tobytes() == _direct(r).tobytes()
        assert st["variant"] == 4 and st["count_launches"] <= bs["count_launches"]
    for p in pls:
        p.close()


def test_batch_mixes_variants_and_objectives(gepi):
    """Requests of every counting variant and both objectives in one call: one
    counting launch per (kernel group) and step, every list byte-identical to
    its direct scan."""
    pls = []
    for i in range(4):
        spec = gepi.SynthSpec(n_snps=150 + 40 * i, n_cases=150 + 60 * i, n_controls=170 + 20 * i,
                              missing=0.03, n_planted=1, seed=800 + i)
        bed, ph, _ = gepi.synth_bed(spec)
        pls.append(gepi.Planes.from_bed(bed, spec.n_snps, ph))
    reqs = []
    for i, p in enumerate(pls):
        for v in (1, 2, 3, 4):
            reqs.append(gepi.ScanRequest(p, 120, variant=v, objective=(i + v) % 2))
    reqs.append(gepi.ScanRequest(pls[0], 90, a0=20, na=60, b0=10, nb=70, variant=3))
    got, stats = gepi.scan_batch(reqs, with_stats=True)
    bs = gepi.scan_batch_stats(0)
    assert bs["count_launches"] <= 5 * bs["steps"]
    for r, g, st in zip(reqs, got, stats):
        assert g.tobytes() == _direct(r).tobytes(), (r.variant, r.objective)
        assert st["variant"] == r.variant
    for p in pls:
        p.close()
