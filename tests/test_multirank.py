"""The multi-rank path on CPU: two gloo ranks each take one shard of the
whole-genome triangle (gepi_shard_range), rank 0 gathers the per-shard ranked
lists and merges them with gepi_merge_results (host only).  The per-shard
lists come from the oracle, so no GPU is needed; the merged list must equal the
oracle's whole-triangle top-k, bit for bit for entropy."""
import os
import socket

import numpy as np
import pytest

import helpers as H

WORLD = 2


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, base, k, objective, out_dir):
    import torch.distributed as dist

    import gepicount_gb300 as g

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        fs = H.read_fileset(base)
        rows = H.decode_rows(fs)
        a0, na, b0, nb = g.shard_range(fs.n_lines, WORLD, rank)
        part, _, _ = H.oracle_topk_range(rows, 2 * a0, 2 * (a0 + na), 2 * b0, 2 * (b0 + nb), k,
                                        objective=objective)
        parts = [None] * WORLD
        dist.all_gather_object(parts, part.tobytes())
        if rank == 0:
            lists = [np.frombuffer(p, dtype=g.RESULT_DTYPE) for p in parts]
            n_samples = int(np.count_nonzero((fs.pheno == 1) | (fs.pheno == 2)))
            merged = g.merge_results(lists, k, n_samples, objective)
            np.save(os.path.join(out_dir, "merged.npy"), merged.view(np.uint8))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("objective", [0, 1], ids=["entropy", "fisher"])
def test_two_rank_shards_merge_to_whole_scan(gepi, tmp_path, objective, monkeypatch):
    import torch.multiprocessing as mp

    here = os.path.dirname(os.path.abspath(__file__))
    # spawned ranks import this module and the helpers by name
    monkeypatch.setenv("PYTHONPATH", os.pathsep.join(
        [here, os.path.dirname(here), os.environ.get("PYTHONPATH", "")]))
    doc = H.load_golden("cfg1")
    base = H.golden_input(doc, str(tmp_path))
    k = 100
    mp.start_processes(_rank_main, args=(_free_port(), base, k, objective, str(tmp_path)),
                       nprocs=WORLD, join=True, start_method="spawn")
    merged = np.load(os.path.join(str(tmp_path), "merged.npy")).view(gepi.RESULT_DTYPE)
    fs = H.read_fileset(base)
    rows = H.decode_rows(fs)
    want, keys, _ = H.oracle_topk(rows, k, objective=objective)
    if objective == 0:
        assert merged.tobytes() == want.tobytes()
    else:
        got_items = [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in merged]
        ex = H.exact_keys(rows, got_items, objective=1)
        probs = H.compare_ranked(got_items, [k_ for k_, _ in ex],
                                 [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in want],
                                 [-float(v) for v in keys], k, rtol=1e-8)
        assert not probs, probs[:5]


def test_shard_ranges_partition_the_triangle(gepi):
    for n in (1, 5, 97, 1000, 100000):
        for shards in (1, 2, 3, 7, 8):
            covered, prev_end = 0, 0
            for s in range(shards):
                a0, na, b0, nb = gepi.shard_range(n, shards, s)
                assert a0 == prev_end and b0 == 0 and nb == a0 + na
                covered += sum(min(a + 1, b0 + nb) - b0 for a in range(a0, a0 + na)) if n < 2000 else 0
                prev_end = a0 + na
            assert prev_end == n
            if n < 2000:
                assert covered == n * (n + 1) // 2  # pairs t <= s, the diagonal included
    with pytest.raises(gepi.GepiError):
        gepi.shard_range(10, 2, 2)


def test_merge_rejects_inconsistent_counts(gepi):
    bad = np.zeros(1, dtype=gepi.RESULT_DTYPE)
    bad["n"] = (5, 1, 3, 4)  # w > y
    with pytest.raises(gepi.GepiError):
        gepi.merge_results([bad], 10, 100)
    empty = gepi.merge_results([], 5, 100)
    assert not np.frombuffer(empty.tobytes(), np.uint8).any()
