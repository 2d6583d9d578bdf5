"""The `gepi` command line as a drop-in for gEpiCount, against the reference's
own output (golden fixtures made by running the unmodified reference), and the
progress reporting behind its -D option (kernel1.cu:417-439,
proc_gold_1.h:140-163), checked against the oracle."""
import os
import re
import subprocess

import numpy as np
import pytest

import helpers as H
from test_gpu_parity import assert_same_topk, make_planes

pytestmark = pytest.mark.gpu

_QC = re.compile(r"^(Checking data in |Sample \d+:\t|SNP \d+:\t|\d+ Samples checked|"
                 r"\d+ SNPs checked|-?\d+ -?\d+ \S+$)")
SYNTH = ["cfg1", "s63", "s64", "s65", "s129", "miss50", "cfg2_small"]


def run_cli(gepi, *args):
    from gepicount_gb300 import build

    r = subprocess.run([build.CLI, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout, r.stderr


@pytest.mark.parametrize("gold", [False, True], ids=["gpu", "gold_flag"])
@pytest.mark.parametrize("name", SYNTH + ["test", "thinhap1"])
def test_cli_output_matches_reference(gepi, tmp_path, name, gold):
    doc = H.load_golden(name)
    base = H.golden_input(doc, str(tmp_path))
    k = doc["k"]
    out, err = run_cli(gepi, *(["-g"] if gold else []), "-i", base, "-N", str(k))
    # stdout: the reference's lines, verbatim
    assert out.splitlines() == doc["stdout"]
    # QC report: the reference's lines in order (golden made with one OpenMP thread)
    qc = [ln for ln in err.splitlines() if _QC.match(ln)]
    assert qc == doc["qc"]
    # ranked table: the reference's ranking up to near-ties of its float scores
    fs = H.read_fileset(base)
    rows = H.decode_rows(fs)
    got = H.parse_ranked(err)
    assert len(got) == k and [r["rank"] for r in got] == list(range(k))
    want, keys, nranked = H.oracle_topk(rows, k)
    for g_, w in zip(got, want):
        assert (g_["sA"], g_["sB"], g_["fun"]) == (int(w["sA"]), int(w["sB"]), int(w["fun"]))
        n = H.cells_to_n(g_["cells"])
        assert n == tuple(int(v) for v in w["n"])
    if nranked >= k:
        gitems = [(r["sA"], r["sB"], r["fun"]) for r in got]
        ritems = [(r["sA"], r["sB"], r["fun"]) for r in doc["rows"]]
        rkeys = [k_ for k_, _ in H.exact_keys(rows, ritems)]
        probs = H.compare_ranked(gitems, [-float(v) for v in keys], ritems, rkeys, k, rtol=2e-5)
        assert not probs, probs[:5]
        lib = H.oracle()
        for g_, r in zip(got, doc["rows"]):
            if (g_["sA"], g_["sB"], g_["fun"]) == (r["sA"], r["sB"], r["fun"]):
                assert g_["obj"] == pytest.approx(r["obj"], rel=2e-5, abs=1e-7)
                # FPv: R's tie rule (a documented deviation); the reference's strict rule
                # gives the same p except on tables with exactly tied terms
                c = g_["cells"]
                tol = lib.orc_fisher_log10p(c[0], c[1], c[2], c[3], 0)
                strict = lib.orc_fisher_log10p(c[0], c[1], c[2], c[3], 1)
                assert g_["fpv"] == pytest.approx(tol, rel=1e-5, abs=1e-6)
                if abs(tol - strict) <= 1e-9:
                    assert g_["fpv"] == pytest.approx(r["fpv"], rel=1e-5, abs=1e-6)
    tag = "G1" if gold else "K1"
    progress = [ln for ln in err.splitlines() if ln.startswith(f"{tag}: Total time ")]
    assert progress and "(100%)" in progress[-1]
    if gold:
        lim = [ln for ln in err.splitlines() if ln.startswith("G1: Sorting... Limit:")]
        assert len(lim) == 1
        if nranked >= k:
            want_lim = float(doc["g1_limit"][0].split(":")[-1])
            assert float(lim[0].split(":")[-1]) == pytest.approx(want_lim, rel=2e-5)
    else:
        assert "K1: Objective function is ENTROPY" in err


def _snapshots(err: str, tag: str):
    """(last processed row, ranked rows printed after it) for every -D block."""
    out, cur = [], None
    for ln in err.splitlines():
        m = re.match(rf"^{tag}: Last processed: (\d+),(\d+)$", ln)
        if m:
            cur = (int(m.group(1)), [])
            out.append(cur)
            continue
        if cur is not None:
            rr = H.parse_ranked(ln)
            if rr:
                cur[1].extend(rr)
            elif ln.startswith(f"{tag}: Total time") or ln.startswith("process_g"):
                cur = None
    return out


@pytest.mark.parametrize("method", ["popc", "tensor"])
def test_cli_intermediate_results_are_exact(gepi, tmp_path, method):
    """-D prints, at each snapshot, the ranked results of every SNP pair done so
    far: the rows printed equal the oracle's top-k of that leading triangle."""
    doc = H.load_golden("cfg1")
    base = H.golden_input(doc, str(tmp_path))
    fs = H.read_fileset(base)
    rows = H.decode_rows(fs)
    k = 100
    out, err = run_cli(gepi, "-D", "--method", method, "-i", base, "-N", str(k))
    snaps = _snapshots(err, "K1")
    assert len(snaps) >= 2
    for last, printed in snaps:
        assert printed and [r["rank"] for r in printed] == list(range(6))  # stride 1e5, context 5
        want, _, _ = H.oracle_topk_range(rows, 0, last + 1, 0, last + 1, k)
        for p, w in zip(printed, want):
            assert (p["sA"], p["sB"], p["fun"]) == (int(w["sA"]), int(w["sB"]), int(w["fun"]))
            assert H.cells_to_n(p["cells"]) == tuple(int(v) for v in w["n"])
    assert snaps[-1][0] == 2 * fs.n_lines - 1


@pytest.mark.parametrize("method", [1, 2])
def test_progress_snapshots_match_oracle(gepi, tmp_path, method):
    kw = dict(n_snps=900, n_cases=140, n_controls=160, missing=0.02, seed=505)
    pl, rows, fs, _ = make_planes(gepi, kw, tmp_path)
    k = 150
    seen = []
    got = pl.scan_progress(k, seen.append, points=0, with_tops=True, method=method)
    assert got.tobytes() == pl.scan(k, method=method).tobytes()
    assert len(seen) >= 3 and seen[-1]["snps_done"] == 900
    assert [s["tiles_done"] for s in seen] == sorted(s["tiles_done"] for s in seen)
    for s in seen:
        want, _, _ = H.oracle_topk_range(rows, 0, 2 * s["snps_done"], 0, 2 * s["snps_done"], k)
        assert_same_topk(s["tops"], want)
    # without snapshots: the same scan, callbacks carry no results
    seen2 = []
    got2 = pl.scan_progress(k, seen2.append, points=4, method=method)
    assert got2.tobytes() == got.tobytes()
    assert 1 <= len(seen2) <= 5 and all(s["tops"] is None for s in seen2)
    assert seen2[-1]["tiles_done"] == seen2[-1]["tiles_total"]
    pl.close()
