"""The process_gpu_1 shim (integration/process_gpu_1_gb300.cpp) links into an
UNMODIFIED gEpiCount main.

integration/Makefile compiles the reference's src/gEpiCount.cpp and
src/version.cpp as they lie, compiles the shim against the reference's own
inc/gEpiCount.h (its static_asserts pin InteractionResult's layout to
gepi_result's), and links them with libgepi.so in place of the reference's
CUDA objects and fisher_p.c.  The linked program must then behave as gEpiCount:
its gold path (-g, CPU) prints the reference's ranked rows for data/test with
fisher_pval served by the shim, and its GPU path reaches process_gpu_1 in the
shim -- on a host with a GPU it prints the reference's ranking, on a host
without one the shim's error line.  Needs the reference tree
(GEPI_REFERENCE_ROOT); skipped where it is absent, e.g. on the GPU host."""
import os
import subprocess

import pytest

import helpers as H

REF = os.environ.get("GEPI_REFERENCE_ROOT", "")
BIN = os.path.join(H.ROOT, "integration", "_build", "gEpiCount")

pytestmark = pytest.mark.skipif(not (REF and os.path.isdir(os.path.join(REF, "src"))),
                                reason="the reference tree (GEPI_REFERENCE_ROOT) is absent")


@pytest.fixture(scope="module")
def linked(gepi):
    r = subprocess.run(["make", "-s", "-C", os.path.join(H.ROOT, "integration"), f"REF={REF}"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return BIN


def _run(binary, *args):
    r = subprocess.run([binary, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout, r.stderr


def test_shim_links_without_the_reference_gpu_objects(linked):
    syms = subprocess.run(["nm", "-C", linked], capture_output=True, text=True, check=True).stdout
    # the reference's launcher, kernels and device helpers are not in the program
    for name in ("launch_process_gpu_1", "k1_count", "k1_entropy", "k1_fisherpv",
                 "computeBlockGridSize", "mergeResults"):
        assert name not in syms, name
    assert "process_gpu_1(PlinkReader<unsigned long long>" in syms
    deps = subprocess.run(["ldd", linked], capture_output=True, text=True).stdout
    assert "libgepi.so" in deps


@pytest.mark.parametrize("name", ["test", "thinhap1"])
def test_shim_program_matches_reference_gold_output(linked, name, tmp_path):
    doc = H.load_golden(name)
    base = H.golden_input(doc, str(tmp_path))
    out, err = _run(linked, "-g", "-i", base, "-N", str(doc["k"]))
    assert out.splitlines() == doc["stdout"]
    got = H.parse_ranked(err)
    assert len(got) == doc["k"]
    lib = H.oracle()
    for g, w in zip(got, doc["rows"]):
        # the gold loop is the reference's, so the rows are its rows
        assert (g["sA"], g["sB"], g["fun"], g["cells"], g["obj"]) == \
               (w["sA"], w["sB"], w["fun"], tuple(w["cells"]), w["obj"])
        # the FPv column is fisher_pval, now the shim's: R's tie rule (a documented
        # deviation), equal to the reference's strict rule except on tables with
        # exactly tied terms
        c = g["cells"]
        tol = lib.orc_fisher_log10p(c[0], c[1], c[2], c[3], 0)
        strict = lib.orc_fisher_log10p(c[0], c[1], c[2], c[3], 1)
        assert g["fpv"] == pytest.approx(tol, rel=1e-5, abs=1e-6), (g, w)
        if abs(tol - strict) <= 1e-9:
            assert g["fpv"] == pytest.approx(w["fpv"], rel=1e-5, abs=1e-6), (g, w)


def test_shim_program_gpu_path_reaches_the_shim(linked, tmp_path):
    doc = H.load_golden("test")
    base = H.golden_input(doc, str(tmp_path))
    out, err = _run(linked, "-i", base, "-N", str(doc["k"]))
    assert out.splitlines() == doc["stdout"]
    got = H.parse_ranked(err)
    if "E[0]: Error in process_gpu_1 (gepi)" in err:
        # no usable GPU on this host: the shim reported it and left tops zeroed
        assert all(r["cells"] == (0, 0, 0, 0) for r in got)
    else:
        # the ranked rows of the GPU scan: the oracle's exact top-k
        want, _, _ = H.oracle_topk(H.decode_rows(H.read_fileset(base)), doc["k"])
        assert [(r["sA"], r["sB"], r["fun"]) for r in got] == \
               [(int(t["sA"]), int(t["sB"]), int(t["fun"])) for t in want]
