"""Generate golden fixtures from the UNMODIFIED reference gEpiCount gold path.

    GEPI_REFERENCE_ROOT=<reference tree> python tests/golden/make_golden.py
    python tests/golden/make_golden.py --ref <reference tree>

Builds the reference with oracle/Makefile.ref into oracle/_ref/ (x86 build
here; never shipped), writes seeded synthetic PLINK filesets with this
package's generator, runs ``gEpiCount -g -i BASE -N k`` on each and stores
the ranked rows it prints (src/misc/print_misc.h:59-78) plus the sha256 of the
input files, so a test can regenerate the same input on any host and check it
is byte-identical before comparing.  The reference's own demo filesets
(data/test: 2 SNPs x 6 samples, the known answer of README.txt; data/thinhap1:
1,020 SNPs x 89 samples) are copied byte for byte into tests/golden/data/, so
the tests run them on hosts without the reference tree (the GPU host).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import gepicount_gb300 as g  # noqa: E402
from helpers import parse_ranked  # noqa: E402

SYNTH_CASES = {
    # config-1 shape: 1,024 SNPs x 512 samples (256/256), MAF U(0.05,0.5), 2% missing
    "cfg1": (dict(n_snps=1024, n_cases=256, n_controls=256, maf_lo=0.05, maf_hi=0.5,
                  missing=0.02, seed=1001), 100),
    # config-2 generator (MAF U(0.01,0.5), 1% missing, 3 planted pairs) at 1,000 SNPs x 4,000
    "cfg2_small": (dict(n_snps=1000, n_cases=2000, n_controls=2000, maf_lo=0.01, maf_hi=0.5,
                        missing=0.01, n_planted=3, odds_ratio=2.0, seed=1002), 1000),
    # word-boundary sample counts
    "s63": (dict(n_snps=48, n_cases=31, n_controls=32, missing=0.02, seed=63), 200),
    "s64": (dict(n_snps=48, n_cases=32, n_controls=32, missing=0.02, seed=64), 200),
    "s65": (dict(n_snps=48, n_cases=33, n_controls=32, missing=0.02, seed=65), 200),
    "s129": (dict(n_snps=70, n_cases=100, n_controls=29, missing=0.05, seed=129), 300),
    # heavy missingness, tiny cohort
    "miss50": (dict(n_snps=33, n_cases=9, n_controls=11, missing=0.5, seed=50), 150),
}
REF_CASES = {"test": ("data/test", 10), "thinhap1": ("data/thinhap1", 200)}
DATA_DIR = os.path.join(HERE, "data")


def sha(path: str) -> str:
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


_QC = re.compile(r"^(Checking data in |Sample \d+:\t|SNP \d+:\t|\d+ Samples checked|"
                 r"\d+ SNPs checked|-?\d+ -?\d+ \S+$)")


def run_gold(gold: str, base: str, k: int):
    """Ranked rows, stdout, the QC report lines (PlinkReader.h:237-335) and the final
    "G1: Sorting... Limit:" line.  One OpenMP thread: the QC report's periodic lines come
    from thread 0's chunk only, so a single chunk makes the report complete and ordered."""
    r = subprocess.run([gold, "-g", "-i", base, "-N", str(k)], capture_output=True, text=True,
                       check=True, env=dict(os.environ, OMP_NUM_THREADS="1"))
    lines = r.stderr.splitlines()
    qc = [ln for ln in lines if _QC.match(ln)]
    limit = [ln for ln in lines if ln.startswith("G1: Sorting... Limit:")]
    return parse_ranked(r.stderr), r.stdout, qc, limit[-1:]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GEPI_REFERENCE_ROOT"),
                    help="root of the reference tree (default: $GEPI_REFERENCE_ROOT)")
    args = ap.parse_args()
    if not args.ref or not os.path.isdir(args.ref):
        ap.error("give the reference tree with --ref or GEPI_REFERENCE_ROOT")
    out_ref = os.path.join(ROOT, "oracle", "_ref")
    gold = os.path.join(out_ref, "gEpiCount")
    if not os.path.exists(gold):
        subprocess.run(["make", "-s", "-f", os.path.join(ROOT, "oracle", "Makefile.ref"),
                        f"REF={args.ref}", f"OUT={out_ref}", "-j8"], check=True)
    from gepicount_gb300 import build as gbuild
    gbuild.build()
    with tempfile.TemporaryDirectory() as td:
        for name, (kw, k) in SYNTH_CASES.items():
            spec = g.SynthSpec(**kw)
            base = os.path.join(td, name)
            g.synth_write(spec, base)
            rows, stdout, qc, limit = run_gold(gold, base, k)
            doc = dict(case=name, kind="synthetic", spec=kw, k=k,
                       sha256={e: sha(base + "." + e) for e in ("bed", "bim", "fam")},
                       stdout=stdout.splitlines(), rows=rows, qc=qc, g1_limit=limit)
            with open(os.path.join(HERE, f"gold_{name}.json"), "w") as f:
                json.dump(doc, f, indent=0)
            print(name, len(rows))
    os.makedirs(DATA_DIR, exist_ok=True)
    for name, (rel, k) in REF_CASES.items():
        base = os.path.join(args.ref, rel)
        for ext in ("bed", "bim", "fam"):
            shutil.copyfile(base + "." + ext, os.path.join(DATA_DIR, name + "." + ext))
        rows, stdout, qc, limit = run_gold(gold, base, k)
        doc = dict(case=name, kind="reference-data", path=rel, k=k,
                   sha256={e: sha(base + "." + e) for e in ("bed", "bim", "fam")},
                   stdout=stdout.splitlines(), rows=rows, qc=qc, g1_limit=limit)
        with open(os.path.join(HERE, f"gold_{name}.json"), "w") as f:
            json.dump(doc, f, indent=0)
        print(name, len(rows))


if __name__ == "__main__":
    main()
