"""The bench's reference arm runs on host cores and prints one JSON line with
the fields the bench contract names (the arm's own cpu_baseline and an e2e
block with no host-device copies)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--config", "cfg1", "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"].startswith("pair-tests/sec")
    assert d["unit"] == "pair-tests/s" and d["value"] > 0
    assert d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 3 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"].startswith("cfg1")


def _reference_line(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        *args], capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_unavailable_where_the_reference_has_no_counterpart():
    """The reference's CPU gold loop ranks by entropy and scans one cohort per
    process: the Fisher, cohort and serving arms print one `unavailable` line
    and exit 0 without running anything."""
    for args in (("--config", "cfg2", "--objective", "fisher"), ("--config", "cohorts64"),
                 ("--config", "serving")):
        d = _reference_line(*args)
        assert d["impl"] == "reference" and d["unavailable"], args
        assert set(d) == {"impl", "unavailable"}, args
