#!/usr/bin/env python3
"""Benchmark: pair-tests/s of the all-pairs Boolean epistasis scan.

One step = one whole scan of the workload (every SNP pair s > t, all 4 allele-
row pairs x 5 Boolean functions, plus the same-SNP row pairs), ranked top-k on
the device, top-k back on the host.  The default workload is the metric's
configuration: 100,000 SNPs x 10,000 samples (5,000 cases / 5,000 controls),
HWE genotypes with MAF ~ U(0.01, 0.5), 1% missing, 10 planted pairs, top-10,000
-- seeded synthetic data from the package's generator.

  value : pair-tests/s with the genotype planes resident in HBM (CUDA events
          on the library stream around each scan).
  e2e   : the same metric through the public C ABI from a pinned host .bed
          image: H2D copy + device decode + scan + top-k D2H every step, a new
          plane set each step (mean step time; the slowest step is reported).

`--impl reference` times the reference's CPU gold loop (the oracle's
restatement of proc_gold_1.h:68-178 with its lookup-table popcount and 2 x
topmost result buffer, all host threads) on a bounded leading sub-triangle of
the same workload.  That arm never loads the scan library: its input fileset
is written by the stand-alone generator tool (gepi-synth) and read back from
disk.  Under torchrun every rank scans its own cohort (weak scaling: seed +
rank, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CONFIGS = {
    "cfg1": dict(n_snps=1024, n_cases=256, n_controls=256, maf_lo=0.05, maf_hi=0.5, missing=0.02,
                 n_planted=0, seed=1001, k=100),
    "cfg2": dict(n_snps=20000, n_cases=2000, n_controls=2000, maf_lo=0.01, maf_hi=0.5,
                 missing=0.01, n_planted=3, seed=1002, k=1000),
    "cfg3": dict(n_snps=100000, n_cases=5000, n_controls=5000, maf_lo=0.01, maf_hi=0.5,
                 missing=0.01, n_planted=10, seed=1003, k=10000),
    # profiling case: cfg3's sample width on 40,000 SNPs (planes 154 MB, above L2;
    # a scan of ~0.1 s), small enough for full ncu captures
    "prof40k": dict(n_snps=40000, n_cases=5000, n_controls=5000, maf_lo=0.01, maf_hi=0.5,
                    missing=0.01, n_planted=4, seed=1005, k=1000),
}
# Many-request workloads (run by --config cohorts64 / serving).
COHORTS64 = dict(n_cohorts=64, snps=(500, 50000), samples=(200, 20000), case_frac=(0.3, 0.7),
                 missing=0.01, k=1000, seed=1004)
SERVING = dict(n_matrices=8, snps=(5000, 100000), samples=(1000, 10000), missing=0.01,
               ranges=(1000, 50000), ks=(100, 1000, 10000), whole_frac=0.2, seed=1006,
               loads=(0.2, 0.5, 0.8, 1.0))
METRIC = "pair-tests/sec at 100k SNP x 10k samples"
UNIT = "pair-tests/s"


def describe(name: str, c: dict) -> str:
    s = c["n_cases"] + c["n_controls"]
    return (f"{name}: {c['n_snps']:,} SNPs x {s:,} samples ({c['n_cases']:,} cases / "
            f"{c['n_controls']:,} controls), MAF U({c['maf_lo']}, {c['maf_hi']}), "
            f"{c['missing']:.0%} missing, {c['n_planted']} planted pairs, top-{c['k']:,}")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


# DRAM bytes per 80 x 64 tile of tc_tile_kernel at 10,000 samples, from one ncu
# capture of the 40,000-SNP profiling scan (dram__bytes_read.sum +
# dram__bytes_write.sum of its 8 launches / its 156,750 tiles, mean of 5 scans);
# the operand blocks are re-read from L2, so traffic grows with the tiles a
# launch processes and roofline.traffic scales it to the average launch.
TC_DRAM_BYTES_PER_TILE = 51213.0


def synth_fileset(cfg: dict, seed: int) -> str:
    """BASE of the workload's fileset, written once per host by the stand-alone
    generator (no CUDA, no scan library) into the temp directory."""
    import tempfile

    tool = os.path.join(HERE, "gepicount_gb300", "_build", "gepi-synth")
    if not os.path.exists(tool):
        subprocess.run([sys.executable, "-m", "gepicount_gb300.build"], cwd=HERE, check=True,
                       stdout=subprocess.DEVNULL)
    d = os.path.join(tempfile.gettempdir(), "gepi_bench_inputs")
    os.makedirs(d, exist_ok=True)
    base = os.path.join(d, f"n{cfg['n_snps']}_s{cfg['n_cases']}_{cfg['n_controls']}_seed{seed}")
    if not os.path.exists(base + ".fam"):
        args = [str(v) for v in (cfg["n_snps"], cfg["n_cases"], cfg["n_controls"], cfg["maf_lo"],
                                 cfg["maf_hi"], cfg["missing"], cfg["n_planted"],
                                 cfg.get("odds_ratio", 2.0), seed)]
        subprocess.run([tool, base + ".tmp", *args], check=True)
        for ext in ("bed", "bim", "fam"):  # .fam last: its presence marks a complete set
            os.replace(base + ".tmp." + ext, base + "." + ext)
    return base


def cpu_baseline(cfg: dict, bed, ph, target_s: float, threads: int):
    """Time the reference gold loop (oracle restatement) on a leading
    sub-triangle sized to about target_s seconds."""
    sys.path.insert(0, os.path.join(HERE, "tests"))
    import numpy as np

    import helpers as H

    fs = H.Fileset(bed=bed, pheno=ph, n_lines=cfg["n_snps"], bim=[])
    # Decode only the leading rows we need.
    lib = H.oracle()
    nw = (ph.size + 63) // 64
    probe_rows = 256
    n_lines = min(cfg["n_snps"], 20000)
    sub = H.Fileset(bed=bed[: 3 + n_lines * ((ph.size + 3) // 4)], pheno=ph, n_lines=n_lines, bim=[])
    bits, valid, m1, m2 = H.decode_rows(sub)
    chk = H.ctypes.c_double()
    k = cfg["k"]
    t0 = time.perf_counter()
    lib.orc_gold_loop(H.ptr(bits), H.ptr(valid), H.ptr(m1), H.ptr(m2), nw, 0, probe_rows, k,
                      threads, H.ctypes.byref(chk))
    dt = max(time.perf_counter() - t0, 1e-6)
    per_pair = dt / (probe_rows * (probe_rows + 1) / 2)
    want_pairs = target_s / per_pair
    r1 = int(min(2 * n_lines, max(probe_rows, (2 * want_pairs) ** 0.5)))
    t0 = time.perf_counter()
    row_pairs = lib.orc_gold_loop(H.ptr(bits), H.ptr(valid), H.ptr(m1), H.ptr(m2), nw, 0, r1, k,
                                  threads, H.ctypes.byref(chk))
    dt = time.perf_counter() - t0
    snp_pairs = row_pairs / 4.0
    return dict(value=snp_pairs / dt, unit=UNIT, seconds=dt, rows=r1,
                sample=(f"allele rows 0..{r1 - 1} against every row <= them (leading "
                        f"sub-triangle, {row_pairs:,} row pairs = {snp_pairs:,.0f} SNP-pair "
                        f"equivalents) of the same workload: 5 functions, popcount through "
                        f"the reference's 64K lookup table, float entropy, 2 x {k:,} result "
                        f"buffer sorted when full (C restatement of proc_gold_1.h:68-178)"))


def run_reference(args, cfg):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np

    base = synth_fileset(cfg, cfg["seed"])
    bed = np.fromfile(base + ".bed", dtype=np.uint8)
    ph = np.array([int(line.split()[5]) for line in open(base + ".fam") if len(line) >= 5],
                  dtype=np.int32)
    threads = os.cpu_count() or 1
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(cfg, bed, ph, target_s=args.ref_seconds, threads=threads)
        if i >= args.warmup:
            vals.append(r)
    value = statistics.median(v["value"] for v in vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * statistics.median(v["seconds"] for v in vals),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic", "config": {"workload": describe(args.config, cfg)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": vals[-1]["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, cfg):
    import numpy as np
    import torch

    import gepicount_gb300 as g

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    g.lib()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    kw = {k: v for k, v in cfg.items() if k != "k"}
    kw["seed"] = cfg["seed"] + 7919 * rank
    spec = g.SynthSpec(**kw)
    nbytes = g.lib().gepi_synth_bed_bytes(g.ctypes.byref(spec._c()))
    pinned = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    bed = pinned.numpy()
    _, ph, _ = g.synth_bed(spec, out=bed)
    k = cfg["k"]
    method = {"auto": g.METHOD_AUTO, "popc": g.METHOD_POPC, "tensor": g.METHOD_TENSOR}[args.method]
    obj = g.FISHER if args.objective == "fisher" else g.ENTROPY

    planes = g.Planes.from_bed(bed, spec.n_snps, ph, device=local)
    tune = planes.autotune() if method == g.METHOD_AUTO else None
    for _ in range(args.warmup):
        planes.scan(k, method=method, objective=obj)
    barrier()
    stats = []
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            tops = planes.scan(k, method=method, objective=obj)
            stats.append(planes.last_stats())
        barrier()
        wall = time.perf_counter() - t0
    dev_ms = sum(s["scan_ms"] for s in stats)
    pairs_per_scan = stats[0]["snp_pairs"]
    # The plain popcount kernel on the same resident planes (the metric's "vs plain kernel").
    plain = None
    if args.plain_steps > 0 and stats[0]["method"] != g.METHOD_POPC:
        planes.scan(k, method=g.METHOD_POPC, objective=obj)
        pms = []
        for _ in range(args.plain_steps):
            planes.scan(k, method=g.METHOD_POPC, objective=obj)
            pms.append(planes.last_stats()["scan_ms"])
        pmean = sum(pms) / len(pms)
        plain = {"value": world * pairs_per_scan / (pmean / 1000.0), "ms_per_step": pmean,
                 "steps": len(pms)}
    # max over ranks of the device time
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([dev_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
    value = world * pairs_per_scan * args.steps / (dev_ms / 1000.0)
    launches = sum(s["count_launches"] + s["other_launches"] for s in stats)

    # Roofline of the dominant kernel (the counting kernel).  Algorithmic work:
    # 9 bit-products per sample per SNP pair (the 3x3 plane Gram per class),
    # 2 ops per 0/1 multiply-accumulate, over the SNP pairs plus the same-SNP
    # row pairs; per launch = the scan's work / its counting launches.
    n_samples = spec.n_cases + spec.n_controls
    pairs_total = pairs_per_scan + stats[0]["diag_snps"]
    count_ms = sum(s["count_ms"] for s in stats)
    nlaunch = sum(s["count_launches"] for s in stats)
    avg_launch_s = count_ms / 1000.0 / max(1, nlaunch)
    ops_per_launch = 2.0 * 9.0 * n_samples * pairs_total / max(1, stats[0]["count_launches"])
    peaks, peak_kind = measured_peaks()
    achieved = ops_per_launch / avg_launch_s / 1e12
    tensor = stats[0]["method"] == g.METHOD_TENSOR
    fp4_peaks = None
    if tensor:
        # The kernel's instruction is a block-scaled FP4 tcgen05.mma.  The
        # dense rate of every exact FP4 encoding of 0/1 operands is measured
        # live on this GPU (back-to-back MMAs on every SM), and the fastest is
        # the denominator; the bf16 figure is for context.
        fp4_peaks = {kname_: g.tensor_peak_probe(kname_, local) for kname_ in g.PEAK_KINDS}
        best_kind = max(fp4_peaks, key=fp4_peaks.get)
        peak = fp4_peaks[best_kind]
        peak_src = (f"measured live: dense tcgen05.mma rate of the fastest exact FP4 encoding "
                    f"({best_kind}; M=128, N=256, K=64, back-to-back on every SM, best of 3)")
    else:
        peak = float(peaks.get("bf16_tflops", 1900.0))
        peak_src = f"{peak_kind} dense bf16 (burst)"
    kname = "tc_tile_kernel" if tensor else "popc_tile_kernel"
    tiles_per_launch = sum(s["tiles"] for s in stats) / max(1, nlaunch)
    traffic = (TC_DRAM_BYTES_PER_TILE * tiles_per_launch
               if tensor and TC_DRAM_BYTES_PER_TILE and n_samples == 10000 else None)
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "kernel": kname, "peak_source": peak_src,
            "bf16_measured_tflops": float(peaks.get("bf16_tflops", 1900.0)),
            "fp4_peaks_tflops": fp4_peaks,
            "work": "2 x 9 x samples ops per SNP pair (0/1 Gram), per launch",
            "avg_launch_ms": avg_launch_s * 1e3, "launches": nlaunch}
    scan_ms = sorted(s["scan_ms"] for s in stats)

    def pct(q):
        i = min(len(scan_ms) - 1, max(0, int(round(q * (len(scan_ms) - 1)))))
        return scan_ms[i]

    latency = {"p50_ms": pct(0.50), "p99_ms": pct(0.99), "steps": len(scan_ms),
               "what": "device time of one whole scan (first to last launch), per step"}

    # End-to-end through the C ABI from pinned host memory.
    planes.close()
    e2e_times = []
    d2h = k * 48
    for i in range(max(1, args.steps)):
        barrier()
        t1 = time.perf_counter()
        with g.Planes.from_bed(bed, spec.n_snps, ph, device=local) as pl:
            pl.scan(k, method=method, objective=obj)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t1)
    e2e_t = sum(e2e_times) / len(e2e_times)  # mean step time: throughput over the steps
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([e2e_t], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e_value = world * pairs_per_scan / e2e_t

    cpu = None
    # the oracle's CPU gold loop ranks by entropy only
    if rank == 0 and not args.no_cpu_baseline and obj == g.ENTROPY:
        r = cpu_baseline(cfg, bed, ph, target_s=args.cpu_seconds, threads=1)
        cpu = {"value": r["value"], "unit": UNIT, "cores": 1, "kind": "port",
               "sample": r["sample"]}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "e2m1 0/1 operands, f32 accumulate (exact counts)" if tensor else "u32 popcount",
            "data": "synthetic (seeded generator, HWE, planted pairs)",
            "config": {"workload": describe(args.config, cfg), "n_snps": spec.n_snps,
                       "n_samples": n_samples, "k": k, "objective": args.objective,
                       "method": ["auto", "popc", "tensor"][stats[0]["method"]] if args.method == "auto" else args.method,
                       "pair_tests_per_step": pairs_per_scan,
                       "boolean_tests_per_step": 5 * (2 * spec.n_snps) * (2 * spec.n_snps + 1) // 2,
                       "l2": "inputs larger than L2 (genotype planes "
                             f"{3 * spec.n_snps * ((n_samples + 255) // 256) * 32 / 1e6:.0f} MB)"},
            "clocks": clk.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(nbytes),
                    "d2h_bytes_per_step": int(d2h), "seconds_per_step": e2e_t,
                    "steps": len(e2e_times), "max_seconds_per_step": max(e2e_times)},
            "gpu_launches": launches,
            "autotune": tune,
            "plain_kernel": plain,
            "vs_plain": (value / plain["value"]) if plain else None,
            "roofline": roof,
            "latency": latency,
            "cpu_baseline": cpu,
            "wall_s": wall,
            "scan_stats": {k_: v for k_, v in stats[-1].items()},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


def _log_uniform(rng, lo, hi):
    import math

    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def _make_cohort(g, rng, snps, samples, case_frac, missing, seed, device):
    n = _log_uniform(rng, *snps)
    s = max(2, _log_uniform(rng, *samples))
    cases = min(s - 1, max(1, int(round(s * rng.uniform(*case_frac)))))
    spec = g.SynthSpec(n_snps=n, n_cases=cases, n_controls=s - cases, maf_lo=0.01, maf_hi=0.5,
                       missing=missing, n_planted=0, seed=seed)
    bed, ph, _ = g.synth_bed(spec)
    return g.Planes.from_bed(bed, n, ph, device=device), n, s


def run_cohorts(args):
    """64 independent uneven cohorts, each scanned all-pairs top-1,000: one
    gepi_scan_batch call per step against the same scans one after another."""
    import numpy as np
    import torch

    import gepicount_gb300 as g

    c = COHORTS64
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rng = np.random.default_rng(c["seed"] + 7919 * rank)
    cohorts = [_make_cohort(g, rng, c["snps"], c["samples"], c["case_frac"], c["missing"],
                            c["seed"] * 100 + i + 7919 * rank, local)
               for i in range(c["n_cohorts"])]
    obj = g.FISHER if args.objective == "fisher" else g.ENTROPY
    reqs = [g.ScanRequest(pl, c["k"], objective=obj) for pl, _, _ in cohorts]
    tunes = [pl.autotune_variants() for pl, _, _ in cohorts]
    for _ in range(args.warmup):
        g.scan_batch(reqs)
    torch.cuda.synchronize()
    times, stats = [], None
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            outs, stats = g.scan_batch(reqs, with_stats=True)
            times.append(time.perf_counter() - t0)
    batch = g.scan_batch_stats(local)  # launches of the last timed call
    pairs = sum(s_["snp_pairs"] for s_ in stats)
    # the same scans one at a time (direct gepi_scan per cohort)
    seq = []
    for _ in range(max(1, min(args.steps, 2))):
        t0 = time.perf_counter()
        for pl, _, _ in cohorts:
            pl.scan(c["k"], objective=obj)
        seq.append(time.perf_counter() - t0)
    same = all(o.tobytes() == pl.scan(c["k"], objective=obj).tobytes()
               for o, (pl, _, _) in zip(outs, cohorts))
    t_b, t_s = statistics.median(times), statistics.median(seq)
    nsamp = [s for _, _, s in cohorts]
    nsnp = [n for _, n, _ in cohorts]
    line = {
        "metric": "pair-tests/sec, 64 uneven cohorts batched (one gepi_scan_batch per step)",
        "value": world * pairs / t_b, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_b, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed (autotuned per cohort)",
        "data": "synthetic (seeded generator, HWE)",
        "config": {"workload": (f"{c['n_cohorts']} cohorts, SNPs log-U{c['snps']}, samples "
                                f"log-U{c['samples']}, case fraction U{c['case_frac']}, "
                                f"{c['missing']:.0%} missing, top-{c['k']:,} each"),
                   "objective": args.objective, "snps_total": sum(nsnp), "snps_max": max(nsnp), "samples_max": max(nsamp),
                   "pair_tests_per_step": pairs,
                   "variants": {name: sum(t["name"] == name for t in tunes)
                                for name in sorted({t["name"] for t in tunes})}},
        "clocks": clk.summary(),
        "sequential": {"value": world * pairs / t_s, "ms_per_step": 1e3 * t_s,
                       "what": "the same 64 scans as direct gepi_scan calls in turn"},
        "vs_sequential": t_s / t_b,
        "same_results_as_sequential": same,
        "engine": dict(batch, what="one gepi_scan_batch call: engine steps (one graph replay "
                                   "each), persistent counting launches (one per kernel group "
                                   "and step, tiles of every cohort claimed from one work list), "
                                   "batched select launches"),
        "gpu_launches": batch["count_launches"] + batch["select_launches"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for pl, _, _ in cohorts:
        pl.close()
    return 0


def run_serving(args):
    """Poisson stream of scan requests against 8 resident genotype matrices,
    through the serving loop: per-request latency alone, then p50/p99 latency
    and pair-tests/s at offered loads relative to the loop's peak rate."""
    import numpy as np
    import torch

    import gepicount_gb300 as g

    c = SERVING
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    rng = np.random.default_rng(c["seed"] + 7919 * rank)
    mats = [_make_cohort(g, rng, c["snps"], c["samples"], (0.5, 0.5), c["missing"],
                         c["seed"] * 100 + i + 7919 * rank, local)
            for i in range(c["n_matrices"])]
    for pl, _, _ in mats:
        pl.autotune()

    def make_requests(n):
        out = []
        for _ in range(n):
            pl, N, _ = mats[int(rng.integers(len(mats)))]
            k = int(c["ks"][int(rng.integers(len(c["ks"])))])
            if rng.random() < c["whole_frac"]:
                out.append(g.ScanRequest(pl, k))
            else:
                la = min(N, _log_uniform(rng, *c["ranges"]))
                lb = min(N, _log_uniform(rng, *c["ranges"]))
                a0 = int(rng.integers(0, N - la + 1))
                b0 = int(rng.integers(0, N - lb + 1))
                out.append(g.ScanRequest(pl, k, a0=a0, na=la, b0=b0, nb=lb))
        return out

    nreq = max(20, args.requests)
    reqs = make_requests(nreq)

    def pct(v, q):
        v = sorted(v)
        return v[min(len(v) - 1, max(0, int(round(q * (len(v) - 1)))))]

    with g.Server(local) as srv:
        for r in reqs[: min(len(reqs), 3 + args.warmup)]:  # warm-up
            srv.wait(srv.submit(r))
        # alone: one request in the loop at a time
        alone, pairs = [], []
        for r in reqs:
            _, info = srv.wait(srv.submit(r))
            alone.append(info["latency_ms"])
            pairs.append(info["snp_pairs"])
        # peak rate: the whole list submitted at once
        t0 = time.perf_counter()
        tickets = [srv.submit(r) for r in reqs]
        for t in tickets:
            srv.wait(t)
        burst_s = time.perf_counter() - t0
        peak_rps = nreq / burst_s
        levels = []
        with ClockSampler(local) as clk:
            for load in c["loads"]:
                st0 = srv.stats()
                rate = load * peak_rps
                gaps = rng.exponential(1.0 / rate, size=nreq)
                infos = [None] * nreq
                tick = [None] * nreq
                ready = threading.Semaphore(0)

                def waiter():
                    for i in range(nreq):
                        ready.acquire()
                        infos[i] = srv.wait(tick[i])[1]

                th = threading.Thread(target=waiter)
                th.start()
                t0 = time.perf_counter()
                due = t0
                for i, r in enumerate(reqs):
                    due += gaps[i]
                    d = due - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    tick[i] = srv.submit(r)
                    ready.release()
                th.join()
                span = time.perf_counter() - t0
                st1 = srv.stats()
                steps = max(1, st1["steps"] - st0["steps"])
                lat = [x["latency_ms"] for x in infos]
                slow = [x["latency_ms"] / max(a, 1e-3) for x, a in zip(infos, alone)]
                levels.append({
                    "offered_load": load, "offered_rps": rate, "p50_ms": pct(lat, 0.5),
                    "p99_ms": pct(lat, 0.99), "pair_tests_per_s": sum(pairs) / span,
                    "p99_over_alone_p99": pct(lat, 0.99) / pct(alone, 0.99),
                    "slowdown_p50": pct(slow, 0.5), "slowdown_p99": pct(slow, 0.99),
                    "queue_p99_ms": pct([x["queue_ms"] for x in infos], 0.99),
                    # the requests that set the tail: latency, alone, queue (ms), pairs
                    "slowest": [[round(infos[i]["latency_ms"], 1), round(alone[i], 1),
                                 round(infos[i]["queue_ms"], 1), int(pairs[i])]
                                for i in sorted(range(nreq), key=lambda i: -infos[i]["latency_ms"])[:6]],
                    "engine": {"steps": st1["steps"] - st0["steps"],
                               "device_ms_per_step": (st1["device_ms"] - st0["device_ms"]) / steps,
                               "host_ms_per_step": (st1["wall_ms"] - st0["wall_ms"]) / steps,
                               "gpu_busy": (st1["device_ms"] - st0["device_ms"]) / (1e3 * span)}})
    at80 = min(levels, key=lambda L: abs(L["offered_load"] - 0.8))
    line = {
        "metric": "p50/p99 request latency, served mixed stream at 80% of peak offered load",
        "value": at80["p99_ms"], "unit": "ms (p99)", "n_gpus": world, "steps": nreq,
        "warmup": args.warmup, "ms_per_step": at80["p50_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "mixed (autotuned per matrix)",
        "data": "synthetic (seeded generator, HWE)",
        "config": {"workload": (f"{c['n_matrices']} resident matrices (SNPs log-U{c['snps']}, "
                                f"samples log-U{c['samples']}); {nreq} requests, "
                                f"{c['whole_frac']:.0%} whole-genome, others range x range with "
                                f"lengths log-U{c['ranges']}; top-k in {c['ks']}; Poisson "
                                "arrivals"),
                   "matrices": [[n, s] for _, n, s in mats]},
        "clocks": clk.summary(),
        "policy": {"order": os.environ.get("GEPI_SERVE_POLICY", "short"),
                   "slack": float(os.environ.get("GEPI_SERVE_SLACK", "1.5")),
                   "quantum_ms": float(os.environ.get("GEPI_QUANTUM_MS", "4"))},
        "alone": {"p50_ms": pct(alone, 0.5), "p99_ms": pct(alone, 0.99)},
        "peak": {"requests_per_s": peak_rps, "pair_tests_per_s": sum(pairs) / burst_s},
        "levels": levels,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for pl, _, _ in mats:
        pl.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS) + ["cohorts64", "serving"],
                    default="cfg3")
    ap.add_argument("--requests", type=int, default=200,
                    help="requests per offered-load level (--config serving)")
    ap.add_argument("--method", choices=["auto", "popc", "tensor"], default="auto")
    ap.add_argument("--objective", choices=["entropy", "fisher"], default="entropy",
                    help="ranking objective of the scan (the metric is quoted on entropy)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-steps", type=int, default=2,
                    help="timed scans of the plain popcount kernel for vs_plain (0 = skip)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.config in ("cohorts64", "serving"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference scans one "
                              "cohort per process and has no request loop"}), flush=True)
            return 0
        return run_cohorts(args) if args.config == "cohorts64" else run_serving(args)
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        if args.objective == "fisher":
            print(json.dumps({"impl": "reference", "unavailable": "the reference ranks by Fisher "
                              "only on its CUDA path; its CPU gold loop ranks by entropy"}),
                  flush=True)
            return 0
        return run_reference(args, cfg)
    return run_ours(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
