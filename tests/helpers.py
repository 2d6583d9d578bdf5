"""Test helpers: the CPU oracle through ctypes, PLINK fileset parsing and the
reference's ranked-output format.

The oracle (oracle/_build/liboracle.so) is test infrastructure: only tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg load it.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
from dataclasses import dataclass

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

RESULT_DTYPE = np.dtype(
    [
        ("sA", "<i4"),
        ("sB", "<i4"),
        ("_pad0", "<i4", (2,)),
        ("n", "<i4", (4,)),
        ("ent", "<f4"),
        ("fun", "i1"),
        ("_pad1", "i1", (11,)),
    ]
)
assert RESULT_DTYPE.itemsize == 48

FUNC_NAMES = ["AND", "NAND", "ANDN", "NANDN", "XOR"]

_oracle = None


def oracle():
    """Load (building if needed) the CPU oracle shared library."""
    global _oracle
    if _oracle is not None:
        return _oracle
    if not os.path.exists(ORACLE_SO):
        subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    lib = ctypes.CDLL(ORACLE_SO)
    P = ctypes.c_void_p
    i32, i64, f32, f64 = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_double
    lib.orc_decode_bed.argtypes = [P, i32, i32, P, P]
    lib.orc_class_masks.argtypes = [P, i32, P, P]
    lib.orc_binfunc.argtypes = [P, P, P, P, i32, i32, i32, i32, P]
    lib.orc_entropy_ref_f32.argtypes = [i32, i32, i32, i32]
    lib.orc_entropy_ref_f32.restype = f32
    lib.orc_entropy_f64.argtypes = [i32, i32, i32, i32]
    lib.orc_entropy_f64.restype = f64
    lib.orc_tfix_bits.argtypes = [i64]
    lib.orc_tfix_bits.restype = i32
    lib.orc_tfix_table.argtypes = [i64, i32, P]
    lib.orc_entropy_fixed.argtypes = [P, i32, i32, i32, i32, i32, P]
    lib.orc_entropy_fixed.restype = f64
    lib.orc_fisher_log10p.argtypes = [i32, i32, i32, i32, i32]
    lib.orc_fisher_log10p.restype = f64
    lib.orc_pair_gram.argtypes = [P, P, P, P, i32, i32, i32, P]
    lib.orc_scan_topk.argtypes = [P, P, P, P, i32, i32, i32, i32, P, P, i32]
    lib.orc_scan_topk.restype = i64
    lib.orc_scan_topk_range.argtypes = [P, P, P, P, i32, i32, i32, i32, i32, i32, i32, P, P, i32]
    lib.orc_scan_topk_range.restype = i64
    lib.orc_gold_loop.argtypes = [P, P, P, P, i32, i32, i32, i32, i32, P]
    lib.orc_gold_loop.restype = i64
    _oracle = lib
    return lib


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class Fileset:
    """A PLINK fileset in memory: .bed image, phenotypes, .bim rows."""

    bed: np.ndarray  # uint8, header included
    pheno: np.ndarray  # int32 per sample
    n_lines: int
    bim: list  # (chr, id, pos, a1, a2) per line

    @property
    def n_samples(self) -> int:
        return int(self.pheno.size)

    @property
    def n_rows(self) -> int:
        return 2 * self.n_lines

    @property
    def n_words(self) -> int:
        return (self.n_samples + 63) // 64


def read_fileset(base: str) -> Fileset:
    pheno = []
    with open(base + ".fam") as f:
        for line in f:
            line = line.rstrip("\n")
            if len(line) < 5:
                continue
            tok = line.split()
            pheno.append(int(tok[5]))
    bim = []
    with open(base + ".bim") as f:
        for line in f:
            line = line.rstrip("\n")
            if len(line) < 9:
                continue
            tok = line.split()
            bim.append((int(tok[0]), tok[1], int(tok[3]), tok[4][0], tok[5][0]))
    bed = np.fromfile(base + ".bed", dtype=np.uint8)
    return Fileset(bed=bed, pheno=np.asarray(pheno, dtype=np.int32), n_lines=len(bim), bim=bim)


def decode_rows(fs: Fileset):
    """Oracle decode: (bits, valid, mask1, mask2) as the reference's rows."""
    lib = oracle()
    nw = fs.n_words
    bits = np.zeros((fs.n_rows, nw), dtype=np.uint64)
    valid = np.zeros((fs.n_rows, nw), dtype=np.uint64)
    m1 = np.zeros(nw, dtype=np.uint64)
    m2 = np.zeros(nw, dtype=np.uint64)
    lib.orc_decode_bed(ptr(fs.bed), fs.n_lines, fs.n_samples, ptr(bits), ptr(valid))
    lib.orc_class_masks(ptr(fs.pheno), fs.n_samples, ptr(m1), ptr(m2))
    return bits, valid, m1, m2


def oracle_topk(rows, k: int, objective: int = 0, threads: int = 0):
    """Exact oracle top-k -> (results structured array, double objective)."""
    bits, valid, m1, m2 = rows
    lib = oracle()
    tops = np.zeros(k, dtype=RESULT_DTYPE)
    keys = np.zeros(k, dtype=np.float64)
    n = lib.orc_scan_topk(ptr(bits), ptr(valid), ptr(m1), ptr(m2), bits.shape[0], bits.shape[1],
                          objective, k, ptr(tops), ptr(keys), threads)
    return tops, keys, int(n)


def oracle_topk_range(rows, ra0, ra1, rb0, rb1, k: int, objective: int = 0, threads: int = 0):
    bits, valid, m1, m2 = rows
    lib = oracle()
    tops = np.zeros(k, dtype=RESULT_DTYPE)
    keys = np.zeros(k, dtype=np.float64)
    n = lib.orc_scan_topk_range(ptr(bits), ptr(valid), ptr(m1), ptr(m2), bits.shape[1], ra0, ra1,
                                rb0, rb1, objective, k, ptr(tops), ptr(keys), threads)
    return tops, keys, int(n)


def oracle_pair_gram(rows, s0, ns, t0, nt):
    bits, valid, m1, m2 = rows
    lib = oracle()
    out = np.zeros((ns, nt, 18), dtype=np.uint32)
    tmp = np.zeros(18, dtype=np.uint32)
    for i in range(ns):
        for j in range(nt):
            lib.orc_pair_gram(ptr(bits), ptr(valid), ptr(m1), ptr(m2), bits.shape[1], s0 + i,
                              t0 + j, ptr(tmp))
            out[i, j] = tmp
    return out


# ---- the reference's ranked output (src/misc/print_misc.h:59,74) ----------
_ROW = re.compile(
    r"^(\d+):\t(\d+)\[(\S+) (\S+) (-?\d+):(-?\d+)\]\t(\w+)\t(\d+)\[(\S+) (\S+) (-?\d+):(-?\d+)\]"
    r"\t(\S+)\t(\S+)\t\((-?\d+),(-?\d+),(-?\d+),(-?\d+)\)$"
)


def parse_ranked(text: str):
    """Parse printInteractions rows into dicts (rank, sA, sB, fun, obj, fpv, cells)."""
    out = []
    for line in text.splitlines():
        m = _ROW.match(line)
        if not m:
            continue
        g = m.groups()
        out.append(
            dict(
                rank=int(g[0]),
                sA=int(g[1]),
                sB=int(g[7]),
                fun=FUNC_NAMES.index(g[6]) if g[6] in FUNC_NAMES else -1,
                obj=float(g[12]),
                fpv=float(g[13]),
                cells=tuple(int(v) for v in g[14:18]),
            )
        )
    return out


def cells_to_n(cells):
    """(c0on, c0off, c1on, c1off) -> InteractionResult.n (w, x, y, z)."""
    a, b, c, d = cells
    return (a, c, a + b, c + d)


# ---- golden fixtures -----------------------------------------------------
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference's demo filesets (data/test, data/thinhap1), copied byte for byte
# by make_golden.py
GOLDEN_DATA_DIR = os.path.join(GOLDEN_DIR, "data")


def load_golden(name: str) -> dict:
    import json

    with open(os.path.join(GOLDEN_DIR, f"gold_{name}.json")) as f:
        return json.load(f)


def golden_names():
    return sorted(f[5:-5] for f in os.listdir(GOLDEN_DIR) if f.startswith("gold_") and f.endswith(".json"))


def golden_input(doc: dict, tmpdir: str):
    """Fileset base path for a golden case: regenerated if synthetic, else the
    reference's demo fileset committed under tests/golden/data/."""
    import hashlib

    if doc["kind"] == "synthetic":
        import gepicount_gb300 as g

        base = os.path.join(tmpdir, doc["case"])
        g.synth_write(g.SynthSpec(**doc["spec"]), base)
    else:
        base = os.path.join(GOLDEN_DATA_DIR, doc["case"])
    for ext, h in doc["sha256"].items():
        got = hashlib.sha256(open(base + "." + ext, "rb").read()).hexdigest()
        assert got == h, f"{base}.{ext}: input differs from the one the golden was made from"
    return base


def exact_keys(rows, items, objective: int = 0):
    """Oracle objective (I bits, or -log10 p) and counts for (sA, sB, fun) items."""
    bits, valid, m1, m2 = rows
    lib = oracle()
    nmax = int(sum(bin(int(v)).count("1") for v in m1) + sum(bin(int(v)).count("1") for v in m2))
    F = lib.orc_tfix_bits(nmax)
    T = np.zeros(nmax + 1, dtype=np.uint64)
    lib.orc_tfix_table(nmax, F, ptr(T))
    out = []
    c = np.zeros(4, dtype=np.int32)
    nz = ctypes.c_int()
    for sA, sB, fun in items:
        lib.orc_binfunc(ptr(bits), ptr(valid), ptr(m1), ptr(m2), bits.shape[1], int(sA), int(sB),
                        int(fun), ptr(c))
        w, x, y, z = (int(v) for v in c)
        if objective == 0:
            key = lib.orc_entropy_fixed(ptr(T), F, w, x, y, z, ctypes.byref(nz))
        else:
            key = -lib.orc_fisher_log10p(w, y - w, x, z - x, 0)
        out.append((key, (w, x, y, z)))
    return out


def compare_ranked(got_items, got_keys, ref_items, ref_keys, k, rtol):
    """Compare two ranked lists allowing reorderings/swaps among entries whose
    keys agree within rtol (near-ties) -- used against the reference's float
    ranking.  Items are (sA, sB, fun) tuples; keys larger = better.
    Returns a list of problems (empty = equivalent)."""
    problems = []
    n = min(len(got_items), len(ref_items), k)
    kth = min(got_keys[n - 1], ref_keys[n - 1])
    def close(a, b):
        return abs(a - b) <= rtol * max(abs(a), abs(b)) + 1e-12
    gset, rset = set(got_items[:n]), set(ref_items[:n])
    for it in gset - rset:
        i = got_items.index(it)
        if not close(got_keys[i], kth):
            problems.append(f"extra {it} key {got_keys[i]} (k-th {kth})")
    for it in rset - gset:
        i = ref_items.index(it)
        if not close(ref_keys[i], kth):
            problems.append(f"missing {it} key {ref_keys[i]} (k-th {kth})")
    for i in range(n):
        if not close(got_keys[i], ref_keys[i]):
            problems.append(f"rank {i}: key {got_keys[i]} vs {ref_keys[i]}")
            break
    return problems
