"""gepicount_gb300 -- GB300-native pairwise Boolean epistasis scan.

Python host mirror of gEpiCount's interface over the C ABI in include/gepi.h
(libgepi.so, built by ``python -m gepicount_gb300.build``):

* ``BinPlinkReader(base)`` -- the reader (src/reader/BinPlinkReader.h): parses
  BASE.fam/.bim/.bed with the reference's semantics.
* ``Params`` -- struct _paramP1 (inc/gEpiCount.h:116-132).
* ``process_gpu_1(reader, tops, par)`` -- the reference's GPU entry point
  (src/kernels/kernel1.cu:508-511): fills ``tops`` (a RESULT_DTYPE array of
  length par.topmost, the InteractionResult layout) ascending by objective.
* ``Planes`` -- device-resident genotype bit-planes, decoded on the GPU from a
  .bed image; ``Planes.scan`` / ``scan_range`` / ``pair_counts``.

There is no CPU fallback: every compute call goes through the CUDA library and
raises ``GepiError`` if it is missing or fails.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "GepiError", "RESULT_DTYPE", "FUNC_NAMES", "Params", "BinPlinkReader", "Planes",
    "process_gpu_1", "process_gpu_1_noalloc", "fisher_pval", "fisher_log10p", "SynthSpec", "synth_bed", "synth_write",
    "library_path", "lib", "ScanRequest", "scan_batch", "Server", "shard_range", "merge_results",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_PKG, "_build", "libgepi.so")

RESULT_DTYPE = np.dtype(
    [("sA", "<i4"), ("sB", "<i4"), ("_pad0", "<i4", (2,)), ("n", "<i4", (4,)), ("ent", "<f4"),
     ("fun", "i1"), ("_pad1", "i1", (11,))]
)
assert RESULT_DTYPE.itemsize == 48

FUNC_NAMES = ["AND", "NAND", "ANDN", "NANDN", "XOR"]
ENTROPY, FISHER = 0, 1
METHOD_AUTO, METHOD_POPC, METHOD_TENSOR = 0, 1, 2

_STATUS = {
    0: "ok", 1: "invalid argument", 2: "i/o error", 3: "format error", 4: "CUDA error",
    5: "out of device memory", 6: "phenotype class 1 or 2 is empty", 7: "device wait timed out",
    8: "unsupported", 9: "request beyond a documented limit",
}


class GepiError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS.get(status, status)}: {message}")
        self.status = status


class _Params(ctypes.Structure):
    _fields_ = [("gpu_num", ctypes.c_int32), ("topmost", ctypes.c_int32),
                ("objective", ctypes.c_int32), ("method", ctypes.c_int32),
                ("verbose", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 6)]


class _SynthSpec(ctypes.Structure):
    _fields_ = [("n_snps", ctypes.c_int32), ("n_cases", ctypes.c_int32),
                ("n_controls", ctypes.c_int32), ("maf_lo", ctypes.c_double),
                ("maf_hi", ctypes.c_double), ("missing", ctypes.c_double),
                ("n_planted", ctypes.c_int32), ("odds_ratio", ctypes.c_double),
                ("seed", ctypes.c_uint64)]


class _ScanStats(ctypes.Structure):
    _fields_ = [("scan_ms", ctypes.c_double), ("count_ms", ctypes.c_double),
                ("max_count_ms", ctypes.c_double), ("count_launches", ctypes.c_int32),
                ("other_launches", ctypes.c_int32), ("batches", ctypes.c_int32),
                ("overflows", ctypes.c_int32), ("snp_pairs", ctypes.c_uint64),
                ("diag_snps", ctypes.c_uint64), ("tiles", ctypes.c_uint64),
                ("candidates", ctypes.c_uint64), ("method", ctypes.c_int32),
                ("tile_snps", ctypes.c_int32), ("variant", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class _ScanReq(ctypes.Structure):
    _fields_ = [("planes", ctypes.c_void_p), ("a0", ctypes.c_int32), ("na", ctypes.c_int32),
                ("b0", ctypes.c_int32), ("nb", ctypes.c_int32), ("topmost", ctypes.c_int32),
                ("objective", ctypes.c_int32), ("method", ctypes.c_int32),
                ("variant", ctypes.c_int32)]


class _BatchStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int64), ("count_launches", ctypes.c_int64),
                ("select_launches", ctypes.c_int64), ("graph_launches", ctypes.c_int64),
                ("device_ms", ctypes.c_double), ("wall_ms", ctypes.c_double)]


class _TuneReport(ctypes.Structure):
    _fields_ = [("variant", ctypes.c_int32), ("n_variants", ctypes.c_int32),
                ("ms", ctypes.c_float * 8)]


class _Progress(ctypes.Structure):
    _fields_ = [("elapsed_s", ctypes.c_double), ("tiles_done", ctypes.c_uint64),
                ("tiles_total", ctypes.c_uint64), ("snps_done", ctypes.c_int32),
                ("ntops", ctypes.c_int32), ("tops", ctypes.c_void_p)]


_PROGRESS_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(_Progress))


class _RequestInfo(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double),
                ("device_ms", ctypes.c_double), ("snp_pairs", ctypes.c_uint64),
                ("method", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_lib = None


def library_path() -> str:
    return _LIB_PATH


def lib():
    """The loaded libgepi.so (raises GepiError if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise GepiError(8, f"native library missing: {_LIB_PATH} "
                           "(run python -m gepicount_gb300.build)")
    L = ctypes.CDLL(_LIB_PATH)
    P, i32, u64, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_size_t
    PP = ctypes.POINTER(ctypes.c_void_p)
    L.gepi_status_string.restype = ctypes.c_char_p
    L.gepi_status_string.argtypes = [i32]
    L.gepi_last_error.restype = ctypes.c_char_p
    L.gepi_abi_version.restype = i32
    L.gepi_plink_open.argtypes = [ctypes.c_char_p, PP]
    L.gepi_plink_close.argtypes = [P]
    for f in ("gepi_plink_num_rows", "gepi_plink_num_samples", "gepi_plink_elements_snp"):
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = i32
    L.gepi_plink_bed.argtypes = [P, ctypes.POINTER(sz)]
    L.gepi_plink_bed.restype = P
    L.gepi_plink_phenotypes.argtypes = [P]
    L.gepi_plink_phenotypes.restype = P
    L.gepi_plink_row_info.argtypes = [P, i32, ctypes.POINTER(ctypes.c_char_p),
                                      ctypes.POINTER(ctypes.c_char), ctypes.POINTER(i32),
                                      ctypes.POINTER(i32)]
    L.gepi_plink_decode_rows.argtypes = [P, P, P, P, P]
    L.gepi_planes_from_bed.argtypes = [P, sz, i32, i32, P, i32, PP]
    L.gepi_planes_from_rows.argtypes = [P, P, i32, i32, P, P, i32, PP]
    L.gepi_planes_destroy.argtypes = [P]
    L.gepi_planes_destroy.restype = None
    L.gepi_planes_num_snps.argtypes = [P]
    L.gepi_planes_num_snps.restype = i32
    L.gepi_planes_class_sizes.argtypes = [P, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.gepi_scan.argtypes = [P, ctypes.POINTER(_Params), P, i32]
    L.gepi_scan_range.argtypes = [P, ctypes.POINTER(_Params), i32, i32, i32, i32, P, i32]
    L.gepi_pair_counts.argtypes = [P, i32, i32, i32, i32, i32, P]
    L.gepi_scan_progress.argtypes = [P, ctypes.POINTER(_Params), i32, i32, i32, i32, P, i32,
                                     _PROGRESS_FN, P, i32, i32]
    L.gepi_process_gpu_1.argtypes = [P, P, i32, i32, P, P, P, ctypes.POINTER(_Params)]
    L.gepi_last_scan_stats.argtypes = [P, ctypes.POINTER(_ScanStats)]
    L.gepi_last_scan_values.argtypes = [P, P, i32]
    L.gepi_planes_autotune.argtypes = [P, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_float),
                                       ctypes.POINTER(ctypes.c_float)]
    L.gepi_tensor_peak_tflops.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    L.gepi_tensor_peak_probe.argtypes = [i32, i32, ctypes.POINTER(ctypes.c_double)]
    L.gepi_planes_autotune_variants.argtypes = [P, ctypes.POINTER(_TuneReport)]
    L.gepi_scan_batch_stats.argtypes = [i32, ctypes.POINTER(_BatchStats)]
    L.gepi_count_variant_name.argtypes = [i32]
    L.gepi_count_variant_name.restype = ctypes.c_char_p
    L.gepi_count_variant_shape.argtypes = [i32] + [ctypes.POINTER(i32)] * 4
    L.gepi_process_gpu_1_noalloc.argtypes = [P, P, i32, i32, P, P, P, ctypes.POINTER(_Params)]
    L.gepi_shard_range.argtypes = [i32, i32, i32] + [ctypes.POINTER(ctypes.c_int32)] * 4
    L.gepi_merge_results.argtypes = [i32, i32, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_int32),
                                     i32, P, i32]
    L.gepi_scan_batch.argtypes = [ctypes.POINTER(_ScanReq), i32, ctypes.POINTER(P),
                                  ctypes.POINTER(_ScanStats)]
    L.gepi_server_create.argtypes = [i32, sz, PP]
    L.gepi_server_submit.argtypes = [P, ctypes.POINTER(_ScanReq), ctypes.POINTER(u64)]
    L.gepi_server_wait.argtypes = [P, u64, P, ctypes.POINTER(_RequestInfo)]
    L.gepi_server_stats.argtypes = [P, ctypes.POINTER(_BatchStats)]
    L.gepi_server_destroy.argtypes = [P]
    L.gepi_server_destroy.restype = None
    L.gepi_fisher_pval.argtypes = [i32, i32, i32, i32]
    L.gepi_fisher_pval.restype = ctypes.c_float
    L.gepi_fisher_log10p.argtypes = [i32, i32, i32, i32]
    L.gepi_fisher_log10p.restype = ctypes.c_double
    L.gepi_synth_bed_bytes.argtypes = [ctypes.POINTER(_SynthSpec)]
    L.gepi_synth_bed_bytes.restype = sz
    L.gepi_synth_bed.argtypes = [ctypes.POINTER(_SynthSpec), P, P, P]
    L.gepi_synth_write.argtypes = [ctypes.POINTER(_SynthSpec), ctypes.c_char_p]
    for f in ("gepi_plink_open", "gepi_plink_row_info", "gepi_plink_decode_rows",
              "gepi_planes_from_bed", "gepi_planes_from_rows", "gepi_planes_class_sizes",
              "gepi_scan", "gepi_scan_range", "gepi_pair_counts", "gepi_process_gpu_1",
              "gepi_last_scan_stats", "gepi_last_scan_values", "gepi_process_gpu_1_noalloc", "gepi_planes_autotune",
              "gepi_tensor_peak_tflops", "gepi_tensor_peak_probe", "gepi_planes_autotune_variants",
              "gepi_count_variant_shape", "gepi_scan_batch_stats", "gepi_scan_batch", "gepi_scan_progress", "gepi_shard_range", "gepi_merge_results", "gepi_server_create",
              "gepi_server_submit", "gepi_server_wait", "gepi_server_stats",
              "gepi_synth_bed", "gepi_synth_write"):
        getattr(L, f).restype = i32
    _lib = L
    return L


def _check(status: int):
    if status != 0:
        msg = lib().gepi_last_error().decode(errors="replace")
        raise GepiError(status, msg)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ---- parameters (struct _paramP1) ------------------------------------------
@dataclass
class Params:
    """struct _paramP1 (inc/gEpiCount.h:116-132) plus the counting method."""

    gpuNum: int = 0
    topmost: int = 1000000
    gold: bool = False
    shmem: bool = False
    alt: bool = False
    intermediate: bool = False
    name: str = ""
    blkSzX: int = 16
    blkSzY: int = 16
    maxGridBlocks: int = 16
    ffun: int = ENTROPY
    qaMissSNPs: float = 0.05
    qaMissSamp: float = 0.05
    qaRemoveMissing: bool = False
    method: int = METHOD_AUTO
    verbose: int = 0
    variant: int = 0

    def _c(self) -> _Params:
        p = _Params()
        p.gpu_num = self.gpuNum
        p.topmost = self.topmost
        p.objective = self.ffun
        p.method = self.method
        p.verbose = self.verbose
        p.variant = self.variant
        return p


# ---- reader ----------------------------------------------------------------
class BinPlinkReader:
    """Host PLINK reader with BinPlinkReader/PlinkReader semantics."""

    ELEMENT_SIZE = 8

    def __init__(self, base: str):
        self.basepath = base
        self._h = ctypes.c_void_p()
        self._bits = self._valid = self._m1 = self._m2 = None

    def checkConsistency(self) -> bool:
        if self._h:
            return True
        st = lib().gepi_plink_open(self.basepath.encode(), ctypes.byref(self._h))
        if st != 0:
            self._h = ctypes.c_void_p()
            self.error = lib().gepi_last_error().decode(errors="replace")
            return False
        return True

    def readData(self) -> bool:
        if not self.checkConsistency():
            return False
        nr, nw = self.numSNPs(), self.elementsSNP()
        self._bits = np.zeros((nr, nw), dtype=np.uint64)
        self._valid = np.zeros((nr, nw), dtype=np.uint64)
        self._m1 = np.zeros(nw, dtype=np.uint64)
        self._m2 = np.zeros(nw, dtype=np.uint64)
        _check(lib().gepi_plink_decode_rows(self._h, _ptr(self._bits), _ptr(self._valid),
                                            _ptr(self._m1), _ptr(self._m2)))
        return True

    def numSNPs(self) -> int:
        return lib().gepi_plink_num_rows(self._h)

    def numSamples(self) -> int:
        return lib().gepi_plink_num_samples(self._h)

    def elementsSNP(self) -> int:
        return lib().gepi_plink_elements_snp(self._h)

    def DataSize(self) -> int:
        return self.ELEMENT_SIZE * self.elementsSNP() * self.numSNPs()

    def BitData(self) -> np.ndarray:
        return self._bits

    def ValidData(self) -> np.ndarray:
        return self._valid

    def classMask(self, key: int) -> np.ndarray | None:
        return {1: self._m1, 2: self._m2}.get(key)

    def bed(self) -> np.ndarray:
        n = ctypes.c_size_t()
        p = lib().gepi_plink_bed(self._h, ctypes.byref(n))
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)),
                                     shape=(n.value,))

    def phenotypes(self) -> np.ndarray:
        p = lib().gepi_plink_phenotypes(self._h)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_int32)),
                                     shape=(self.numSamples(),)).copy()

    def getSnp(self, row: int):
        """(id, allele, chr, pos) of allele row `row`."""
        sid, al = ctypes.c_char_p(), ctypes.c_char()
        ch, pos = ctypes.c_int(), ctypes.c_int()
        _check(lib().gepi_plink_row_info(self._h, row, ctypes.byref(sid), ctypes.byref(al),
                                         ctypes.byref(ch), ctypes.byref(pos)))
        return sid.value.decode(), al.value.decode(), ch.value, pos.value

    def close(self):
        if self._h:
            lib().gepi_plink_close(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- device planes ------------------------------------------------------------
class Planes:
    """Device-resident class-sorted genotype bit-planes of one cohort."""

    def __init__(self, handle: ctypes.c_void_p, device: int):
        self._h = handle
        self.device = device

    @classmethod
    def from_bed(cls, bed: np.ndarray, n_bim_snps: int, phenotype: np.ndarray,
                 device: int = 0) -> "Planes":
        bed = np.ascontiguousarray(bed, dtype=np.uint8)
        ph = np.ascontiguousarray(phenotype, dtype=np.int32)
        h = ctypes.c_void_p()
        _check(lib().gepi_planes_from_bed(_ptr(bed), bed.size, n_bim_snps, ph.size, _ptr(ph),
                                          device, ctypes.byref(h)))
        return cls(h, device)

    @classmethod
    def from_rows(cls, bits: np.ndarray, valid: np.ndarray, mask1: np.ndarray,
                  mask2: np.ndarray, device: int = 0) -> "Planes":
        bits = np.ascontiguousarray(bits, dtype=np.uint64)
        valid = np.ascontiguousarray(valid, dtype=np.uint64)
        m1 = np.ascontiguousarray(mask1, dtype=np.uint64)
        m2 = np.ascontiguousarray(mask2, dtype=np.uint64)
        h = ctypes.c_void_p()
        _check(lib().gepi_planes_from_rows(_ptr(bits), _ptr(valid), bits.shape[0], bits.shape[1],
                                           _ptr(m1), _ptr(m2), device, ctypes.byref(h)))
        return cls(h, device)

    @property
    def n_snps(self) -> int:
        return lib().gepi_planes_num_snps(self._h)

    def class_sizes(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(lib().gepi_planes_class_sizes(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def scan(self, k: int, objective: int = ENTROPY, method: int = METHOD_AUTO,
             verbose: int = 0, variant: int = 0) -> np.ndarray:
        par = Params(topmost=k, ffun=objective, method=method, verbose=verbose, gpuNum=self.device,
                     variant=variant)
        tops = np.zeros(k, dtype=RESULT_DTYPE)
        _check(lib().gepi_scan(self._h, ctypes.byref(par._c()), _ptr(tops), k))
        return tops

    def scan_range(self, a0: int, na: int, b0: int, nb: int, k: int, objective: int = ENTROPY,
                   method: int = METHOD_AUTO, variant: int = 0) -> np.ndarray:
        par = Params(topmost=k, ffun=objective, method=method, gpuNum=self.device, variant=variant)
        tops = np.zeros(k, dtype=RESULT_DTYPE)
        _check(lib().gepi_scan_range(self._h, ctypes.byref(par._c()), a0, na, b0, nb,
                                     _ptr(tops), k))
        return tops

    def scan_progress(self, k: int, callback, points: int = 0, with_tops: bool = False,
                      objective: int = ENTROPY, method: int = METHOD_AUTO, a0: int = 0,
                      na: int | None = None, b0: int = 0, nb: int | None = None) -> np.ndarray:
        """scan_range with progress: callback(dict) at tile-band ends (see
        gepi_scan_progress); with_tops adds the exact ranked top-k so far."""
        n = self.n_snps
        na = n - a0 if na is None else na
        nb = n - b0 if nb is None else nb
        par = Params(topmost=k, ffun=objective, method=method, gpuNum=self.device)
        tops = np.zeros(k, dtype=RESULT_DTYPE)
        errors = []

        def tramp(_user, pp):
            try:
                p = pp.contents
                snap = None
                if p.tops and p.ntops > 0:
                    buf = (ctypes.c_char * (p.ntops * RESULT_DTYPE.itemsize)).from_address(p.tops)
                    snap = np.frombuffer(bytes(buf), dtype=RESULT_DTYPE).copy()
                callback({"elapsed_s": p.elapsed_s, "tiles_done": p.tiles_done,
                          "tiles_total": p.tiles_total, "snps_done": p.snps_done, "tops": snap})
            except Exception as e:  # re-raised after the scan
                errors.append(e)

        fn = _PROGRESS_FN(tramp)
        _check(lib().gepi_scan_progress(self._h, ctypes.byref(par._c()), a0, na, b0, nb,
                                        _ptr(tops), k, fn, None, points, 1 if with_tops else 0))
        if errors:
            raise errors[0]
        return tops

    def pair_counts(self, a0: int, na: int, b0: int, nb: int,
                    method: int = METHOD_POPC) -> np.ndarray:
        out = np.zeros((na, nb, 18), dtype=np.uint32)
        _check(lib().gepi_pair_counts(self._h, method, a0, na, b0, nb, _ptr(out)))
        return out

    def autotune_variants(self) -> dict:
        """The counting variant METHOD_AUTO uses on these planes and every
        variant's time on the tuning triangle ({name: ms}, 0 = not timed)."""
        r = _TuneReport()
        _check(lib().gepi_planes_autotune_variants(self._h, ctypes.byref(r)))
        return {"variant": r.variant, "name": variant_name(r.variant),
                "ms": {variant_name(v): float(r.ms[v - 1]) for v in range(1, r.n_variants + 1)}}

    def autotune(self) -> dict:
        """The counting method METHOD_AUTO uses on these planes, with the two
        kernels' timings on the tuning triangle (tuned on first use)."""
        m = ctypes.c_int32()
        tp, tt = ctypes.c_float(), ctypes.c_float()
        _check(lib().gepi_planes_autotune(self._h, ctypes.byref(m), ctypes.byref(tp),
                                          ctypes.byref(tt)))
        return {"method": m.value, "popc_ms": tp.value, "tensor_ms": tt.value}

    def last_stats(self) -> dict:
        """Device timings and counters of the last scan on these planes."""
        st = _ScanStats()
        _check(lib().gepi_last_scan_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _ScanStats._fields_}

    def last_values(self, k: int) -> np.ndarray:
        """The FP64 objective each `ent` of the last ranked list was rounded
        from (entropy -I bits, Fisher log10 p; 0 for zero-filled slots)."""
        out = np.zeros(k, dtype=np.float64)
        _check(lib().gepi_last_scan_values(self._h, out.ctypes.data, k))
        return out

    def close(self):
        if self._h:
            lib().gepi_planes_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def process_gpu_1(pr: BinPlinkReader, tops: np.ndarray, par: Params) -> None:
    """Drop-in for process_gpu_1 (kernel1.cu:508-511): fills tops[:par.topmost]."""
    if tops.dtype != RESULT_DTYPE or tops.size < par.topmost:
        raise GepiError(1, "tops must be a RESULT_DTYPE array of length >= topmost")
    bits, valid = pr.BitData(), pr.ValidData()
    m1, m2 = pr.classMask(1), pr.classMask(2)
    if bits is None or m1 is None or m2 is None:
        raise GepiError(1, "reader has no data (call readData first)")
    _check(lib().gepi_process_gpu_1(_ptr(bits), _ptr(valid), bits.shape[0], bits.shape[1],
                                    _ptr(m1), _ptr(m2), _ptr(tops), ctypes.byref(par._c())))


def process_gpu_1_noalloc(pr: BinPlinkReader, tops: np.ndarray, par: Params) -> None:
    """process_gpu_1 for hosts that cannot allocate device memory: every
    device buffer comes from the library's fixed 32 MiB scratch array (see
    gepi_process_gpu_1_noalloc in include/gepi.h for limits and sharing)."""
    if tops.dtype != RESULT_DTYPE or tops.size < par.topmost:
        raise GepiError(1, "tops must be a RESULT_DTYPE array of length >= topmost")
    bits, valid = pr.BitData(), pr.ValidData()
    m1, m2 = pr.classMask(1), pr.classMask(2)
    if bits is None or m1 is None or m2 is None:
        raise GepiError(1, "reader has no data (call readData first)")
    _check(lib().gepi_process_gpu_1_noalloc(_ptr(bits), _ptr(valid), bits.shape[0],
                                            bits.shape[1], _ptr(m1), _ptr(m2), _ptr(tops),
                                            ctypes.byref(par._c())))


# ---- sharded scans ----------------------------------------------------------------
def shard_range(n_snps: int, n_shards: int, shard: int):
    """(a0, na, b0, nb) of shard `shard` of the whole-genome triangle: a
    scan_range over it covers a disjoint, about equal share of the pairs."""
    v = [ctypes.c_int32() for _ in range(4)]
    _check(lib().gepi_shard_range(n_snps, n_shards, shard, *[ctypes.byref(x) for x in v]))
    return tuple(x.value for x in v)


def merge_results(lists, k: int, n_samples: int, objective: int = ENTROPY) -> np.ndarray:
    """k-way merge of ranked RESULT_DTYPE lists from disjoint scans of one
    cohort (gepi_merge_results): the k best, ranked as one scan ranks them.
    Host only: no device is needed."""
    lists = [np.ascontiguousarray(x, dtype=RESULT_DTYPE) for x in lists]
    n = len(lists)
    ptrs = (ctypes.c_void_p * max(1, n))(*[_ptr(x) if x.size else None for x in lists])
    lens = (ctypes.c_int32 * max(1, n))(*[x.size for x in lists])
    out = np.zeros(k, dtype=RESULT_DTYPE)
    _check(lib().gepi_merge_results(n_samples, objective, ptrs, lens, n, _ptr(out), k))
    return out


# ---- many scans at once --------------------------------------------------------
@dataclass
class ScanRequest:
    """One scan: SNP ranges [a0, a0+na) x [b0, b0+nb) of `planes` (na or nb
    negative: the whole plane set), the k best by `objective`."""
    planes: Planes
    k: int
    objective: int = ENTROPY
    method: int = METHOD_AUTO
    a0: int = 0
    na: int = -1
    b0: int = 0
    nb: int = -1
    variant: int = 0

    def _c(self) -> _ScanReq:
        return _ScanReq(self.planes._h, self.a0, self.na, self.b0, self.nb, self.k,
                        self.objective, self.method, self.variant)


def scan_batch(reqs, with_stats: bool = False):
    """Runs the requests together (gepi_scan_batch); returns one RESULT_DTYPE
    array per request (and the per-request scan stats if asked)."""
    reqs = list(reqs)
    n = len(reqs)
    creqs = (_ScanReq * n)(*[r._c() for r in reqs])
    outs = [np.zeros(r.k, dtype=RESULT_DTYPE) for r in reqs]
    ptrs = (ctypes.c_void_p * n)(*[_ptr(o) for o in outs])
    stats = (_ScanStats * n)()
    _check(lib().gepi_scan_batch(creqs, n, ptrs, stats))
    if with_stats:
        return outs, [{f: getattr(st, f) for f, _ in _ScanStats._fields_} for st in stats]
    return outs


def scan_batch_stats(device: int = 0) -> dict:
    """Counters of the last scan_batch call on `device`: engine steps,
    counting launches, batched select launches, step-graph replays, and the
    steps' device and host milliseconds."""
    st = _BatchStats()
    _check(lib().gepi_scan_batch_stats(device, ctypes.byref(st)))
    return {f: getattr(st, f) for f, _ in _BatchStats._fields_}


class Server:
    """The serving loop (gepi_server_*): submit() returns a ticket at once,
    wait(ticket) blocks for that request's results and timings."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        h = ctypes.c_void_p()
        _check(lib().gepi_server_create(device, hbm_budget_bytes, ctypes.byref(h)))
        self._h = h
        self._k = {}

    def submit(self, req: ScanRequest) -> int:
        t = ctypes.c_uint64()
        c = req._c()
        _check(lib().gepi_server_submit(self._h, ctypes.byref(c), ctypes.byref(t)))
        self._k[t.value] = req.k
        return t.value

    def wait(self, ticket: int):
        """(results, info dict) of the ticket's request."""
        k = self._k.pop(ticket, 1)
        tops = np.zeros(k, dtype=RESULT_DTYPE)
        info = _RequestInfo()
        _check(lib().gepi_server_wait(self._h, ticket, _ptr(tops), ctypes.byref(info)))
        return tops, {f: getattr(info, f) for f, _ in _RequestInfo._fields_ if f != "reserved"}

    def stats(self) -> dict:
        """The server engine's counters since creation (gepi_server_stats)."""
        st = _BatchStats()
        _check(lib().gepi_server_stats(self._h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in _BatchStats._fields_}

    def close(self):
        if self._h:
            lib().gepi_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tensor_peak_tflops(device: int = 0) -> float:
    """Dense kind::mxf4 tensor-core rate of `device` (TFLOP/s), measured now."""
    v = ctypes.c_double()
    _check(lib().gepi_tensor_peak_tflops(device, ctypes.byref(v)))
    return v.value


PEAK_KINDS = {"mxf4": 0, "mxf4nvf4_2x_ue8m0": 1, "mxf4nvf4_4x_ue4m3": 2}
NUM_VARIANTS = 4


def variant_name(v: int) -> str:
    """Name of counting variant v (gepi_count_variant_name)."""
    return lib().gepi_count_variant_name(v).decode()


def variant_shape(v: int) -> dict:
    m, ta, tb, w = (ctypes.c_int32() for _ in range(4))
    _check(lib().gepi_count_variant_shape(v, ctypes.byref(m), ctypes.byref(ta), ctypes.byref(tb),
                                          ctypes.byref(w)))
    return {"method": m.value, "tile_a": ta.value, "tile_b": tb.value, "stage_words": w.value}


def variant_method(v: int) -> int:
    """The `method` argument of pair_counts() that selects counting variant v."""
    return 16 + v


def tensor_peak_probe(kind: str, device: int = 0) -> float:
    """Dense FP4 tensor-core rate (TFLOP/s) of one exact 0/1 encoding (PEAK_KINDS)."""
    v = ctypes.c_double()
    _check(lib().gepi_tensor_peak_probe(device, PEAK_KINDS[kind], ctypes.byref(v)))
    return v.value


def fisher_pval(n11: int, n12: int, n21: int, n22: int) -> float:
    """fisher_pval (src/misc/fisher_p.c:52-76): float log10 of the two-sided p."""
    return float(lib().gepi_fisher_pval(n11, n12, n21, n22))


def fisher_log10p(n11: int, n12: int, n21: int, n22: int) -> float:
    return float(lib().gepi_fisher_log10p(n11, n12, n21, n22))


# ---- seeded synthetic PLINK data --------------------------------------------
@dataclass
class SynthSpec:
    n_snps: int
    n_cases: int
    n_controls: int
    maf_lo: float = 0.05
    maf_hi: float = 0.5
    missing: float = 0.02
    n_planted: int = 0
    odds_ratio: float = 2.0
    seed: int = 1000

    def _c(self) -> _SynthSpec:
        s = _SynthSpec()
        for f in ("n_snps", "n_cases", "n_controls", "maf_lo", "maf_hi", "missing", "n_planted",
                  "odds_ratio", "seed"):
            setattr(s, f, getattr(self, f))
        return s

    @property
    def n_samples(self) -> int:
        return self.n_cases + self.n_controls


def synth_bed(spec: SynthSpec, out: np.ndarray | None = None):
    """-> (bed image uint8, phenotype int32, planted SNP pairs int32[n_planted, 2])."""
    c = spec._c()
    nb = lib().gepi_synth_bed_bytes(ctypes.byref(c))
    if nb == 0:
        raise GepiError(1, "bad synthetic spec")
    bed = out if out is not None else np.empty(nb, dtype=np.uint8)
    if bed.size != nb or bed.dtype != np.uint8:
        raise GepiError(1, "output buffer has the wrong size")
    ph = np.empty(spec.n_samples, dtype=np.int32)
    pl = np.empty(max(1, 2 * spec.n_planted), dtype=np.int32)
    _check(lib().gepi_synth_bed(ctypes.byref(c), _ptr(bed), _ptr(ph), _ptr(pl)))
    return bed, ph, pl[: 2 * spec.n_planted].reshape(-1, 2)


def synth_write(spec: SynthSpec, base: str) -> None:
    _check(lib().gepi_synth_write(ctypes.byref(spec._c()), base.encode()))
