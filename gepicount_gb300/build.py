"""Build recipe for the native library and the CLI (no cmake).

    python -m gepicount_gb300.build          # -> gepicount_gb300/_build/libgepi.so, gepi, gepi-synth

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), host code with -ffp-contract=off so
the synthetic-data generator and the scoring tables give identical bits on
x86 and Arm hosts.  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgepi.so")
CLI = os.path.join(OUT, "gepi")
SYNTH = os.path.join(OUT, "gepi-synth")  # the data generator alone (no CUDA)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["scan.cu", "decode.cu", "count_popc.cu", "select.cu", "noalloc.cu", "count_tc.cu",
              "engine.cu"]
CPP_SOURCES = ["plink.cpp", "synth.cpp", "tables.cpp"]
CLI_SOURCES = ["cli.cpp"]
SYNTH_SOURCES = ["synth.cpp", "synth_main.cpp"]
HOST_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-Wall",
              "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers():
    hs = [os.path.join(ROOT, "include", "gepi.h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile and link; returns the path of libgepi.so."""
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    heads = _headers()
    cuda_home = os.path.dirname(os.path.dirname(nvcc))
    tasks = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + heads):
            tasks.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                          "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + heads):
            tasks.append(["g++", *HOST_FLAGS, f"-I{cuda_home}/include", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(lambda c: _run(c, verbose), tasks))
    if tasks or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"], verbose)
    cli_srcs = [os.path.join(CSRC, s) for s in CLI_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if cli_srcs and _stale(CLI, cli_srcs + heads + [LIB]):
        _run(["g++", *HOST_FLAGS, *cli_srcs, "-o", CLI, f"-L{OUT}", "-lgepi",
              "-Wl,-rpath,$ORIGIN"], verbose)
    synth_srcs = [os.path.join(CSRC, s) for s in SYNTH_SOURCES]
    if _stale(SYNTH, synth_srcs + heads):
        _run(["g++", *HOST_FLAGS, *synth_srcs, "-o", SYNTH], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
