"""Builds libufemism_gb300.so in-tree (``ufemism_gb300/_build``) with nvcc for sm_103a.

Every translation unit compiles in parallel; host code and device code are built with
``-ffp-contract=off`` / ``--fmad=false`` so that each multiply and add rounds separately,
as the reference Fortran's arithmetic does (gfortran -O3 on x86-64 emits no FMA). The CUDA
runtime is linked statically so the library does not depend on a loader path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Build variants: the product library; a profiling build whose persistent solver records
# per-phase SM-cycle totals (ufe_debug_phase_cycles); builds whose mixed sweeps decide
# convergence two sweeps late (for measuring the lag). UFE_BUILD_VARIANT selects the one that
# ufemism_gb300._native loads.
VARIANTS = {"": [], "phase_timers": ["-DUFE_PHASE_TIMERS=1"], "lag2": ["-DUFE_MIXED_LAG=2"],
            "lag2_phase_timers": ["-DUFE_MIXED_LAG=2", "-DUFE_PHASE_TIMERS=1"]}
VARIANT = os.environ.get("UFE_BUILD_VARIANT", "")
if VARIANT not in VARIANTS:
    raise RuntimeError("UFE_BUILD_VARIANT must be one of %s" % sorted(VARIANTS))
OUT = os.path.join(HERE, "_build" + ("_" + VARIANT if VARIANT else ""))
LIB = os.path.join(OUT, "libufemism_gb300.so")

CU_SOURCES = ["ufe_mesh.cu", "ufe_ssa.cu", "ufe_sia.cu", "ufe_geom.cu"]
CPP_SOURCES = ["ufe_capi.cpp", "aaac_build.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(SRC, f) for f in CU_SOURCES + CPP_SOURCES] + \
        [os.path.join(SRC, "ufe_internal.h"), os.path.join(HERE, "..", "include", "ufemism_gb300.h")]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + os.path.join(HERE, "..", "include")]
    jobs = []
    for f in CU_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        jobs.append([nvcc, *ARCH, "-lineinfo", "--fmad=false", *common, *VARIANTS[VARIANT], *(extra_flags or []),
                     "-c", os.path.join(SRC, f), "-o", obj])
    for f in CPP_SOURCES:
        obj = os.path.join(OUT, f + ".o")
        jobs.append([nvcc, *common, "-c", os.path.join(SRC, f), "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("compile failed: " + cmd[-3])
        return cmd[-1]

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    link = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
