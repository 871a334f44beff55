"""Builds the tcstencil_gb300 native library in-tree.

    python -m tcstencil_gb300.build          (or __graft_entry__.build())

Outputs go to tcstencil_gb300/_build/:
    libtcs.so                          the engine (C-ABI of include/tcs.h)
    libtcs_host_<engine>_<stencil>.so  per-variant `host_code` for the
                                       reference's common/main_1r.cu / main_2r.cu
Every CUDA unit is compiled for sm_103a only, in parallel, and only when a
source or header is newer than its object.
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
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_build")

CU_SOURCES = ["layout.cu", "sweep_cc.cu", "sweep_tc.cu", "api.cu", "sweep_noalloc.cu", "batch.cu", "server.cu", "sweep_tb.cu", "drift.cu", "memory.cu"]
HEADERS = ["tcs_device.cuh", "tcs_internal.h", "tc_core.cuh", "batch.h", "tile_walk.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-Wall",
                     "--expt-relaxed-constexpr", "-I", INCLUDE]
STENCILS = ["star2d1r", "star2d2r", "box2d1r", "box2d2r"]
ENGINES = {"tensor": 0, "cudacore": 1}

LIB = os.path.join(OUT, "libtcs.so")


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tcstencil_gb300")
    return exe


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}")
    if r.stdout.strip():
        sys.stderr.write(r.stdout)


def build(verbose: bool = False, extra_flags: list[str] | None = None) -> str:
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "tcs.h")]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, "obj", src.replace(".cu", ".o"))
        objs.append(o)
        if _newer(o, [s] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + (extra_flags or []) + ["-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    if _newer(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-ldl",
                                                                "-lpthread", "-lrt"])
    shim = os.path.join(CSRC, "host_code_variant.c")
    cc = shutil.which("gcc") or "cc"
    shim_jobs = []
    for eng, eid in ENGINES.items():
        for si, st in enumerate(STENCILS):
            out = os.path.join(OUT, f"libtcs_host_{eng}_{st}.so")
            if _newer(out, [shim, LIB, os.path.join(INCLUDE, "tcs.h")]):
                shim_jobs.append([cc, "-O2", "-fPIC", "-shared", f"-DTCS_STENCIL={si}",
                                  f"-DTCS_ENGINE={eid}", "-o", out, shim, "-L", OUT, "-ltcs",
                                  "-Wl,-rpath,$ORIGIN"])
    if shim_jobs:
        with ThreadPoolExecutor(max_workers=8) as ex:
            for f in [ex.submit(_run, j) for j in shim_jobs]:
                f.result()
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra_flags=sys.argv[1:] or None)
