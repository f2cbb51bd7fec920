"""Build the in-tree native libraries of thindb_gb300.

    libthindb_gpu.so      the CUDA engine behind include/thindb_gpu.h (sm_103a)
    libthindb_datagen.so  seeded synthetic inputs (host C++)

Each translation unit compiles in parallel; nothing is installed outside the
package directory.  Run as ``python -m thindb_gb300.build``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_lib")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
ENGINE_SOURCES = ["api.cpp", "scan.cu", "scan_inline.cu", "scan_batch.cu", "scan_staged.cu", "scan_pipe.cu", "scan_split.cu", "sketch.cu", "radix.cu", "segment.cu", "distinct.cu", "finalize.cu", "table.cu", "noalloc.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs + [os.path.join(INCLUDE, "thindb_gpu.h")]


def build_engine(verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(OUT, "libthindb_gpu.so")
    srcs = [s for s in ENGINE_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []
    jobs = []
    hdrs = _headers()
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs) or ptxas_v:
            cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                   "--expt-relaxed-constexpr", "-I", INCLUDE, "-c", src, "-o", obj]
            if ptxas_v and s.endswith(".cu"):
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=min(max(8, os.cpu_count() or 8), max(1, len(jobs)))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if _stale(so, objs) or jobs:
        _run([nvcc(), *ARCH, "-shared", "-o", so, *objs, "-lpthread"])
    if verbose:
        print("built", so)
    return so


def build_datagen(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libthindb_datagen.so")
    src = os.path.join(CSRC, "datagen.cpp")
    if _stale(so, [src]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", src, "-o", so])
    if verbose:
        print("built", so)
    return so


def build_all(verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fs = [ex.submit(build_engine, verbose), ex.submit(build_datagen, verbose)]
        for f in fs:
            f.result()


if __name__ == "__main__":
    build_engine(verbose=True, ptxas_v="-v" in sys.argv)
    build_datagen(verbose=True)
