"""Build recipe for the CPU oracle (test infrastructure only).

    oracle/_build/liboracle.so   from oracle/oracle.cpp and oracle/segment.cpp

thinDB itself is Zig 0.17 and no Zig toolchain exists on either machine, so
there is no `oracle/_ref` build of the reference: the oracle is a C++
restatement pinned against the reference's known-answer tests
(tests/golden/).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
SO = os.path.join(OUT, "liboracle.so")


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "segment.cpp")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(os.path.dirname(HERE), "include", "thindb_gpu.h")]
    if not os.path.exists(SO) or any(os.path.getmtime(d) > os.path.getmtime(SO) for d in deps):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", *srcs, "-o", SO]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    if verbose:
        print("built", SO)
    return SO


if __name__ == "__main__":
    build(verbose=True)
