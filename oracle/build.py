"""Build recipe for the oracle (test infrastructure only).

Compiles oracle.cpp (the binary field POLYVAL) and oracle_bb.cpp (the prime
field BabyBear) with the host C++ compiler into oracle/_build/liboracle.so.
On aarch64 the carry-less multiply uses the PMULL instruction (the analogue of
the reference's NEON backend, p3/src/polyval/aarch64_neon.rs); elsewhere the
portable 4-bit-window multiply is used.  Both give identical results.
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


SOURCES = ["oracle.cpp", "oracle_bb.cpp"]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(f) for f in srcs):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    # no fused multiply-add contraction: the query-count formulas in double
    # must round as the reference's Rust (which never contracts) does
    flags = ["-O3", "-std=c++17", "-shared", "-fPIC", "-pthread", "-Wall", "-ffp-contract=off"]
    if platform.machine() in ("aarch64", "arm64"):
        flags += ["-march=armv8-a+crypto", "-DORACLE_PMULL"]
    tmp = LIB + ".tmp"
    subprocess.check_call([cxx, *flags, *srcs, "-o", tmp])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
