"""Build libbasefold_gpu.so in-tree for sm_103a.

    python learn-zkp_gb300/build.py [--force]

Compiles the CUDA translation units in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a) and links them into
learn-zkp_gb300/basefold_gpu/_lib/libbasefold_gpu.so.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "basefold_gpu", "_lib")
LIB = os.path.join(OUT_DIR, "libbasefold_gpu.so")
SOURCES = ["kernels.cu", "kernels_tail.cu", "kernels_verify.cu", "kernels_bb.cu", "api_pcs.cu", "api_open.cu", "api_verify.cu", "api_sumcheck.cu", "api_engine.cu", "api_noalloc.cu", "api_tune.cu", "api_bb.cu"]
HEADERS = ["gf128.cuh", "keccak.cuh", "bf_internal.h", "host_math.h", "api_common.h", "bb.cuh", "bb_internal.h", "bb_host.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "basefold_gpu.h"))
    return any(os.path.getmtime(f) > t for f in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    # host code: no fused multiply-add contraction, so the query-count
    # formulas in double round as the reference's Rust does
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                    "-Xcompiler", "-ffp-contract=off", "-diag-suppress", "177"]
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    subprocess.check_call([cc, *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
