"""Builds libwhir_gb300.so in-tree: every .cu translation unit compiled in parallel for sm_103a and
linked into one shared library next to this file."""

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwhir_gb300.so")
SOURCES = ["commit.cu", "commit_mont.cu", "sumcheck.cu", "sumcheck_mont.cu", "prover.cu", "verifier.cu",
           "noalloc.cu"]
HEADERS = ["field.cuh", "hash.cuh", "kernels.hpp", "protocol.hpp", "status.hpp", "roots.cuh", "encode.cuh",
           "sumcheck.cuh", "sponge.cuh", "wide.cuh", "bulk.cuh"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-std=c++20", "--expt-relaxed-constexpr", "-lineinfo",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-Xptxas", "-O3",
]


def nvcc_path():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newest_input():
    paths = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    paths.append(os.path.join(HERE, "..", "include", "whir_gb300.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build(force=False, verbose=False):
    """Compile if any source is newer than the library. Returns the library path."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = nvcc_path()

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
