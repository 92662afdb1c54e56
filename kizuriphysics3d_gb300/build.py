"""In-tree build of libkzg.so for sm_103a (GB300) with nvcc.

Floating-point flags are part of the contract: --fmad=false (no contraction on the device),
IEEE division and square root, no flush-to-zero, and -ffp-contract=off for host code, so the
library reproduces the reference's float results bit for bit.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libkzg.so")
SOURCES = ["kzg_step.cu", "kzg_api.cu", "kzg_hull.cpp", "kzg_noalloc.cu", "kzg_mlp.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "kzg.h"))
    objs = []
    jobs = []
    for s in SOURCES:
        src = os.path.join(SRC, s)
        obj = os.path.join(OUT, s + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + headers):
            lang = ["-x", "cu"] if s.endswith(".cu") else ["-x", "c++"]
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + lang + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or not _newer(LIB, objs):
        run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # C++ facade example (include/kizuri_gpu/PhysicsWorld.h), linked against the library
    for name in ("pyramid_example", "joints_example"):
        ex_src = os.path.join(HERE, "cpp", name + ".cpp")
        ex = os.path.join(OUT, name)
        if force or not _newer(ex, [ex_src, LIB, os.path.join(HERE, "..", "include", "kizuri_gpu", "PhysicsWorld.h")]):
            run(["g++", "-std=c++17", "-O2", "-I", os.path.join(HERE, "..", "include"), ex_src, "-o", ex, "-L", OUT,
                 "-lkzg", f"-Wl,-rpath,{OUT}"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
