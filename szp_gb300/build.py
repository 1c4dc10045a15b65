"""Builds libszp_gb300.so in-tree with nvcc for sm_103a (GB300).

Each CUDA translation unit compiles in parallel to an object under
szp_gb300/_build/, then nvcc links the shared library next to this file.
The same recipe runs on x86-64 (cross-compile) and on the aarch64 GPU host.
"""
import concurrent.futures
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build", platform.machine())
LIB = os.path.join(HERE, "libszp_gb300.so")
SOURCES = ["api.cu", "compress.cu", "decompress.cu", "fm1_pipes.cu", "noalloc.cu", "batch.cu", "serve.cu", "lorenzo.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
CFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp,-O2",
                 "-I", os.path.join(HERE, "..", "include")]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(HERE, "..", "include", "szp_gb300.h")]


def build(verbose=False, force=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _headers()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([NVCC] + CFLAGS + list(extra) + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for err in ex.map(run, jobs):
            if verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or _newer(LIB, objs):
        run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
