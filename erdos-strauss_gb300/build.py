"""Build the GB300 engine in-tree: nvcc for sm_103a, no cmake.

Outputs, next to this file:
  libes_sieve.so      the engine and its C ABI (include/es_sieve.h)
  rung_scan3_gb300    the rung_scan3-compatible command line over that library

Run as `python erdos-strauss_gb300/build.py` or call build(). Compiles the translation
units in parallel; a full build takes well under a minute on either host architecture.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libes_sieve.so")
CLI = os.path.join(HERE, "rung_scan3_gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"),
                  "--expt-relaxed-constexpr"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-I" + os.path.join(ROOT, "include")]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []
    objs = {
        "es_engine.o": [nvcc] + NVFLAGS + extra + ["-c", os.path.join(CSRC, "es_engine.cu"), "-o"],
        "es_noalloc.o": [nvcc] + NVFLAGS + extra + ["-c", os.path.join(CSRC, "es_noalloc.cu"), "-o"],
        "es_wheel.o": ["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, "es_wheel.cpp"), "-o"],
        "es_digest.o": ["g++"] + CXXFLAGS + ["-O3", "-c", os.path.join(CSRC, "es_digest.cpp"), "-o"],
        "es_cli.o": ["g++"] + CXXFLAGS + ["-c", os.path.join(CSRC, "es_cli.cpp"), "-o"],
    }
    logs = []
    with ThreadPoolExecutor(max_workers=5) as ex:
        futs = [ex.submit(_run, cmd + [os.path.join(BUILD, o)]) for o, cmd in objs.items()]
        for f in futs:
            logs.append(f.result())
    _run([nvcc] + ARCH + ["-shared", "-ldl", "-o", LIB, os.path.join(BUILD, "es_engine.o"), os.path.join(BUILD, "es_noalloc.o"),
                          os.path.join(BUILD, "es_wheel.o"), os.path.join(BUILD, "es_digest.o")])
    _run(["g++", "-o", CLI, os.path.join(BUILD, "es_cli.o"), "-L" + HERE, "-les_sieve", "-Wl,-rpath,$ORIGIN",
          "-pthread"])
    if verbose or ptxas_info:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB, CLI)
