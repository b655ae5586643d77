"""Build libtopopt_gb300.so in-tree with nvcc for sm_103a (no cmake, no torch).

    python topopt.jl_gb300/build.py

The translation units are compiled in parallel and linked with the static
CUDA runtime, so the library needs only the NVIDIA driver at run time.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtopopt_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-I" + os.path.join(HERE, "..", "include")]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    jobs = [
        [NVCC] + COMMON + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, "tog_api.cu"),
                                  "-o", os.path.join(BUILD, "tog_api.o")] + (["-Xptxas", "-v"] if verbose else []),
        [NVCC] + COMMON + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, "tog_batch.cu"),
                                  "-o", os.path.join(BUILD, "tog_batch.o")],
        [NVCC] + COMMON + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, "tog_noalloc.cu"),
                                  "-o", os.path.join(BUILD, "tog_noalloc.o")],
        [NVCC] + COMMON + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, "tog_nn.cu"),
                                  "-o", os.path.join(BUILD, "tog_nn.o")],
        [NVCC] + COMMON + ["-x", "c++", "-c", os.path.join(CSRC, "tog_host.cpp"),
                           "-o", os.path.join(BUILD, "tog_host.o")],
    ]
    with ThreadPoolExecutor(len(jobs)) as ex:
        logs = list(ex.map(_run, jobs))
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp, os.path.join(BUILD, "tog_api.o"), os.path.join(BUILD, "tog_batch.o"),
                          os.path.join(BUILD, "tog_noalloc.o"), os.path.join(BUILD, "tog_nn.o"),
                          os.path.join(BUILD, "tog_host.o")])
    os.replace(tmp, LIB)
    if verbose:
        print("".join(logs))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
