"""Builds the in-tree shared library libtp_gb300.so (CUDA kernels for
sm_103a + the C ABI + the host side) and the `tp_run` command-line driver.

Each translation unit compiles in parallel; host C++ is built with
-ffp-contract=off so that the kept host arithmetic (finalisation, constants)
rounds exactly like the reference on every architecture (aarch64 compilers
fuse a*b+c by default).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtp_gb300.so")
CLI = os.path.join(HERE, "tp_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc():
    for cand in (os.path.join(CUDA_HOME, "bin", "nvcc"), shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s" % (" ".join(cmd), p.stdout))
    return p.stdout


def build(verbose=False, extra_nvcc=()):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", CSRC, "-I", os.path.join(HERE, "..", "include")]
    host_flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]
    jobs = []
    for src in ("tp_kernels.cu", "tp_noalloc.cu"):
        obj = os.path.join(BUILD, src + ".o")
        jobs.append([nvcc, "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-std=c++17", *ARCH,
                     "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-v", *inc, *extra_nvcc])
    for src in ("tp_capi.cpp", "tp_host.cpp", "tp_rng.cpp", "tp_main.cpp"):
        obj = os.path.join(BUILD, src + ".o")
        jobs.append(["g++", "-c", os.path.join(CSRC, src), "-o", obj, *host_flags, *inc,
                     "-I", os.path.join(CUDA_HOME, "include")])
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    objs = [os.path.join(BUILD, s + ".o")
            for s in ("tp_kernels.cu", "tp_noalloc.cu", "tp_capi.cpp", "tp_host.cpp", "tp_rng.cpp")]
    cudalib = ["-L", os.path.join(CUDA_HOME, "lib64"), "-lcudart"]
    _run([nvcc, "-shared", *ARCH, "-o", LIB + ".tmp", *objs, *cudalib])
    os.replace(LIB + ".tmp", LIB)
    _run(["g++", "-o", CLI, os.path.join(BUILD, "tp_main.cpp.o"), LIB, "-Wl,-rpath,$ORIGIN", *cudalib,
          "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")])
    return outs[0]


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
