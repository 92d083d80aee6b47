"""Builds libether_gpu.so in-tree (ether_gb300/libether_gpu.so) for sm_103a.

Each translation unit is compiled in parallel with nvcc (CUDA) or g++ (host C++), then
linked with nvcc.  The CUDA units use --fmad=false: the sweep kernels round every FP32
operation separately and fuse only where the source calls fmaf(), which keeps the GPU
bit-reproducible against the CPU mirror of the same expressions.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libether_gpu.so")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["ether_api.cu", "k_ising.cu", "k_xyz.cu", "k_obs.cu", "noalloc.cu", "k_sq.cu", "k_batch.cu", "k_learn.cu", "k_learn_xyz.cu", "k_moments.cu", "k_ion.cu"]
CXX = ["lattice.cpp", "deck.cpp"]


def _nvcc():
    for p in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if p and os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(verbose=False):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    jobs = []
    for f in CU:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                     "-c", os.path.join(CSRC, f), "-o", obj])
    for f in CXX:
        obj = os.path.join(BUILD, f + ".o")
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                     "-I", os.path.join(os.path.dirname(nvcc), "..", "include"),
                     "-c", os.path.join(CSRC, f), "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    objs = [os.path.join(BUILD, f + ".o") for f in CU + CXX]
    tmp = OUT + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs, "-Xlinker", "--no-undefined"])
    os.replace(tmp, OUT)
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
