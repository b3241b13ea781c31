"""Builds libberthagpu.so in-tree with nvcc for sm_103a."""
import os
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
REPO = os.path.dirname(ROOT)
SRC = os.path.join(ROOT, "csrc", "bertha_gpu.cu")
INC = os.path.join(REPO, "include")
LIB = os.path.join(PKG, "libberthagpu.so")

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-shared",
]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    hdr = os.path.join(INC, "bertha_gpu.h")
    csrc = os.path.dirname(SRC)
    deps = [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cu", ".cuh"))]
    return any(os.path.getmtime(p) > t for p in deps + [hdr, __file__])


def build(force=False, verbose=False):
    """Compile the CUDA library; returns the path of the shared object."""
    if not force and not needs_build():
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + NVCC_FLAGS + ["-I" + INC, "-o", tmp, SRC]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB
