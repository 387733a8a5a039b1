"""Builds libshci_gpu.so in-tree for sm_103a with nvcc (no cmake).

Each translation unit is compiled in parallel, then linked into
dice_gb300/libshci_gpu.so next to this file. `python -m dice_gb300.build`
does the same from a shell.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshci_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["kernels_core.cu", "kernels_ham.cu", "kernels_select.cu", "kernels_sigma.cu", "kernels_mlp.cu",
                "kernels_pt.cu", "kernels_rdm.cu", "engine.cu"]
CXX_SOURCES = ["host_io.cpp"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers_mtime():
    m = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) > max(os.path.getmtime(path), _headers_mtime()) \
            and not os.environ.get("SHCI_NVCC_FLAGS"):
        return obj
    common = ["-O3", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    common += os.environ.get("SHCI_NVCC_FLAGS", "").split()  # extra flags for experiments
    if src.endswith(".cu"):
        cmd = [nvcc()] + ARCH + common + ["-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
                                          "-Xptxas", "-O3", "-c", path, "-o", obj]
    else:
        cmd = [nvcc(), "-x", "c++"] + common + ["-Xcompiler", "-fPIC", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = CUDA_SOURCES + CXX_SOURCES
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) > max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
