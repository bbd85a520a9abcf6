"""Builds libpga_gb300.so in-tree for sm_103a (nvcc only, no cmake).

Each translation unit compiles in parallel; the shared library links the
CUDA runtime statically so it loads in any process (ctypes, torch, C++).
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
# PGA_CHECKS=1 builds the bounds-checked variant (every table, queue and output
# access checked; a failed check raises PGA_ERR_INTERNAL instead of accessing).
CHECKED = os.environ.get("PGA_CHECKS") == "1"
LIB = os.path.join(HERE, "libpga_gb300_checked.so" if CHECKED else "libpga_gb300.so")
SOURCES = ["derive.cu", "derive_gen.cu", "derive_blk.cu", "lbvh.cu", "mesh.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no FMA contraction anywhere in the derivation path (the kernels
# also use explicit round-to-nearest intrinsics); -ffp-contract=off for the
# host code, which builds Rotate's matrices as the reference's host code does
# (gcc contracts to FMA by default on aarch64).
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off"]
if CHECKED:
    FLAGS += ["-DPGA_CHECKS=1"]
    BUILD = BUILD + "_checked"


def nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _deps_mtime():
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    paths.append(os.path.join(HERE, "..", "include", "pga_gb300.h"))
    return max(os.path.getmtime(p) for p in paths)


def up_to_date():
    return os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime()


def build(force=False, verbose=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)

    def compile_one(src):
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc()] + ARCH + FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
