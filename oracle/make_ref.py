#!/usr/bin/env python3
"""Build recipe for oracle/_ref: the reference's OWN host-side derivation path.

This is test infrastructure (a checker), never part of the product.

What it does
------------
1. When the reference checkout is present (first argument, default
   /root/reference), copy the header-only operator library it ships
   (``include/pga/core``), the vendored math headers (``deps/math/include``),
   the Whippletree headers that ``CPUEvaluator.h`` pulls in
   (``deps/whippletree/include``) and the mesh vertex counts
   (``include/pga/rendering/ShapeMeshAttributes.cuh``) into ``oracle/_ref/shadow``.  Nothing is
   copied into the tracked tree: ``oracle/_ref`` is git-ignored.
2. Apply the mechanical MSVC-portability edits listed in ``EDITS`` to the
   shadow copy.  None of them touches operator math: they replace
   ``std::exception(const char*)`` (an MSVC extension) with
   ``std::runtime_error``, add missing ``template``/``typename`` keywords,
   drop ``cudaDeviceProp::clockRate`` (removed in CUDA 13) from the unused
   instrumentation code, and fix two undeclared identifiers in ``toString``
   helpers.
3. Compile ``oracle/ref_harness.cu`` against the shadow copy with
   ``-DPGA_CPU -ffp-contract=off`` into ``oracle/_ref/ref_harness``.

When the reference checkout is absent (the GPU host), step 1-2 are skipped
and the shadow copy that travelled with the working tree is used as is.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SHADOW = os.path.join(REF_OUT, "shadow")

# (relative path in shadow, old text, new text, expected number of occurrences)
EDITS = [
    ("pga/core/CPUBaseContext.h", "#pragma once\n", "#pragma once\n#include <stdexcept>\n", 1),
    ("pga/core/CUDAException.h", "#include <exception>", "#include <stdexcept>", 1),
    ("pga/core/CUDAException.h", "public std::exception", "public std::runtime_error", 1),
    ("pga/core/CUDAException.h", "std::exception(getErrorString(error, file, line).c_str())",
     "std::runtime_error(getErrorString(error, file, line))", 1),
    ("pga/core/CUDAException.h", "std::exception(cudaGetErrorString(error))",
     "std::runtime_error(cudaGetErrorString(error))", 1),
    ("pga/core/Instrumentation.cuh", "realTechnique->insertIntoQueue<",
     "realTechnique->template insertIntoQueue<", 1),
    ("pga/core/Instrumentation.cuh", "realTechnique->execute<",
     "realTechnique->template execute<", 2),
    ("pga/core/Instrumentation.cuh", "prop.clockRate", "0", 2),
    ("pga/core/Instrumentation.h", "prop.clockRate * 1000ULL", "0", 1),
    ("pga/core/LinkedList.cuh", "int j, BaseDoublyLinkedList<T, N>::Node& n",
     "int j, typename BaseDoublyLinkedList<T, N>::Node& n", 1),
    ("pga/core/Parameters.cuh", "std::to_string(Index)", "std::to_string((ComponentT * 4) + AxisT)", 1),
    ("pga/core/Parameters.cuh", "packOperand(ORT_RAND, packFloat2(",
     "packOperand(ORT_RAND, PackUtils::packFloat2(", 1),
]


def make_shadow(ref_root):
    if os.path.isdir(SHADOW):
        shutil.rmtree(SHADOW)
    os.makedirs(SHADOW)
    shutil.copytree(os.path.join(ref_root, "include", "pga", "core"), os.path.join(SHADOW, "pga", "core"))
    shutil.copytree(os.path.join(ref_root, "deps", "math", "include", "math"), os.path.join(SHADOW, "math"))
    shutil.copytree(os.path.join(ref_root, "deps", "whippletree", "include"), os.path.join(SHADOW, "whippletree"))
    # the vertex and index counts of the triangle-mesh generation function
    os.makedirs(os.path.join(SHADOW, "pga", "rendering"))
    shutil.copy(os.path.join(ref_root, "include", "pga", "rendering", "ShapeMeshAttributes.cuh"),
                os.path.join(SHADOW, "pga", "rendering", "ShapeMeshAttributes.cuh"))
    stubs = os.path.join(SHADOW, "stubs")
    os.makedirs(stubs)
    # HighResClock.h and ClockCycleCounter.cuh include Windows headers but use
    # their non-Windows branches on Linux; empty stand-ins satisfy the include.
    for name in ("windows.h", "intrin.h"):
        with open(os.path.join(stubs, name), "w") as f:
            f.write("#pragma once\n")
    for rel, old, new, count in EDITS:
        path = os.path.join(SHADOW, rel)
        with open(path, "r", encoding="latin-1") as f:
            text = f.read()
        found = text.count(old)
        if found != count:
            raise SystemExit(f"make_ref: edit for {rel!r} expected {count} match(es) of {old!r}, found {found}")
        text = text.replace(old, new)
        with open(path, "w", encoding="latin-1") as f:
            f.write(text)


def build_harness():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = os.path.join(REF_OUT, "ref_harness")
    cmd = [nvcc, "-std=c++14", "-O2", "-DPGA_CPU", "-Xcompiler", "-ffp-contract=off",
           "-w", "-I", os.path.join(SHADOW, "stubs"), "-I", SHADOW,
           "-I", os.path.join(SHADOW, "whippletree"),
           os.path.join(HERE, "ref_harness.cu"), "-o", out, "-lcupti"]
    subprocess.check_call(cmd)
    return out


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if os.path.isdir(os.path.join(ref_root, "include", "pga", "core")):
        make_shadow(ref_root)
    elif not os.path.isdir(SHADOW):
        print("make_ref: no reference checkout and no shadow copy; oracle/_ref not built")
        return 1
    print(build_harness())
    return 0


if __name__ == "__main__":
    sys.exit(main())
