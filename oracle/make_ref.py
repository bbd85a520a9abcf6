#!/usr/bin/env python3
"""Build recipe for oracle/_ref: the reference's OWN host-side derivation path.

This is test infrastructure (a checker), never part of the product.

What it does
------------
1. When the reference checkout is present (first argument, default
   REFERENCE_ROOT below), copy the header-only operator library it ships
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
   helpers.  Then apply ``PATH_EDITS``: a derivation-path hash carried on
   every symbol and mixed at the reference's own child-creation call sites,
   so the reference's evaluator reports the path of each terminal.
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
# The reference checkout this recipe reads (PGA_REFERENCE_ROOT overrides it);
# the rest of the repository takes the path from here.
REFERENCE_ROOT = os.environ.get("PGA_REFERENCE_ROOT", "/root/reference")
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


# Derivation-path instrumentation.  The reference has no path hash, so these
# edits add one without touching operator math: a 64-bit field on Symbol
# (copied with the symbol), set at the axiom from the axiom index and, at every
# call site that creates a child or takes a branch, mixed from the parent's
# hash, the child's ordinal and the child's entry index.  The ordinal is the
# seed modifier the site already uses (Subdivide k, Repeat 1 / i / reps,
# ComponentSplit face + 2 / bottom 1 / top 0, Extrude 0), or the successor
# taken (IfSizeLess and If: 0 true / 1 false; RandomRule: the pair picked;
# Replicate: the successor).  In-place 1->1 operators (Translate, Scale,
# Rotate, SwapSize) keep the hash.  The mix is the splitmix64 finaliser:
# root = mix(axiom + 0x9E3779B97F4A7C15), child = mix(parent ^ (ordinal << 32 | entry)).
PATH_HELPERS = r"""
namespace PGA
{
	namespace Operators { template <unsigned int SuccessorOffsetT, int EdgeIndexT> class DCall; }
	namespace PathHash
	{
		__host__ __device__ inline unsigned long long mix(unsigned long long z)
		{
			z ^= z >> 30; z *= 0xbf58476d1ce4e5b9ULL;
			z ^= z >> 27; z *= 0x94d049bb133111ebULL;
			z ^= z >> 31;
			return z;
		}
		// Axiom index of the axiom being generated, and the number of entries of
		// one table copy when a batch gives each axiom its own copy (0: none).
		inline unsigned long long& currentAxiom() { static unsigned long long a = 0; return a; }
		inline unsigned int& entryModulus() { static unsigned int m = 0; return m; }
		inline unsigned long long root() { return mix(currentAxiom() + 0x9E3779B97F4A7C15ULL); }
		__host__ __device__ inline unsigned long long child(unsigned long long parent, unsigned int ordinal, int entry)
		{
			unsigned int e = (unsigned int)entry;
#if (!defined(__CUDA_ARCH__) || (__CUDA_ARCH__ == 0))
			if (entryModulus() != 0) e %= entryModulus();
#endif
			return mix(parent ^ (((unsigned long long)ordinal << 32) | e));
		}
		// The successor offset of a DCall<k> (the branch a static RandomRule takes).
		template <typename T> struct Offset { static const unsigned int value = 0; };
		template <unsigned int S, int E> struct Offset<Operators::DCall<S, E> > { static const unsigned int value = S; };
	}
}
"""

PATH_EDITS = [
    ("pga/core/Symbol.cuh", "#include <math/vector.h>\n", "#include <math/vector.h>\n" + PATH_HELPERS, 1),
    ("pga/core/Symbol.cuh", "\t\tint predecessor;\n", "\t\tint predecessor;\n\t\tunsigned long long pathHash;\n", 1),
    ("pga/core/Symbol.cuh", "entryIndex(-1), predecessor(-1)", "entryIndex(-1), predecessor(-1), pathHash(0)", 2),
    ("pga/core/Symbol.cuh", "predecessor = other.predecessor;",
     "predecessor = other.predecessor; pathHash = other.pathHash;", 2),
    ("pga/core/CPUEvaluator.h", "symbol.entryIndex = entryIndex;",
     "symbol.entryIndex = entryIndex; symbol.pathHash = PathHash::root();", 2),
    # static Subdivide: ordinal = the pair's index (its seed modifier)
    ("pga/core/Subdivide.cuh", "SymbolDecorator<NextOperator>::run(symbol, &newSymbol);",
     "SymbolDecorator<NextOperator>::run(symbol, &newSymbol); "
     "newSymbol.pathHash = PathHash::child(symbol->pathHash, ParameterIndex, newSymbol.entryIndex);", 2),
    # Subdivide<DynParams>: the symbol is reused in place, so keep the parent's hash
    ("pga/core/Subdivide.cuh", "auto baseModel = symbol->getModel4();",
     "auto baseModel = symbol->getModel4(); auto basePath = symbol->pathHash;", 1),
    ("pga/core/Subdivide.cuh", "symbol->entryIndex = entry.successors[j].entryIndex;",
     "symbol->entryIndex = entry.successors[j].entryIndex; "
     "symbol->pathHash = PathHash::child(basePath, j, symbol->entryIndex);", 1),
    ("pga/core/Repeat.cuh",
     "newSymbol.setSeed(symbol->generateNextSeed(1.0f));\n\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol);",
     "newSymbol.setSeed(symbol->generateNextSeed(1.0f));\n\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol); "
     "newSymbol.pathHash = PathHash::child(symbol->pathHash, 1u, newSymbol.entryIndex);", 1),
    ("pga/core/Repeat.cuh",
     "generateNextSeed(static_cast<float>(i)));\n#endif\n\t\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol);",
     "generateNextSeed(static_cast<float>(i)));\n#endif\n\t\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol); "
     "newSymbol.pathHash = PathHash::child(symbol->pathHash, i, newSymbol.entryIndex);", 1),
    ("pga/core/Repeat.cuh",
     "generateNextSeed(static_cast<float>(repetitions)));\n#endif\n\t\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol);",
     "generateNextSeed(static_cast<float>(repetitions)));\n#endif\n\t\t\t\t\tSymbolDecorator<NextOperatorT>::run(symbol, &newSymbol); "
     "newSymbol.pathHash = PathHash::child(symbol->pathHash, repetitions, newSymbol.entryIndex);", 1),
    ("pga/core/ComponentSplit.cuh", "SymbolDecorator<SidesOperatorT>::run(symbol, &sideNewSymbol);",
     "SymbolDecorator<SidesOperatorT>::run(symbol, &sideNewSymbol); "
     "sideNewSymbol.pathHash = PathHash::child(symbol->pathHash, faceIndex + 2, sideNewSymbol.entryIndex);", 1),
    ("pga/core/ComponentSplit.cuh", "SymbolDecorator<BottomOperatorT>::run(symbol, &bottomNewSymbol);",
     "SymbolDecorator<BottomOperatorT>::run(symbol, &bottomNewSymbol); "
     "bottomNewSymbol.pathHash = PathHash::child(symbol->pathHash, 1u, bottomNewSymbol.entryIndex);", 1),
    ("pga/core/ComponentSplit.cuh", "SymbolDecorator<TopOperatorT>::run(symbol, &topNewSymbol);",
     "SymbolDecorator<TopOperatorT>::run(symbol, &topNewSymbol); "
     "topNewSymbol.pathHash = PathHash::child(symbol->pathHash, 0u, topNewSymbol.entryIndex);", 1),
    ("pga/core/Extrude.cuh", "SymbolDecorator<NextOperatorT>::run(symbol, &newSymbol);",
     "SymbolDecorator<NextOperatorT>::run(symbol, &newSymbol); "
     "newSymbol.pathHash = PathHash::child(symbol->pathHash, 0u, newSymbol.entryIndex);", 1),
    # If and IfSizeLess (in place): 0 for the true branch, 1 for the false one
    ("pga/core/If.cuh", "SymbolDecorator<NextOperatorIfTrueT>::run(symbol, symbol);",
     "SymbolDecorator<NextOperatorIfTrueT>::run(symbol, symbol); "
     "symbol->pathHash = PathHash::child(symbol->pathHash, 0u, symbol->entryIndex);", 2),
    ("pga/core/If.cuh", "SymbolDecorator<NextOperatorIfFalseT>::run(symbol, symbol);",
     "SymbolDecorator<NextOperatorIfFalseT>::run(symbol, symbol); "
     "symbol->pathHash = PathHash::child(symbol->pathHash, 1u, symbol->entryIndex);", 2),
    # static RandomRule: the picked pair's successor offset
    ("pga/core/RandomRule.cuh", "SymbolDecorator<NextOperator>::run(symbol, symbol);",
     "SymbolDecorator<NextOperator>::run(symbol, symbol); "
     "symbol->pathHash = PathHash::child(symbol->pathHash, PathHash::Offset<NextOperator>::value, symbol->entryIndex);", 2),
    ("pga/core/RandomRule.cuh", "symbol->entryIndex = entry.successors[i - 1].entryIndex;",
     "symbol->entryIndex = entry.successors[i - 1].entryIndex; "
     "symbol->pathHash = PathHash::child(symbol->pathHash, i - 1, symbol->entryIndex);", 1),
    # Replicate<DynParams>: the symbol is reused in place, so keep the parent's hash
    ("pga/core/Replicate.cuh", "auto numParameters = entry.numSuccessors;",
     "auto numParameters = entry.numSuccessors; auto basePath = symbol->pathHash;", 1),
    ("pga/core/Replicate.cuh", "symbol->entryIndex = entry.successors[i].entryIndex;",
     "symbol->entryIndex = entry.successors[i].entryIndex; "
     "symbol->pathHash = PathHash::child(basePath, i, symbol->entryIndex);", 1),
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
    for rel, old, new, count in EDITS + PATH_EDITS:
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
    ref_root = sys.argv[1] if len(sys.argv) > 1 else REFERENCE_ROOT
    if os.path.isdir(os.path.join(ref_root, "include", "pga", "core")):
        make_shadow(ref_root)
    elif not os.path.isdir(SHADOW):
        print("make_ref: no reference checkout and no shadow copy; oracle/_ref not built")
        return 1
    print(build_harness())
    return 0


if __name__ == "__main__":
    sys.exit(main())
