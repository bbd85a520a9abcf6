// Device-side core of the derivation engine: rule table, shape state, the
// operator semantics of the hot path and warp-aggregated emission.
//
// Every float operation of the derivation is written with explicit
// round-to-nearest intrinsics (__fadd_rn / __fmul_rn / __fdiv_rn, no FMA) so
// results are bit-identical to the reference's host build
// (include/pga/core/*.cuh compiled with -ffp-contract=off).  The reference
// multiplies full 4x4 matrices (deps/math/include/math/matrix.h:776-782); its
// products with translate(), scale() and the fixed face/extrude rotations
// reduce exactly to: translation t' = fl(fl(R[:,a] * o) + t) for a one-axis
// offset o, column permutations/negations of R, and R[:,j] * s_j (the other
// terms are products with exact zeros and ones).  Only the sign of a zero can
// differ, which no output distinguishes.
//
// Axioms start with the identity rotation (the reference's axiom generators
// only place and size them, Grid.cuh:199-204) and the operators of this path
// only permute and negate columns, so every rotation is a signed permutation.
// A shape therefore carries a 9-bit frame code instead of nine floats: column
// j of R is sign_j * e_{perm_j}.  fl(R[i][a] * o) is then exactly +-o in row
// perm_a and a signed zero elsewhere, so a translation is one rounded add.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pga_gb300.h"

namespace pga {

constexpr int kMaxChain = 64;           // inline 1->1 steps before PGA_ERR_DEPTH
constexpr uint32_t kAxiomLink = 0x80000000u;

// ------------------------------------------------------------ device tables

struct __align__(16) DevParam {
  int32_t type;    // PgaParameterType
  float v0, v1;    // value[0], value[1]
  uint32_t aux;    // PGA_PT_EXP: offset of its 16 values in the expression pool
};

struct __align__(16) DevRule {
  uint8_t op;        // PgaOperator, 0xFF = invalid operator code
  uint8_t shape;     // PgaShape the procedure expects
  uint8_t nParams;
  uint8_t nSucc;
  uint16_t nChildren;  // PGA_OP_SUBDIVIDE_STATIC
  uint16_t flags;      // kRulePure: no parameter reads the shape (scalar or block values only)
  uint32_t paramBase;  // into DevParam[]
  uint32_t succBase;   // into int32 successor entries
};
constexpr uint16_t kRulePure = 1;
constexpr uint16_t kRuleConstTerminal = 2;  // Generate with a scalar terminal index, kept in nChildren
constexpr uint16_t kRuleLeaf = 4;           // Subdivide whose children all end at once (expanded in place)

struct DevTables {
  const DevRule* rules;
  const DevParam* params;
  const int32_t* succ;
  const float* expPool;
  uint32_t numEntries;
};

// 64-byte queued work item: a shape plus the range of its children that this
// item produces (a branching shape with many children is queued as several
// items of at most `subItem` children each).
struct __align__(16) Node {
  float4 ts;     // translation xyz, size x
  float4 sf;     // size y, size z, seed, frame code (bits)
  uint4 meta;    // entry, axiom, path lo, path hi
  uint4 ext;     // first child, end child, tape link (parent item or kAxiomLink | axiom), ordinal
};

struct DevState {
  unsigned long long termCount;   // terminals emitted (exact, after compaction in the paged engine)
  unsigned long long nodeNext;    // queued item slots handed out (plain form)
  unsigned long long termPages;   // terminal pages handed out (paged engine)
  unsigned long long nodePages;   // item pages handed out (paged engine)
  unsigned long long cursor;
  unsigned long long levelLo, levelHi;
  unsigned long long maxLevelNodes;
  int32_t status, detail;
  uint32_t barrierArrive, barrierGen;
  uint32_t levels, stop;
  unsigned long long clockStart;  // %globaltimer when block 0 started (paged engine)
  unsigned long long clockEnd;    // %globaltimer when the last block finished
};

struct DeriveArgs {
  DevTables tab;
  const PgaAxiom* axioms;
  uint32_t numAxioms;
  uint32_t axiomBase;        // plain form: index of the first axiom of this launch
  const float* blocks;
  uint32_t blockStride;
  PgaTerminal* out;
  unsigned long long cap;
  unsigned long long* outCount;
  Node* nodes;
  unsigned long long nodeCap;
  uint2* termLinks;
  unsigned long long termLinkCap;
  unsigned long long* levelStart;
  unsigned long long* levelClock;  // %globaltimer when each level's range was fixed
  uint32_t maxLevels;
  uint32_t spinLimit;
  uint32_t subItem;     // children per queued item (1..8)
  uint32_t useSeeds;    // 0: no parameter of the grammar reads a seed, skip seed updates
  uint32_t itemsPerLane;
  uint32_t narrowSubItem;
  uint32_t inlineLeaves;      // expand kRuleLeaf children in the lane that creates them  // work items per lane in one warp chunk
  PgaTerminal* tail;      // terminal slots at or beyond `cap` (pages straddling the end of the output)
  uint2* tailLinks;
  unsigned long long tailCap;
  unsigned long long* scratch;  // compaction: 6 x (warps + 2) words
  uint32_t numWarps;
  uint32_t tableInSmem; // 1: rule table copied to shared memory at launch
  uint32_t numParams, numSucc;
  DevState* st;
};

// ------------------------------------------------------------ shape state

struct Shape {
  float t[3];      // translation (model column 3)
  float s[3];      // size
  float seed;
  uint32_t frame;  // rotation: bits 2j..2j+1 = row of column j's nonzero, bit 6+j = column j negated
  int32_t entry;
  uint32_t axiom;
  uint32_t kind;   // PgaShape
  uint64_t path;
};

constexpr uint32_t kIdentityFrame = 0u | (1u << 2) | (2u << 4);

__device__ __forceinline__ uint32_t frame_row(uint32_t f, uint32_t col) { return (f >> (2 * col)) & 3u; }
__device__ __forceinline__ uint32_t frame_neg(uint32_t f, uint32_t col) { return (f >> (6 + col)) & 1u; }
// Column `col` of the result is column `src` of f, negated when `flip`.
__device__ __forceinline__ uint32_t frame_set(uint32_t g, uint32_t col, uint32_t f, uint32_t src, uint32_t flip) {
  g &= ~((3u << (2 * col)) | (1u << (6 + col)));
  return g | (frame_row(f, src) << (2 * col)) | ((frame_neg(f, src) ^ flip) << (6 + col));
}
// R[row][col] of a frame: 0, 1 or -1.
__device__ __forceinline__ float frame_entry(uint32_t f, uint32_t row, uint32_t col) {
  return frame_row(f, col) == row ? (frame_neg(f, col) ? -1.0f : 1.0f) : 0.0f;
}

__device__ __forceinline__ void raise_error(DevState* st, int code, int detail) {
  if (atomicCAS(&st->status, 0, code) == 0) atomicExch(&st->detail, detail);
}

// Host static_cast<unsigned>(float) for the values grammars produce; negative
// and NaN give 0, huge values saturate (device conversion semantics).
__device__ __forceinline__ uint32_t f2u(float x) { return __float2uint_rz(x); }

// Random::hybridTaus / nextSeed (include/pga/core/Random.cuh:15-49).
__device__ __forceinline__ float next_seed(float base, uint32_t modifier) {
  uint32_t z = (f2u(base) * 0xFFFFFFFFu) + (modifier * 41231278u) % 0xFFFFFFFFu;
  uint32_t z1 = (z + 7873234u) % 0xFFFFFFFFu;
  uint32_t z2 = (z1 + 1237217827u) % 0xFFFFFFFFu;
  uint32_t z3 = (z2 + 87382u) % 0xFFFFFFFFu;
  uint32_t z4 = (z3 + 1410022u) % 0xFFFFFFFFu;
  uint32_t b1 = (((z1 << 13) ^ z1) >> 19); z1 = (((z1 & 4294967294u) << 12) ^ b1);
  uint32_t b2 = (((z2 << 2) ^ z2) >> 25);  z2 = (((z2 & 4294967288u) << 4) ^ b2);
  uint32_t b3 = (((z3 << 3) ^ z3) >> 11);  z3 = (((z3 & 4294967280u) << 17) ^ b3);
  z4 = 1664525u * z4 + 1013904223u;
  return __double2float_rn(__dmul_rn(2.3283064365387e-10, (double)(z1 ^ z2 ^ z3 ^ z4)));
}

// Random::range (Random.cuh:51-57).
__device__ __forceinline__ float rand_range(float seed, float lo, float hi) {
  return seed < 1.0f ? __fadd_rn(__fmul_rn(seed, __fsub_rn(hi, lo)), lo) : hi;
}

// Derivation-path hash: splitmix64 finaliser (no reference counterpart).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z ^= z >> 30; z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27; z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
__device__ __forceinline__ uint64_t child_path(uint64_t parent, uint32_t ordinal, int32_t entry) {
  return mix64(parent ^ (((uint64_t)ordinal << 32) | (uint32_t)entry));
}

// Component k (0..2) of a 3-vector without run-time indexing (keeps shapes in
// registers instead of local memory).
__device__ __forceinline__ float pick3(const float v[3], uint32_t k) {
  return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]);
}
__device__ __forceinline__ void put3(float v[3], uint32_t k, float x) {
  v[0] = (k == 0) ? x : v[0];
  v[1] = (k == 1) ? x : v[1];
  v[2] = (k == 2) ? x : v[2];
}

// Shape::at (include/pga/core/Shape.cuh:120-171).
__device__ __forceinline__ float shape_attr(const Shape& x, uint32_t i, float custom) {
  if (i < 12) {
    uint32_t row = i >> 2, col = i & 3;
    return col == 3 ? pick3(x.t, row) : frame_entry(x.frame, row, col);
  }
  if (i < 15) return pick3(x.s, i - 12);
  if (i == 15) return x.seed;
  if (i == 16) return custom;
  return 0.0f;
}

// EncExp<Stack<4>>::eval (include/pga/core/Parameters.cuh:518-664).
__device__ inline float eval_exp(const float* b, const Shape& x, float custom, DevState* st) {
  float stack[PGA_MAX_EXP_LEVELS];
  uint32_t top = 0;
  uint32_t size = f2u(b[0]);
  for (uint32_t i = 1; i <= size && i < PGA_MAX_NUM_PARAMETER_VALUES; i++) {
    uint32_t r = __float_as_uint(b[i]);
    uint32_t p = r >> 30;
    float v = __uint_as_float(r << 2);
    float val;
    if (p == 0) {
      val = v;
    } else if (p == 1) {  // PackUtils::unpackFloat2 (PackUtils.h:39-43)
      float hi = __fdiv_rn(fmodf(v, 4096.0f), 4095.0f);
      float lo = __fdiv_rn(floorf(__fdiv_rn(v, 4096.0f)), 4095.0f);
      val = rand_range(x.seed, lo, hi);
    } else if (p == 2) {
      val = shape_attr(x, f2u(roundf(v)), custom);
    } else {
      if (top < 2) { raise_error(st, PGA_ERR_BAD_PARAM, x.entry); return 0.0f; }
      float p2 = stack[--top], p1 = stack[--top];
      switch (f2u(roundf(v))) {
        case 0: val = __fadd_rn(p1, p2); break;
        case 1: val = __fsub_rn(p1, p2); break;
        case 2: val = __fdiv_rn(p1, p2); break;
        case 3: val = __fmul_rn(p1, p2); break;
        case 4: val = (float)(p1 == p2); break;
        case 5: val = (float)(p1 != p2); break;
        case 6: val = (float)(p1 < p2); break;
        case 7: val = (float)(p1 > p2); break;
        case 8: val = (float)(p1 <= p2); break;
        case 9: val = (float)(p1 >= p2); break;
        case 10: val = (float)(p1 != 0.0f && p2 != 0.0f); break;
        case 11: val = (float)(p1 != 0.0f || p2 != 0.0f); break;
        default: val = 0.0f; break;
      }
    }
    if (top >= PGA_MAX_EXP_LEVELS) { raise_error(st, PGA_ERR_BAD_PARAM, x.entry); return 0.0f; }
    stack[top++] = val;
  }
  if (top == 0) { raise_error(st, PGA_ERR_BAD_PARAM, x.entry); return 0.0f; }
  return stack[top - 1];
}

}  // namespace pga
