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
//
// Rotate (Rotate.cuh:24-41) leaves that set.  The device code is therefore
// compiled twice: by default with frame codes, and with PGA_GENERAL_FRAMES
// (derive_gen.cu, for tables with Rotate rules) with the rotation as nine
// floats and the reference's 4x4 products written out term by term.  The shape
// state and the kernels of each build live in an inline namespace of their
// own (pga::perm, pga::gen), so the two sets of kernels have distinct names.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/pga_gb300.h"

#ifndef PGA_GENERAL_FRAMES
#define PGA_GENERAL_FRAMES 0
#endif
// PGA_INLINE_BLOCKS (derive_blk.cu): the frame-code build again, with block
// parameters (PGA_PT_BLOCK) read inline instead of on the out-of-line path;
// engines whose table has block parameters launch it.  A separate build so
// that the kernels of tables without them keep their register allocation.
#ifndef PGA_INLINE_BLOCKS
#define PGA_INLINE_BLOCKS 0
#endif
#if PGA_GENERAL_FRAMES
#define PGA_FRAMES_NS gen
#elif PGA_INLINE_BLOCKS
#define PGA_FRAMES_NS permb
#else
#define PGA_FRAMES_NS perm
#endif

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
constexpr uint16_t kRuleMesh = 8;           // a triangle-mesh Generate (lowered to op GENERATE for the derivation)
constexpr uint16_t kRuleScalar = 16;        // every parameter a scalar constant
constexpr uint32_t kRulePhaseShift = 8;     // flags bits 8..11: the phase of the edges into the rule (multi-phase)
constexpr uint32_t kMaxPhases = 16;

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
  unsigned long long cursor;      // next dynamic chunk of the level being expanded (PGA_FLAG_DYNAMIC_CHUNKS)
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
  const uint32_t* axiomOrder;  // seed order: axiomOrder[i] is the i-th axiom seeded (null: index order)
  const float* blocks;
  uint32_t blockStride;
  PgaTerminal* out;
  unsigned long long cap;
  unsigned long long* outCount;
  Node* nodes;
  unsigned long long nodeCap;
  float4* nodeRot;           // general frames: rotation entries 0..7 of each item (2 x float4; entry 8 in Node::sf.w)
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
  uint32_t inlineLeaves;  // expand kRuleLeaf children in the lane that creates them
  PgaTerminal* tail;      // terminal slots at or beyond `cap` (pages straddling the end of the output)
  uint2* tailLinks;
  unsigned long long tailCap;
  unsigned long long* scratch;  // compaction: 6 x (warps + 2) words
  uint32_t numWarps;
  uint32_t tableInSmem; // 1: rule table copied to shared memory at launch
  uint32_t numParams, numSucc;
  DevState* st;
  // Multi-phase derivation (tables whose successors name phases > 0).
  uint32_t phase;                      // the phase being derived
  const Node* deferIn;                 // shapes deferred to this phase (seeded instead of the axioms when set)
  const float4* deferRotIn;            // their rotations (general frames)
  unsigned long long numDeferIn;
  Node* deferOut;                      // shapes reaching a rule of a later phase
  float4* deferRotOut;
  unsigned long long deferCap;
  unsigned long long* phaseCounters;   // [0] colliders stored, [1] shapes deferred by this launch
  PgaTerminal* colRec;                 // Collider shapes as records (model * scale, tag, path): the LBVH input
  float4* colShape;                    // and as oriented boxes: 5 float4 per collider (see store_collider)
  unsigned long long colCap;
  const int32_t* colNodes;             // LBVH over the colliders of earlier phases
  const float* colAabbs;
  const uint32_t* colLeaf;
  uint32_t numColliders;
};

// Entry points of one build of the kernels (host stubs), for the host code.
struct FrameKernels {
  const void* persistent[4];  // k_derive_persistent<LEAF, AFF = 0 / 1>, index LEAF + 2 AFF
  const void* persistentDyn[2];  // k_derive_persistent<false, AFF = 0 / 1, DYN = true> (PGA_FLAG_DYNAMIC_CHUNKS)
  const void* phased;         // k_derive_persistent<false, 2>: multi-phase tables
  const void* seed;           // k_seed (plain form)
  const void* expand;         // k_expand_level (plain form)
  const void* adjoint;        // k_adjoint: the one the engine launches
  const void* adjointWide;    // k_adjoint_wide (3 blocks per SM; the general-frame build: k_adjoint)
};

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

// ------------------------------------------------------------ shape state

inline namespace PGA_FRAMES_NS {

struct Shape {
  float t[3];      // translation (model column 3)
  float s[3];      // size
  float seed;
#if PGA_GENERAL_FRAMES
  float R[9];      // rotation (model columns 0..2), row-major
#else
  uint32_t frame;  // rotation: bits 2j..2j+1 = row of column j's nonzero, bit 6+j = column j negated
#endif
  int32_t entry;
  uint32_t axiom;
  uint32_t kind;   // PgaShape
  uint64_t path;
};

#if PGA_GENERAL_FRAMES

__device__ __forceinline__ void frame_identity(Shape& x) {
#pragma unroll
  for (int k = 0; k < 9; k++) x.R[k] = (k % 4 == 0) ? 1.0f : 0.0f;
}
// R[row][col] for run-time row and col, without local memory.
__device__ __forceinline__ float frame_at(const Shape& x, uint32_t row, uint32_t col) {
  const float r0 = pick3(&x.R[0], col), r1 = pick3(&x.R[3], col), r2 = pick3(&x.R[6], col);
  return row == 0 ? r0 : (row == 1 ? r1 : r2);
}
// The model axis a translation runs along.
struct AxisRef {
  uint32_t col;
};
__device__ __forceinline__ AxisRef axis_ref(const Shape&, uint32_t ax) { return AxisRef{ax}; }
// model * translate(o e_col): column 3 of the 4x4 product is, per row,
// ((R[i][0] T03 + R[i][1] T13) + R[i][2] T23) + t_i with one nonzero T, so
// t_i' = fl(fl(R[i][col] * o) + t_i) (the other products are exact zeros).
__device__ __forceinline__ void translate_ref(Shape& y, const Shape& x, AxisRef r, float o) {
  const float t0 = __fadd_rn(__fmul_rn(pick3(&x.R[0], r.col), o), x.t[0]);
  const float t1 = __fadd_rn(__fmul_rn(pick3(&x.R[3], r.col), o), x.t[1]);
  const float t2 = __fadd_rn(__fmul_rn(pick3(&x.R[6], r.col), o), x.t[2]);
  y.t[0] = t0;
  y.t[1] = t1;
  y.t[2] = t2;
}
// y's rotation = x's with columns ca and cb replaced by x's columns sa and sb,
// negated when fa / fb (the products with the fixed face and extrude matrices,
// whose entries are 0 and +-1).  The column arguments are constants at every
// call site, so the entries stay in registers.
__device__ __forceinline__ void frame_set2(Shape& y, const Shape& x, uint32_t ca, uint32_t sa, uint32_t fa,
                                           uint32_t cb, uint32_t sb, uint32_t fb) {
  float nr[9];
#pragma unroll
  for (int k = 0; k < 9; k++) nr[k] = x.R[k];
#pragma unroll
  for (uint32_t i = 0; i < 3; i++) {
    nr[i * 3 + ca] = fa ? -x.R[i * 3 + sa] : x.R[i * 3 + sa];
    nr[i * 3 + cb] = fb ? -x.R[i * 3 + sb] : x.R[i * 3 + sb];
  }
#pragma unroll
  for (int k = 0; k < 9; k++) y.R[k] = nr[k];
}
// R[i][j] * s_j: column j of model4 * scale(size).
__device__ __forceinline__ void frame_scaled(const Shape& x, float m[3][3]) {
#pragma unroll
  for (uint32_t i = 0; i < 3; i++)
#pragma unroll
    for (uint32_t j = 0; j < 3; j++) m[i][j] = __fmul_rn(x.R[i * 3 + j], x.s[j]);
}
// model4 * rotateXYZ(q) (Rotate.cuh:37, matrix.h:776-782): R'[i][j] =
// ((R[i][0] q[0][j] + R[i][1] q[1][j]) + R[i][2] q[2][j]) + t_i * 0; the
// translation is unchanged.
__device__ __forceinline__ void frame_rotate(Shape& x, const float* q) {
  // row by row: a row of R' needs only that row of R, so the update is in
  // place and q is read as it is used (fewer live registers than a copy)
#pragma unroll
  for (uint32_t i = 0; i < 3; i++) {
    const float r0 = x.R[i * 3 + 0], r1 = x.R[i * 3 + 1], r2 = x.R[i * 3 + 2];
#pragma unroll
    for (uint32_t j = 0; j < 3; j++)
      x.R[i * 3 + j] = __fadd_rn(__fadd_rn(__fmul_rn(r0, q[j]), __fmul_rn(r1, q[3 + j])),
                                 __fmul_rn(r2, q[6 + j]));
  }
}

#else  // signed-permutation frames

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

__device__ __forceinline__ void frame_identity(Shape& x) { x.frame = kIdentityFrame; }
__device__ __forceinline__ float frame_at(const Shape& x, uint32_t row, uint32_t col) {
  return frame_entry(x.frame, row, col);
}
// The model axis a translation runs along: its row in the frame and its sign.
struct AxisRef {
  uint32_t row;
  float sign;
};
__device__ __forceinline__ AxisRef axis_ref(const Shape& x, uint32_t ax) {
  return AxisRef{frame_row(x.frame, ax), frame_neg(x.frame, ax) ? -1.0f : 1.0f};
}
// Translation by o along a model axis: t' = fl(fl(R[:,ax] * o) + t), which
// for a signed-permutation R is one rounded add in row perm_ax.
__device__ __forceinline__ void translate_ref(Shape& y, const Shape& x, AxisRef r, float o) {
  const float v = __fmul_rn(r.sign, o);  // exact: sign is +-1
#pragma unroll
  for (uint32_t i = 0; i < 3; i++) y.t[i] = (i == r.row) ? __fadd_rn(v, x.t[i]) : x.t[i];
}
__device__ __forceinline__ void frame_set2(Shape& y, const Shape& x, uint32_t ca, uint32_t sa, uint32_t fa,
                                           uint32_t cb, uint32_t sb, uint32_t fb) {
  const uint32_t f = x.frame;
  y.frame = frame_set(frame_set(f, ca, f, sa, fa), cb, f, sb, fb);
}
// R[i][j] * s_j is exactly +-s_j in row perm_j and zero elsewhere.
__device__ __forceinline__ void frame_scaled(const Shape& x, float m[3][3]) {
#pragma unroll
  for (uint32_t j = 0; j < 3; j++) {
    const uint32_t row = frame_row(x.frame, j);
    const float v = frame_neg(x.frame, j) ? -x.s[j] : x.s[j];
#pragma unroll
    for (uint32_t i = 0; i < 3; i++) m[i][j] = (i == row) ? v : 0.0f;
  }
}

#endif

__device__ __forceinline__ void translate_axis(Shape& y, const Shape& x, uint32_t ax, float o) {
  translate_ref(y, x, axis_ref(x, ax), o);
}

// Shape::at (include/pga/core/Shape.cuh:120-171).
__device__ __forceinline__ float shape_attr(const Shape& x, uint32_t i, float custom) {
  if (i < 12) {
    uint32_t row = i >> 2, col = i & 3;
    return col == 3 ? pick3(x.t, row) : frame_at(x, row, col);
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

}  // inline namespace PGA_FRAMES_NS
}  // namespace pga
