// Derivation kernels (device code of derive.cu), compiled once per frame
// representation: derive.cu includes it with signed-permutation frame codes,
// derive_gen.cu with PGA_GENERAL_FRAMES (general rotations, for Rotate) and
// derive_blk.cu with PGA_INLINE_BLOCKS (frame codes, block parameters read
// inline).  Everything here is in the build's inline namespace
// (pga::perm / pga::gen / pga::permb).
#pragma once

#include <cuda_runtime.h>

#include "engine.cuh"

namespace pga {
inline namespace PGA_FRAMES_NS {


constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kMaxAdjointBlocks = 8192;  // blocks of the reverse launch (slot-map scan)
// Engines with at least this terminal capacity launch the 3-blocks-per-SM adjoint (k_adjoint_wide).
constexpr unsigned long long kWideAdjointTerminals = 1ull << 23;
enum Kind { kNone = 0, kTerm = 1, kNode = 2 };

struct __align__(16) Smem {
  // Rule table of this block: generic pointers to the shared-memory copy or to
  // global memory, fixed once in setup_block (no per-access address-space choice).
  const DevRule* rules;
  const DevParam* params;
  const int32_t* succ;
};

extern __shared__ __align__(16) unsigned char smem_raw[];

// Checked builds (-DPGA_CHECKS) test every table, queue and axiom index
// before the access; a failure raises PGA_ERR_INTERNAL with the site number and
// skips the access.
#ifdef PGA_CHECKS
#define PGA_GUARD(cond, site, ...)                  \
  do {                                              \
    if (!(cond)) {                                  \
      raise_error(a.st, PGA_ERR_INTERNAL, (site));  \
      __VA_ARGS__;                                  \
    }                                               \
  } while (0)
#else
#define PGA_GUARD(cond, site, ...) \
  do {                             \
  } while (0)
#endif

__device__ __forceinline__ Smem& block_smem() { return *reinterpret_cast<Smem*>(smem_raw); }

// Rule-table reads through the block's table pointers (shared-memory copy when
// the table fits, else global memory).
__device__ __forceinline__ DevRule rule_at(const DeriveArgs& a, uint32_t e) {
  PGA_GUARD(e < a.tab.numEntries, 1, {
    DevRule bad{};
    bad.op = 0xFF;
    return bad;
  });
  return block_smem().rules[e];
}
__device__ __forceinline__ DevParam param_at(const DeriveArgs& a, uint32_t k) {
  PGA_GUARD(k < a.numParams, 2, return DevParam{});
  return block_smem().params[k];
}
__device__ __forceinline__ int32_t succ_at(const DeriveArgs& a, uint32_t k) {
  PGA_GUARD(k < a.numSucc, 3, return -1);
  return block_smem().succ[k];
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ uint32_t warp_excl_scan(uint32_t v, uint32_t& total) {
  const unsigned lane = threadIdx.x & 31u;
  uint32_t x = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, d);
    if (lane >= (unsigned)d) x += y;
  }
  total = __shfl_sync(kFull, x, 31);
  return x - v;
}

// ------------------------------------------------------------- parameters

// A block value (PGA_PT_BLOCK): slot p.v0 of the parameter block of the
// shape's axiom.  The block build (PGA_INLINE_BLOCKS) reads it inline in
// param(), since it needs only the axiom index: two loads.
__device__ __forceinline__ float block_param(const DeriveArgs& a, const DevParam& p, const Shape& x) {
  const uint32_t slot = f2u(p.v0);
  if (a.blocks == nullptr || slot >= a.blockStride) {
    raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return 0.0f;
  }
  const uint32_t b = __ldg(&a.axioms[x.axiom].block);
  return __ldg(&a.blocks[(size_t)b * a.blockStride + slot]);
}

// Non-scalar parameters (random ranges, shape attributes, expressions, and
// block values outside the block build) take this out-of-line path so the
// common scalar case stays small.
__device__ __noinline__ float eval_param_slow(const DeriveArgs& a, DevParam p, Shape x) {
  switch (p.type) {
    case PGA_PT_SCALAR:
      return p.v0;
    case PGA_PT_RAND:
      return rand_range(x.seed, p.v0, p.v1);
    case PGA_PT_SHAPE_ATTR: {
      uint32_t i = f2u(p.v0);
      PGA_GUARD(x.axiom < a.numAxioms, 7, return 0.0f);
      float custom = (i == 16) ? __ldg(&a.axioms[x.axiom].custom) : 0.0f;
      return shape_attr(x, i, custom);
    }
    case PGA_PT_EXP:
      return eval_exp(a.tab.expPool + p.aux, x, __ldg(&a.axioms[x.axiom].custom), a.st);
    case PGA_PT_BLOCK:
      return block_param(a, p, x);
    default:
      return 0.0f;  // unknown types evaluate to 0 (Parameters.cuh:697-709 without invariant checks)
  }
}

__device__ __forceinline__ float param(const DeriveArgs& a, const DevRule& r, uint32_t k, const Shape& x) {
  const DevParam p = param_at(a, r.paramBase + k);
  if (p.type == PGA_PT_SCALAR) return p.v0;
#if PGA_INLINE_BLOCKS
  if (p.type == PGA_PT_BLOCK) return block_param(a, p, x);
#endif
  return eval_param_slow(a, p, x);
}

__device__ __forceinline__ bool axis_param(const DeriveArgs& a, const DevRule& r, const Shape& x, uint32_t& axis) {
  axis = f2u(param(a, r, 0, x));
  if (axis > 2) {
    raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return false;
  }
  return true;
}

__device__ __forceinline__ float seed_of(const DeriveArgs& a, float base, uint32_t modifier) {
  return a.useSeeds ? next_seed(base, modifier) : 0.0f;
}

// ------------------------------------------------- 1 -> 1 chain resolution

// Translate<X, Y, Z, Next>::execute (Translate.cuh:24-43): model * translate(v)
// in place.  Column 3 of the 4x4 product is ((R[i][0] v0 + R[i][1] v1) +
// R[i][2] v2) + t_i; with a signed-permutation R each row has one nonzero
// product, so it is one rounded add per row.
__device__ __forceinline__ void apply_translate(const DeriveArgs& a, const DevRule& r, Shape& x) {
  const float v0 = param(a, r, 0, x), v1 = param(a, r, 1, x), v2 = param(a, r, 2, x);
#if PGA_GENERAL_FRAMES
#pragma unroll
  for (uint32_t i = 0; i < 3; i++)
    x.t[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x.R[i * 3 + 0], v0), __fmul_rn(x.R[i * 3 + 1], v1)),
                                 __fmul_rn(x.R[i * 3 + 2], v2)),
                       x.t[i]);
#else
  translate_axis(x, x, 0, v0);
  translate_axis(x, x, 1, v1);
  translate_axis(x, x, 2, v2);
#endif
}

// Scale<X, Y, Z, Next>::execute (Scale.cuh:23-45): per axis
// ((v < 0) * size * v * -1) + ((v > 0) * v): a negative value scales the size,
// a positive one replaces it, zero makes it zero.
__device__ __forceinline__ float scaled_size(float s, float v) {
  return __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn((float)(v < 0.0f), s), v), -1.0f), __fmul_rn((float)(v > 0.0f), v));
}

__device__ __forceinline__ void apply_scale(const DeriveArgs& a, const DevRule& r, Shape& x) {
  const float v[3] = {param(a, r, 0, x), param(a, r, 1, x), param(a, r, 2, x)};
#pragma unroll
  for (int k = 0; k < 3; k++) x.s[k] = scaled_size(x.s[k], v[k]);
}

// RandomRule<DynParams>::execute (RandomRule.cuh:121-150): chance = frac(p0);
// the weights p1.. summed left to right; the first successor whose running
// share reaches the chance, or -1 when rounding leaves none (the shape is
// dropped).  The static form RandomRule<Chance, Pair<weight, next>...>
// (RandomRule.cuh:33-99, PGA_OP_RANDOM_RULE_STATIC) sums the weights right to
// left (p1 + (p2 + ...)), never picks a zero share and takes the last pair
// when no other is picked.
__device__ __forceinline__ int random_pick(const DeriveArgs& a, const DevRule& r, const Shape& x) {
  const float c0 = param(a, r, 0, x);
  const float chance = __fsub_rn(c0, floorf(c0));
  const bool dyn = r.op == PGA_OP_RANDOM_RULE;
  float sum = 0.0f;
  if (dyn) {
    for (uint32_t i = 1; i < r.nParams; i++) sum = __fadd_rn(sum, param(a, r, i, x));
  } else {
    sum = param(a, r, r.nParams - 1u, x);
    for (uint32_t i = r.nParams - 1u; i > 1; i--) sum = __fadd_rn(param(a, r, i - 1u, x), sum);
  }
  float acc = 0.0f;
  for (uint32_t i = 1; i < r.nParams; i++) {
    const float share = __fdiv_rn(param(a, r, i, x), sum);
    acc = __fadd_rn(acc, share);
    if (dyn ? (chance <= acc) : (i + 1 == r.nParams || (share != 0.0f && chance <= acc))) return (int)i - 1;
  }
  return -1;
}

// SwapSize<X, Y, Z, Next>::execute (SwapSize.cuh:20-38): size = (size[x],
// size[y], size[z]) for the axes the parameters name (truncated toward zero);
// an axis above 2 is an error (the reference would read past the vector).
__device__ __forceinline__ bool swap_size(const DeriveArgs& a, const DevRule& r, Shape& x) {
  const uint32_t ax = f2u(param(a, r, 0, x)), ay = f2u(param(a, r, 1, x)), az = f2u(param(a, r, 2, x));
  if (ax > 2 || ay > 2 || az > 2) {
    raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return false;
  }
  const float sx = pick3(x.s, ax), sy = pick3(x.s, ay), sz = pick3(x.s, az);
  x.s[0] = sx;
  x.s[1] = sy;
  x.s[2] = sz;
  return true;
}

// ------------------------------------------------------ phases and colliders

// A shape reaching a rule of a later phase waits there: it is written to the
// deferred buffer, which seeds the next phase's launch (the reference puts it
// in that phase's queue, CPUEvaluator.h:155-190).
__device__ __noinline__ void defer_shape(const DeriveArgs& a, const Shape& x) {
  const unsigned long long i = atomicAdd(a.phaseCounters + 1, 1ull);
  if (i >= a.deferCap) {
    raise_error(a.st, PGA_ERR_QUEUE_OVERFLOW, x.entry);
    return;
  }
#if PGA_GENERAL_FRAMES
  const float w = x.R[8];
  a.deferRotOut[2 * i] = make_float4(x.R[0], x.R[1], x.R[2], x.R[3]);
  a.deferRotOut[2 * i + 1] = make_float4(x.R[4], x.R[5], x.R[6], x.R[7]);
#else
  const float w = __uint_as_float(x.frame);
#endif
  float4* p = reinterpret_cast<float4*>(a.deferOut + i);
  p[0] = make_float4(x.t[0], x.t[1], x.t[2], x.s[0]);
  p[1] = make_float4(x.s[1], x.s[2], x.seed, w);
  reinterpret_cast<uint4*>(p)[2] = make_uint4((uint32_t)x.entry, x.axiom, (uint32_t)x.path, (uint32_t)(x.path >> 32));
  reinterpret_cast<uint4*>(p)[3] = make_uint4(0u, 0u, kAxiomLink | x.axiom, 0u);
}

// Collider<Tag, Next> (Collider.cuh:20-45) stores the shape with its tag
// (IntermediateSymbolsBufferAdapter.cuh:200-215): here as a record for the
// LBVH (model * scale, tag, shape bit, path) and as an oriented box of 5
// float4: rotation columns u0 u1 u2 (9) and centre (3), half extents (3), tag.
__device__ __noinline__ void store_collider(const DeriveArgs& a, const Shape& x, uint32_t tag) {
  const unsigned long long i = atomicAdd(a.phaseCounters, 1ull);
  if (i >= a.colCap) {
    raise_error(a.st, PGA_ERR_QUEUE_OVERFLOW, x.entry);
    return;
  }
  float m[3][3];
  frame_scaled(x, m);
  float4* rec = reinterpret_cast<float4*>(a.colRec + i);
  rec[0] = make_float4(m[0][0], m[0][1], m[0][2], x.t[0]);
  rec[1] = make_float4(m[1][0], m[1][1], m[1][2], x.t[1]);
  rec[2] = make_float4(m[2][0], m[2][1], m[2][2], x.t[2]);
  const uint32_t quad = x.kind == PGA_SHAPE_QUAD ? 0x80000000u : 0u;
  reinterpret_cast<uint4*>(rec)[3] = make_uint4((tag & 0xFFFFFFu) | quad, 0u, (uint32_t)x.path, (uint32_t)(x.path >> 32));
  float u[3][3];
#pragma unroll
  for (uint32_t j = 0; j < 3; j++)
#pragma unroll
    for (uint32_t r = 0; r < 3; r++) u[j][r] = frame_at(x, r, j);
  float4* sh = a.colShape + 5 * i;
  sh[0] = make_float4(u[0][0], u[0][1], u[0][2], u[1][0]);
  sh[1] = make_float4(u[1][1], u[1][2], u[2][0], u[2][1]);
  sh[2] = make_float4(u[2][2], x.t[0], x.t[1], x.t[2]);
  sh[3] = make_float4(__fmul_rn(x.s[0], 0.5f), __fmul_rn(x.s[1], 0.5f), __fmul_rn(x.s[2], 0.5f),
                      __uint_as_float(quad ? 1u : 0u));
  sh[4] = make_float4(__int_as_float((int)tag), 0.0f, 0.0f, 0.0f);
}

// An oriented box for the separating-axis test: centre, axes (model columns),
// half extents, and the half extents in the projected sums (a quad: z = 0).
struct Obb {
  float c[3], u[3][3], e[3], es[3];
};

__device__ __forceinline__ float dot3(const float* p, const float* q) {
  return __fadd_rn(__fadd_rn(__fmul_rn(p[0], q[0]), __fmul_rn(p[1], q[1])), __fmul_rn(p[2], q[2]));
}

// Collision::check for Box/Box, Box/Quad and Quad/Quad (Collision.cuh:35-738):
// the separating-axis test of Gottschalk, Lin and Manocha (OBBTree, 1996) over
// A's 3 face axes, B's 3 and the 9 edge cross products, separated when
// |T . L| > ra + rb, every sum left to right as the reference writes it.
__device__ __forceinline__ bool obb_overlap(const Obb& A, const Obb& B) {
  const float v[3] = {__fsub_rn(B.c[0], A.c[0]), __fsub_rn(B.c[1], A.c[1]), __fsub_rn(B.c[2], A.c[2])};
  float T[3], R[3][3], AR[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++) T[i] = dot3(v, A.u[i]);
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      R[i][j] = dot3(A.u[i], B.u[j]);
      AR[i][j] = fabsf(R[i][j]);
    }
  const float* a = A.es;
  const float* b = B.es;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float rb = __fadd_rn(__fadd_rn(__fmul_rn(b[0], AR[i][0]), __fmul_rn(b[1], AR[i][1])), __fmul_rn(b[2], AR[i][2]));
    if (fabsf(T[i]) > __fadd_rn(A.e[i], rb)) return false;
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float ra = __fadd_rn(__fadd_rn(__fmul_rn(a[0], AR[0][k]), __fmul_rn(a[1], AR[1][k])), __fmul_rn(a[2], AR[2][k]));
    const float t =
        fabsf(__fadd_rn(__fadd_rn(__fmul_rn(T[0], R[0][k]), __fmul_rn(T[1], R[1][k])), __fmul_rn(T[2], R[2][k])));
    if (t > __fadd_rn(ra, B.e[k])) return false;
  }
  // L = A_i x B_j: (p, q) the other axes of A, (r, s) those of B.
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const int p = i == 0 ? 1 : 0, q = i == 2 ? 1 : 2;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const int r = j == 0 ? 1 : 0, s = j == 2 ? 1 : 2;
      const float ra = __fadd_rn(__fmul_rn(a[p], AR[q][j]), __fmul_rn(a[q], AR[p][j]));
      const float rb = __fadd_rn(__fmul_rn(b[r], AR[i][s]), __fmul_rn(b[s], AR[i][r]));
      const float t = i == 1 ? fabsf(__fsub_rn(__fmul_rn(T[p], R[q][j]), __fmul_rn(T[q], R[p][j])))
                             : fabsf(__fsub_rn(__fmul_rn(T[q], R[p][j]), __fmul_rn(T[p], R[q][j])));
      if (t > __fadd_rn(ra, rb)) return false;
    }
  }
  return true;
}

__device__ __forceinline__ Obb collider_obb(const float4* sh, bool& quad, int& tag) {
  const float4 s0 = __ldg(sh), s1 = __ldg(sh + 1), s2 = __ldg(sh + 2), s3 = __ldg(sh + 3), s4 = __ldg(sh + 4);
  Obb o;
  o.u[0][0] = s0.x; o.u[0][1] = s0.y; o.u[0][2] = s0.z;
  o.u[1][0] = s0.w; o.u[1][1] = s1.x; o.u[1][2] = s1.y;
  o.u[2][0] = s1.z; o.u[2][1] = s1.w; o.u[2][2] = s2.x;
  o.c[0] = s2.y; o.c[1] = s2.z; o.c[2] = s2.w;
  o.e[0] = o.es[0] = s3.x;
  o.e[1] = o.es[1] = s3.y;
  o.e[2] = s3.z;
  quad = __float_as_uint(s3.w) != 0u;
  o.es[2] = quad ? 0.0f : s3.z;
  tag = __float_as_int(s4.x);
  return o;
}

// IfCollides<Tag, ...> (IfCollides.cuh:18-36, BVHTraversal.cuh:16-120): does a
// collider stored with the tag in an earlier phase overlap x?  The colliders'
// LBVH is traversed with a conservative box test (x's world box, widened by a
// relative 1e-5, against a node's box), so that no collider the exact test
// would report is pruned: the answer is "any collider with the tag overlaps",
// with Collision::check(stored, x) deciding at the leaves.
__device__ __noinline__ bool collides(const DeriveArgs& a, const Shape& x, uint32_t tag) {
  const uint32_t n = a.numColliders;
  if (n == 0) return false;
  Obb me;
  const bool quad = x.kind == PGA_SHAPE_QUAD;
#pragma unroll
  for (uint32_t j = 0; j < 3; j++)
#pragma unroll
    for (uint32_t r = 0; r < 3; r++) me.u[j][r] = frame_at(x, r, j);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    me.c[k] = x.t[k];
    me.e[k] = me.es[k] = __fmul_rn(x.s[k], 0.5f);
  }
  if (quad) me.es[2] = 0.0f;
  float lo[3], hi[3];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    float h = fabsf(me.u[0][r]) * me.e[0] + fabsf(me.u[1][r]) * me.e[1] + fabsf(me.u[2][r]) * me.e[2];
    h = h * 1.00001f + 1e-5f * (fabsf(me.c[r]) + 1.0f);
    lo[r] = me.c[r] - h;
    hi[r] = me.c[r] + h;
  }
  auto leaf_hits = [&](uint32_t leaf) -> bool {
    const uint32_t rec = __ldg(a.colLeaf + leaf);
    bool cq;
    int ctag;
    const Obb other = collider_obb(a.colShape + 5ull * rec, cq, ctag);
    if (ctag != (int)tag) return false;
    // Collision::check(Quad, Box) is check(Box, Quad) (Collision.cuh:734-737)
    return (cq && !quad) ? obb_overlap(me, other) : obb_overlap(other, me);
  };
  if (n == 1) return leaf_hits(0);
  int stack[64];
  int top = 0;
  stack[top++] = 0;
  while (top > 0) {
    const int node = stack[--top];
#pragma unroll
    for (int side = 1; side <= 2; side++) {
      const int child = __ldg(a.colNodes + 3 * node + side);
      if (child >= 0) {
        if (leaf_hits((uint32_t)child)) return true;
      } else {
        const float* bx = a.colAabbs + 6ll * (-child);
        const bool overlap = __ldg(bx) <= hi[0] && __ldg(bx + 3) >= lo[0] && __ldg(bx + 1) <= hi[1] &&
                             __ldg(bx + 4) >= lo[1] && __ldg(bx + 2) <= hi[2] && __ldg(bx + 5) >= lo[2];
        if (overlap) {
          if (top >= 64) {
            raise_error(a.st, PGA_ERR_DEPTH, x.entry);
            return false;
          }
          stack[top++] = -child;
        }
      }
    }
  }
  return false;
}

// Resolves a freshly created shape through IfSizeLess / Extrude / Translate /
// Scale / RandomRule rules (If.cuh:65-89, Extrude.cuh:29-56, Translate.cuh:24-43,
// Scale.cuh:23-45, RandomRule.cuh:121-150) until it reaches a Generate (terminal), a
// Discard, or a branching rule (queued).  The Translate / Scale / RandomRule
// steps are compiled in with AFF only: the persistent kernel has an
// instantiation without them for grammars that use none, which keeps their
// registers out of its expansion loops.
template <int AFF>
__device__ __forceinline__ int resolve(const DeriveArgs& a, Shape& x, uint32_t& tidx) {
  for (int step = 0; step < kMaxChain; step++) {
    if (x.entry < 0 || (uint32_t)x.entry >= a.tab.numEntries) {
      raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry);
      return kNone;
    }
    const DevRule r = rule_at(a, (uint32_t)x.entry);
    if (r.op == 0xFF || r.shape != x.kind) {
      raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry);
      return kNone;
    }
    if (AFF >= 2) {
      // phases and colliders: compiled in the instantiation for multi-phase tables only
      if ((uint32_t)(r.flags >> kRulePhaseShift) > a.phase) {
        defer_shape(a, x);
        return kNone;
      }
      if (r.op == PGA_OP_COLLIDER) {
        if (r.nParams < 1 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        const uint32_t tag = f2u(param(a, r, 0, x));
        if (tag > 0) store_collider(a, x, tag);
        x.entry = succ_at(a, r.succBase);
        continue;
      }
      if (r.op == PGA_OP_IF_COLLIDES) {
        if (r.nParams < 1 || r.nSucc < 2) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        const uint32_t branch = collides(a, x, f2u(param(a, r, 0, x)) & 0xFFu) ? 0u : 1u;
        const int32_t nxt = succ_at(a, r.succBase + branch);
        x.path = child_path(x.path, branch, nxt);
        x.entry = nxt;
        continue;
      }
    }
    switch (r.op) {
      case PGA_OP_IF_SIZE_LESS: {
        if (r.nParams < 2) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        uint32_t axis;
        if (!axis_param(a, r, x, axis)) return kNone;
        float size = param(a, r, 1, x);
        uint32_t branch = (pick3(x.s, axis) < size) ? 0u : 1u;
        if (branch >= r.nSucc) { raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry); return kNone; }
        int32_t nxt = succ_at(a, r.succBase + branch);
        x.path = child_path(x.path, branch, nxt);
        x.entry = nxt;
        continue;
      }
      case PGA_OP_EXTRUDE: {
        if (r.nParams < 2 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        float extent = param(a, r, 1, x);
        int32_t nxt = succ_at(a, r.succBase);
        // model * [x, z, -y] columns; size (sx, extent, sy).
        frame_set2(x, x, 1, 2, 0, 2, 1, 1);
        x.s[2] = x.s[1];
        x.s[1] = extent;
        x.seed = seed_of(a, x.seed, 0u);
        x.kind = PGA_SHAPE_BOX;
        x.path = child_path(x.path, 0u, nxt);
        x.entry = nxt;
        continue;
      }
      case PGA_OP_GENERATE: {
        if (r.flags & kRuleConstTerminal) {
          tidx = r.nChildren;
          return kTerm;
        }
        if (r.nParams < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        tidx = f2u(param(a, r, 0, x));
        if (tidx > 127u) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        return kTerm;
      }
      case PGA_OP_TRANSLATE: {
        if (!AFF || r.nParams < 3 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        apply_translate(a, r, x);
        x.entry = succ_at(a, r.succBase);
        continue;
      }
      case PGA_OP_SCALE: {
        if (!AFF || r.nParams < 3 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        apply_scale(a, r, x);
        x.entry = succ_at(a, r.succBase);
        continue;
      }
      case PGA_OP_RANDOM_RULE:
      case PGA_OP_RANDOM_RULE_STATIC: {
        if (!AFF || r.nParams < 2 || r.nSucc + 1 < r.nParams) {
          raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
          return kNone;
        }
        const int pick = random_pick(a, r, x);
        if (pick < 0) return kNone;
        const int32_t nxt = succ_at(a, r.succBase + (uint32_t)pick);
        x.path = child_path(x.path, (uint32_t)pick, nxt);
        x.entry = nxt;
        continue;
      }
      case PGA_OP_IF: {
        // If<Expression, True, False>::execute (If.cuh:22-49): a nonzero value
        // takes the first successor.
        if (!AFF || r.nParams < 1 || r.nSucc < 2) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        const uint32_t branch = (param(a, r, 0, x) != 0.0f) ? 0u : 1u;
        const int32_t nxt = succ_at(a, r.succBase + branch);
        x.path = child_path(x.path, branch, nxt);
        x.entry = nxt;
        continue;
      }
      case PGA_OP_SWAP_SIZE: {
        if (!AFF || r.nParams < 3 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        if (!swap_size(a, r, x)) return kNone;
        x.entry = succ_at(a, r.succBase);
        continue;
      }
#if PGA_GENERAL_FRAMES
      case PGA_OP_ROTATE: {
        // Rotate<X, Y, Z, Next>::execute (Rotate.cuh:24-41): model * rotateXYZ
        // of the scalar angles, whose matrix the engine built at creation
        // (its 9 entries in the expression pool at parameter 0's aux).
        if (!AFF || r.nParams < 3 || r.nSucc < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return kNone; }
        frame_rotate(x, a.tab.expPool + param_at(a, r.paramBase).aux);
        x.entry = succ_at(a, r.succBase);
        continue;
      }
#endif
      // (tables with Rotate run the general-frame kernels; in the frame-code
      // build a Rotate rule is queued and its expansion raises BAD_OPCODE)
      case PGA_OP_DISCARD:
        return kNone;
      default:
        return kNode;
    }
  }
  raise_error(a.st, PGA_ERR_DEPTH, x.entry);
  return kNone;
}

// ---------------------------------------------------- branching operators

// Per-thread state of one branching operator while its children are produced.
struct Expander {
  Shape base;       // the executing shape
  DevRule r;
  uint32_t axis;
  AxisRef axisRef;  // the split axis in the frame (Subdivide, Repeat)
  float offset;     // running offset along the axis
  float scale;
  uint32_t reps;
  float e2, startExt, endExt, halfMid;
  float prevSize, prevOff;  // Subdivide<DynParams>: the previous child, i.e. the symbol as updated in place
};

// Repeat<false, ...> set-up (Repeat.cuh:70-146).  Out of line (it is needed
// once per Repeat shape) and returned by value so that callers keep their
// state in registers.
struct RepeatSetup {
  uint32_t axis, reps;
  float e1, e2, e3;
  uint32_t flags;  // bit 0: arguments valid, bit 1: anchored to start
};

__device__ __noinline__ RepeatSetup repeat_setup(const DeriveArgs& a, DevRule r, Shape x, bool raise) {
  RepeatSetup R{0u, 0u, 0.0f, 0.0f, 0.0f, 0u};
  if (r.nParams < 3 || r.nSucc < 1) {
    if (raise) raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return R;
  }
  R.axis = f2u(param(a, r, 0, x));
  if (R.axis > 2) {
    if (raise) raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return R;
  }
  const uint32_t mode = f2u(param(a, r, 2, x));
  const float ext = param(a, r, 1, x);
  const float total = pick3(x.s, R.axis);
  const float extent = __fadd_rn(__fmul_rn(__fmul_rn((float)(ext < 0.0f), total), fabsf(ext)),
                                 __fmul_rn((float)(ext > 0.0f), ext));
  if (extent <= 0.0f || total < 0.0f) {
    if (raise) raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return R;
  }
  const float division = __fdiv_rn(total, extent);
  if (mode == 0u || mode == 1u) {
    const float rest = fmodf(total, extent);
    const bool exact = (rest == 0.0f);
    R.reps = f2u(ceilf(division));
    R.e1 = __fadd_rn(__fmul_rn((float)exact, extent), __fmul_rn((float)(!exact), rest));
    R.e2 = R.e3 = extent;
  } else if (mode == 2u) {
    R.reps = f2u(floorf(division));
    R.e1 = R.e2 = R.e3 = (R.reps > 0) ? __fdiv_rn(total, __uint2float_rn(R.reps)) : 0.0f;
  } else {
    if (raise) raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry);
    return R;
  }
  R.flags = 1u | (mode == 0u ? 2u : 0u);
  return R;
}

// Number of children a branching shape produces (decides how many work items
// it is queued as).  Errors are raised when the item is executed.
__device__ __forceinline__ uint32_t count_children(const DeriveArgs& a, const Shape& y) {
  const DevRule r = rule_at(a, (uint32_t)y.entry);
  switch (r.op) {
    case PGA_OP_SUBDIVIDE:
      return r.nParams >= 1 ? r.nParams - 1u : 1u;
    case PGA_OP_SUBDIVIDE_STATIC:
      return r.nChildren;
    case PGA_OP_COMPONENT_SPLIT:
      return 6u;
    case PGA_OP_REPLICATE:
      return r.nSucc > 0 ? r.nSucc : 1u;
    case PGA_OP_REPEAT: {
      const RepeatSetup R = repeat_setup(a, r, y, false);
      if (!(R.flags & 1u)) return 1u;
      return R.reps > 1 ? R.reps : 1u;
    }
    default:
      return 1u;  // raises BAD_OPCODE when executed
  }
}

// Subdivide set-up shared by the work-item expander and the in-place leaf
// expansion: axis, starting offset -size/2 and the scale of relative factors
// (size - sum of absolute) / sum of relative; returns the child count, 0 on error.
// Subdivide<DynParams>::execute (Subdivide.cuh:177-216) and the static form
// Subdivide<Axis, Pair<DynParam<k+1>, DCall<k>>...> (Subdivide.cuh:139-156).
__device__ __forceinline__ uint32_t subdivide_setup(const DeriveArgs& a, const DevRule& r, const Shape& x,
                                                    uint32_t& axis, float& offset, float& scale) {
  const bool dyn = r.op == PGA_OP_SUBDIVIDE;
  uint32_t n = dyn ? (r.nParams >= 1 ? r.nParams - 1u : 0u) : r.nChildren;
  if (r.nParams < n + 1 || r.nParams < 1) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return 0; }
  if (!axis_param(a, r, x, axis)) return 0;
  float total = pick3(x.s, axis);
  offset = __fmul_rn(total, -0.5f);
  float absSum = 0.0f, relSum = 0.0f;
  for (uint32_t i = 1; i <= n; i++) {
    float f = param(a, r, i, x);
    absSum = __fadd_rn(absSum, __fmul_rn((float)(f > 0.0f), f));
    relSum = __fadd_rn(relSum, __fmul_rn((float)(f < 0.0f), __fmul_rn(f, -1.0f)));
  }
  scale = (relSum == 0.0f) ? 0.0f : __fdiv_rn(__fsub_rn(total, absSum), relSum);
  if (dyn && scale < 0.0f) { raise_error(a.st, PGA_ERR_BAD_PARAM, x.entry); return 0; }
  return n;
}

// Operator set-up; returns the number of child slots (0 on error).  Replicate
// is compiled in with AFF only (see resolve).
template <int AFF = 1>
__device__ __forceinline__ uint32_t expander_init(const DeriveArgs& a, Expander& E) {
  const Shape& x = E.base;
  const DevRule& r = E.r;
  // Replicate<DynParams>::execute (Replicate.cuh:95-110): one child per successor.
  if (AFF && r.op == PGA_OP_REPLICATE) return r.nSucc;
  switch (r.op) {
    case PGA_OP_SUBDIVIDE:
    case PGA_OP_SUBDIVIDE_STATIC: {
      const uint32_t n = subdivide_setup(a, r, x, E.axis, E.offset, E.scale);
      if (n == 0) return 0;
      E.axisRef = axis_ref(x, E.axis);
      E.prevSize = 0.0f;
      E.prevOff = 0.0f;
      return n;
    }
    case PGA_OP_REPEAT: {
      const RepeatSetup R = repeat_setup(a, r, x, true);
      if (!(R.flags & 1u)) return 0;
      E.axis = R.axis;
      E.axisRef = axis_ref(x, R.axis);
      E.reps = R.reps;
      E.e2 = R.e2;
      const float e1 = R.e1, e3 = R.e3;
      const bool start = (R.flags & 2u) != 0;
      E.startExt = __fadd_rn(__fmul_rn((float)start, e1), __fmul_rn((float)(!start), e3));
      E.endExt = __fadd_rn(__fmul_rn((float)start, e3), __fmul_rn((float)(!start), e1));
      E.halfMid = __fmul_rn(E.e2, 0.5f);
      return E.reps > 1 ? E.reps : 1;
    }
    case PGA_OP_COMPONENT_SPLIT:
      // ComponentSplit<false, Top, Bottom, Sides>::execute (ComponentSplit.cuh:238-255).
      if (r.nSucc < 3) { raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry); return 0; }
      return 6;
    default:
      raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry);
      return 0;
  }
}

// Subdivide<DynParams> reads factor c+1 from the symbol as left by child c
// (Subdivide.cuh:220-235 update the symbol in place).
__device__ __forceinline__ float dyn_factor(const DeriveArgs& a, const Expander& E, uint32_t c) {
  const DevRule& r = E.r;
  if ((r.flags & kRulePure) || c == 0) return param(a, r, c + 1, E.base);
  Shape cur = E.base;
  put3(cur.s, E.axis, E.prevSize);
  translate_axis(cur, E.base, E.axis, E.prevOff);
  cur.seed = seed_of(a, E.base.seed, c - 1);
  cur.entry = (c - 1 < r.nSucc) ? succ_at(a, r.succBase + c - 1) : -1;
  return param(a, r, c + 1, cur);
}

__device__ __forceinline__ float subdivide_size(float f, float scale) {
  return __fadd_rn(__fmul_rn(__fmul_rn(__fmul_rn((float)(f < 0.0f), scale), f), -1.0f),
                   __fmul_rn((float)(f > 0.0f), f));
}

// Advances the running state past children [0, c0) without producing them.
__device__ __forceinline__ void expander_skip(const DeriveArgs& a, Expander& E, uint32_t c0) {
  const DevRule& r = E.r;
  if (c0 == 0) return;
  switch (r.op) {
    case PGA_OP_SUBDIVIDE:
      for (uint32_t c = 0; c < c0; c++) {
        float newSize = subdivide_size(dyn_factor(a, E, c), E.scale);
        E.prevOff = __fadd_rn(E.offset, __fmul_rn(newSize, 0.5f));
        E.prevSize = newSize;
        E.offset = __fadd_rn(E.offset, newSize);
      }
      return;
    case PGA_OP_SUBDIVIDE_STATIC:
      for (uint32_t c = 0; c < c0; c++) {
        float f = param(a, r, c + 1, E.base);
        if (f != 0.0f) E.offset = __fadd_rn(E.offset, subdivide_size(f, E.scale));
      }
      return;
    case PGA_OP_REPEAT: {
      float half = __fmul_rn(E.startExt, 0.5f);
      E.offset = __fadd_rn(__fadd_rn(__fmul_rn(pick3(E.base.s, E.axis), -0.5f), half), half);
      for (uint32_t c = 1; c < c0; c++) E.offset = __fadd_rn(__fadd_rn(E.offset, E.halfMid), E.halfMid);
      return;
    }
    default:
      return;
  }
}

// Produces child slot c (slots are produced in increasing order).  Returns
// false when the slot yields no child (a zero factor of a static Subdivide).
// PATH = false leaves y.path as the parent's (for the adjoint, which has no
// use for path hashes).
template <int AFF = 1, bool PATH = true>
__device__ __forceinline__ bool expander_child(const DeriveArgs& a, Expander& E, uint32_t c, Shape& y,
                                               uint32_t& ordinal) {
  const Shape& x = E.base;
  const DevRule& r = E.r;
  if (AFF && r.op == PGA_OP_REPLICATE) {
    // The symbol unchanged (seed included) but for its entry.
    const int32_t nxt = succ_at(a, r.succBase + c);
    y = x;
    y.entry = nxt;
    if (PATH) y.path = child_path(x.path, c, nxt);
    ordinal = c;
    return true;
  }
  switch (r.op) {
    case PGA_OP_SUBDIVIDE:
    case PGA_OP_SUBDIVIDE_STATIC: {
      const bool dyn = r.op == PGA_OP_SUBDIVIDE;
      float f = dyn ? dyn_factor(a, E, c) : param(a, r, c + 1, x);
      if (!dyn && f == 0.0f) return false;
      float newSize = subdivide_size(f, E.scale);
      float o = __fadd_rn(E.offset, __fmul_rn(newSize, 0.5f));
      if (c >= r.nSucc) { raise_error(a.st, PGA_ERR_BAD_OPCODE, x.entry); return false; }
      int32_t nxt = succ_at(a, r.succBase + c);
      y = x;
      put3(y.s, E.axis, newSize);
      translate_ref(y, x, E.axisRef, o);
      y.seed = seed_of(a, x.seed, c);
      y.entry = nxt;
      if (PATH) y.path = child_path(x.path, c, nxt);
      E.offset = __fadd_rn(E.offset, newSize);
      E.prevSize = newSize;
      E.prevOff = o;
      ordinal = c;
      return true;
    }
    case PGA_OP_REPEAT: {
      // Repeat.cuh:145-190: first piece, middle pieces, last piece.
      int32_t nxt = succ_at(a, r.succBase);
      float size, o;
      uint32_t mod;
      if (c == 0) {
        float half = __fmul_rn(E.startExt, 0.5f);
        o = __fadd_rn(__fmul_rn(pick3(x.s, E.axis), -0.5f), half);
        E.offset = __fadd_rn(o, half);
        size = E.startExt;
        mod = 1u;
      } else if (c + 1 < E.reps) {
        o = __fadd_rn(E.offset, E.halfMid);
        E.offset = __fadd_rn(o, E.halfMid);
        size = E.e2;
        mod = c + 1;
      } else {
        o = __fadd_rn(E.offset, __fmul_rn(E.endExt, 0.5f));
        size = E.endExt;
        mod = E.reps;
      }
      y = x;
      put3(y.s, E.axis, size);
      translate_ref(y, x, E.axisRef, o);
      y.seed = seed_of(a, x.seed, mod);
      y.entry = nxt;
      if (PATH) y.path = child_path(x.path, mod, nxt);
      ordinal = mod;
      return true;
    }
    case PGA_OP_COMPONENT_SPLIT: {
      // FaceSplitter<Box> (ComponentSplit.cuh:85-172): sides 0..3 (back, front,
      // left, right; seed modifier face + 2), then bottom (1), then top (0).
      y = x;
      y.kind = PGA_SHAPE_QUAD;
      float hx = __fmul_rn(x.s[0], 0.5f), hy = __fmul_rn(x.s[1], 0.5f), hz = __fmul_rn(x.s[2], 0.5f);
      uint32_t succ, mod;
      switch (c) {
        case 0:  // back: translate(0, 0, -hz) * diag(-1, 1, -1)
          translate_axis(y, x, 2, -hz);
          frame_set2(y, x, 0, 0, 1, 2, 2, 1);
          y.s[0] = x.s[0]; y.s[1] = x.s[1];
          succ = 2; mod = 2;
          break;
        case 1:  // front: translate(0, 0, hz)
          translate_axis(y, x, 2, hz);
          y.s[0] = x.s[0]; y.s[1] = x.s[1];
          succ = 2; mod = 3;
          break;
        case 2:  // left: translate(-hx, 0, 0) * columns [z, y, -x]
          translate_axis(y, x, 0, -hx);
          frame_set2(y, x, 0, 2, 0, 2, 0, 1);
          y.s[0] = x.s[2]; y.s[1] = x.s[1];
          succ = 2; mod = 4;
          break;
        case 3:  // right: translate(hx, 0, 0) * columns [-z, y, x]
          translate_axis(y, x, 0, hx);
          frame_set2(y, x, 0, 2, 1, 2, 0, 0);
          y.s[0] = x.s[2]; y.s[1] = x.s[1];
          succ = 2; mod = 5;
          break;
        case 4:  // bottom: translate(0, -hy, 0) * columns [x, z, -y]
          translate_axis(y, x, 1, -hy);
          frame_set2(y, x, 1, 2, 0, 2, 1, 1);
          y.s[0] = x.s[0]; y.s[1] = x.s[2];
          succ = 1; mod = 1;
          break;
        default:  // top: translate(0, hy, 0) * columns [x, -z, y]
          translate_axis(y, x, 1, hy);
          frame_set2(y, x, 1, 2, 1, 2, 1, 0);
          y.s[0] = x.s[0]; y.s[1] = x.s[2];
          succ = 0; mod = 0;
          break;
      }
      y.s[2] = 1.0f;
      int32_t nxt = succ_at(a, r.succBase + succ);
      y.seed = seed_of(a, x.seed, mod);
      y.entry = nxt;
      if (PATH) y.path = child_path(x.path, mod, nxt);
      ordinal = c;
      return true;
    }
    default:
      return false;
  }
}

// ------------------------------------------------------ records in memory

// A work item: the 64-byte Node; with general frames the rotation's entries
// 0..7 in two float4s of nodeRot at the same index and entry 8 in sf.w.
__device__ __forceinline__ void load_node(const DeriveArgs& ar, unsigned long long i, Shape& x, uint4& ext) {
  const float4* p = reinterpret_cast<const float4*>(ar.nodes + i);
  const float4 a = __ldcg(p + 0), b = __ldcg(p + 1);
  const uint4 m = __ldcg(reinterpret_cast<const uint4*>(p + 2));
  ext = __ldcg(reinterpret_cast<const uint4*>(p + 3));
  x.t[0] = a.x; x.t[1] = a.y; x.t[2] = a.z; x.s[0] = a.w;
  x.s[1] = b.x; x.s[2] = b.y; x.seed = b.z;
#if PGA_GENERAL_FRAMES
  const float4 r0 = __ldcg(ar.nodeRot + 2 * i), r1 = __ldcg(ar.nodeRot + 2 * i + 1);
  x.R[0] = r0.x; x.R[1] = r0.y; x.R[2] = r0.z; x.R[3] = r0.w;
  x.R[4] = r1.x; x.R[5] = r1.y; x.R[6] = r1.z; x.R[7] = r1.w;
  x.R[8] = b.w;
#else
  x.frame = __float_as_uint(b.w);
#endif
  x.entry = (int32_t)m.x;
  x.axiom = m.y;
  x.path = ((uint64_t)m.w << 32) | m.z;
}

__device__ __forceinline__ void store_node(const DeriveArgs& ar, unsigned long long i, const Shape& x, uint4 ext) {
  float4* p = reinterpret_cast<float4*>(ar.nodes + i);
#if PGA_GENERAL_FRAMES
  const float w = x.R[8];
  __stcg(ar.nodeRot + 2 * i, make_float4(x.R[0], x.R[1], x.R[2], x.R[3]));
  __stcg(ar.nodeRot + 2 * i + 1, make_float4(x.R[4], x.R[5], x.R[6], x.R[7]));
#else
  const float w = __uint_as_float(x.frame);
#endif
  __stcg(p + 0, make_float4(x.t[0], x.t[1], x.t[2], x.s[0]));
  __stcg(p + 1, make_float4(x.s[1], x.s[2], x.seed, w));
  __stcg(reinterpret_cast<uint4*>(p + 2),
         make_uint4((uint32_t)x.entry, x.axiom, (uint32_t)x.path, (uint32_t)(x.path >> 32)));
  __stcg(reinterpret_cast<uint4*>(p + 3), ext);
}

// GenerationFunction<.., 1>::perShape (GenerationFunctions.cuh:158-188):
// model4 * scale(size) and the custom attribute, as four 16-byte stores.
__device__ __forceinline__ void store_terminal(const DeriveArgs& a, PgaTerminal* dst, unsigned long long slot,
                                               const Shape& x, uint32_t tidx) {
  float4* p = reinterpret_cast<float4*>(dst + slot);
  PGA_GUARD(x.axiom < a.numAxioms, 8, return);
  float custom = __ldg(&a.axioms[x.axiom].custom);
  uint32_t rule = ((uint32_t)x.entry & 0xFFFFFFu) | (tidx << 24) | (x.kind == PGA_SHAPE_QUAD ? 0x80000000u : 0u);
  float m[3][3];
  frame_scaled(x, m);
  __stcs(p + 0, make_float4(m[0][0], m[0][1], m[0][2], x.t[0]));
  __stcs(p + 1, make_float4(m[1][0], m[1][1], m[1][2], x.t[1]));
  __stcs(p + 2, make_float4(m[2][0], m[2][1], m[2][2], x.t[2]));
  __stcs(reinterpret_cast<uint4*>(p + 3),
         make_uint4(rule, __float_as_uint(custom), (uint32_t)x.path, (uint32_t)(x.path >> 32)));
}

// Output of the persistent engine: every warp owns a page of kTermPage
// terminal slots and a page of kNodePage item slots at a time, taken with one
// atomic on a page counter; a round's lanes write consecutive slots of the
// warp's page.  This cuts the same-address atomics on the output counters by
// the page size.  Item pages are closed at every level end (their unused slots
// marked empty); the warps' last terminal pages leave holes that a compaction
// at the end of the launch fills, so the output is dense.
constexpr uint32_t kTermPage = 256;
constexpr uint32_t kNodePage = 64;
constexpr uint32_t kEmptyItem = 0xFFFFFFFFu;

struct WarpOut {
  unsigned long long tPage, nPage;
  uint32_t tFill, nFill;  // slots used in the current page (page size when there is none)
  uint32_t sub;           // children per queued work item for the level being expanded
};

__device__ __forceinline__ void warpout_init(const DeriveArgs& a, WarpOut& w) {
  w.tPage = w.nPage = ~0ull;
  w.tFill = kTermPage;
  w.nFill = kNodePage;
  w.sub = a.subItem;
}

// A level with fewer items than the grid has threads leaves most lanes idle:
// its children are queued in finer work items (more parallelism next level).
__device__ __forceinline__ void warpout_level(const DeriveArgs& a, WarpOut& w, unsigned long long items) {
  w.sub = items < (unsigned long long)gridDim.x * kThreads ? a.narrowSubItem : a.subItem;
}

// Reserves cnt consecutive slots (warp-uniform) of a paged stream: a lane's
// rank r < cnt maps to first + r (r < rem) or next + (r - rem).
struct Span {
  unsigned long long first, next;
  uint32_t rem;
};

__device__ __forceinline__ Span page_reserve(unsigned long long* counter, uint32_t pageSize,
                                             unsigned long long& page, uint32_t& fill, uint32_t cnt) {
  Span sp;
  sp.rem = min(pageSize - fill, cnt);
  sp.first = page * pageSize + fill;
  sp.next = 0;
  if (cnt > sp.rem) {
    const uint32_t need = cnt - sp.rem;
    const uint32_t np = (need + pageSize - 1) / pageSize;
    unsigned long long p0 = 0;
    if ((threadIdx.x & 31u) == 0) p0 = atomicAdd(counter, (unsigned long long)np);
    p0 = __shfl_sync(kFull, p0, 0);
    sp.next = p0 * pageSize;
    page = p0 + np - 1;
    fill = need - (np - 1) * pageSize;
  } else {
    fill += cnt;
  }
  return sp;
}

__device__ __forceinline__ unsigned long long span_slot(const Span& sp, uint32_t r) {
  return r < sp.rem ? sp.first + r : sp.next + (r - sp.rem);
}

// Terminal slot s: the caller's buffer below `cap`, the engine's tail buffer above.
__device__ __forceinline__ void write_terminal(const DeriveArgs& a, unsigned long long s, const Shape& y, uint32_t tidx,
                                               uint32_t link, uint32_t ordinal) {
  if (s < a.cap) {
    store_terminal(a, a.out, s, y, tidx);
    if (a.termLinks != nullptr && s < a.termLinkCap) a.termLinks[s] = make_uint2(link, ordinal);
  } else if (s - a.cap < a.tailCap) {
    store_terminal(a, a.tail, s - a.cap, y, tidx);
    if (a.tailLinks != nullptr) a.tailLinks[s - a.cap] = make_uint2(link, ordinal);
  }
}

// Warp-collective emission of one shape per lane (kind kNone / kTerm / kNode,
// a branching shape with nChild children queued as ceil(nChild / subItem)
// work items); each round writes a contiguous run in lane order.  PAGED: warp
// pages; otherwise (the plain form) one atomic per round and kind.
template <bool PAGED>
__device__ __forceinline__ void emit_round(const DeriveArgs& a, WarpOut& w, int kind, const Shape& y, uint32_t tidx,
                                           uint32_t nChild, uint32_t link, uint32_t ordinal) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned tm = __ballot_sync(kFull, kind == kTerm);
  if (tm) {
    const uint32_t cnt = __popc(tm), rank = __popc(tm & lanemask_lt());
    unsigned long long slot;
    if (PAGED) {
      const Span sp = page_reserve(&a.st->termPages, kTermPage, w.tPage, w.tFill, cnt);
      slot = span_slot(sp, rank);
    } else {
      unsigned long long base = 0;
      const unsigned leader = __ffs(tm) - 1;
      if (lane == leader) base = atomicAdd(&a.st->termCount, (unsigned long long)cnt);
      slot = __shfl_sync(kFull, base, leader) + rank;
    }
    if (kind == kTerm) write_terminal(a, slot, y, tidx, link, ordinal);
  }
  const unsigned nm = __ballot_sync(kFull, kind == kNode);
  if (nm) {
    const uint32_t S = w.sub;
    const uint32_t m = (kind == kNode) ? (nChild + S - 1) / S : 0u;
    uint32_t total;
    const uint32_t pre = warp_excl_scan(m, total);
    Span sp;
    if (PAGED) {
      sp = page_reserve(&a.st->nodePages, kNodePage, w.nPage, w.nFill, total);
    } else {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&a.st->nodeNext, (unsigned long long)total);
      sp.first = __shfl_sync(kFull, base, 0);
      sp.rem = total;
      sp.next = 0;
    }
    for (uint32_t j = 0; j < m; j++) {
      const unsigned long long slot = span_slot(sp, pre + j);
      if (slot >= a.nodeCap) {
        raise_error(a.st, PGA_ERR_QUEUE_OVERFLOW, -1);
        break;
      }
      store_node(a, slot, y, make_uint4(j * S, min((j + 1) * S, nChild), link, ordinal));
    }
  }
}

// Marks the unused slots of the warp's item page empty and gives the page up
// (at the end of a level: the next level's items are exactly the pages handed
// out during this one).
__device__ __forceinline__ void close_node_page(const DeriveArgs& a, WarpOut& w) {
  const unsigned lane = threadIdx.x & 31u;
  if (w.nPage != ~0ull) {
    for (uint32_t k = w.nFill + lane; k < kNodePage; k += 32) {
      const unsigned long long slot = w.nPage * kNodePage + k;
      if (slot < a.nodeCap)
        __stcg(reinterpret_cast<uint4*>(a.nodes + slot) + 3, make_uint4(kEmptyItem, 0u, 0u, 0u));
    }
  }
  w.nPage = ~0ull;
  w.nFill = kNodePage;
}

// Emits a new child per lane (kind from resolve); a branching child is queued
// as ceil(children / subItem) work items.
template <bool PAGED>
__device__ __forceinline__ void emit_child(const DeriveArgs& a, WarpOut& w, int kind, const Shape& y, uint32_t tidx,
                                           uint32_t link, uint32_t ordinal) {
  const uint32_t nY = (kind == kNode) ? count_children(a, y) : 0u;
  emit_round<PAGED>(a, w, kind, y, tidx, nY, link, ordinal);
}

// In-place expansion of leaf children.  A leaf rule (flagged at engine
// creation) is a Subdivide whose factors do not read the shape and whose
// successors are all Generates with a constant terminal index or Discards, so
// its children are known to end right away.  The lane that created such a
// child emits the child's terminals itself instead of queuing a work item for
// the next level: the same arithmetic (subdivide_setup, subdivide_size, the
// running offset, translate_ref, child seeds and path hashes) in a loop that
// holds only the Subdivide's state.
template <bool PAGED>
__device__ __forceinline__ void emit_leaf(const DeriveArgs& a, WarpOut& w, bool leaf, const Shape& y, uint32_t link) {
  DevRule r;
  uint32_t n = 0, axis = 0;
  AxisRef ref{};
  float offset = 0.0f, scale = 0.0f;
  if (leaf) {
    r = rule_at(a, (uint32_t)y.entry);
    n = subdivide_setup(a, r, y, axis, offset, scale);
    ref = axis_ref(y, axis);
  }
  for (uint32_t g = 0; __any_sync(kFull, g < n); g++) {
    int kind = kNone;
    Shape z;
    uint32_t tidx = 0;
    if (g < n) {
      const float f = param(a, r, g + 1, y);
      if (r.op == PGA_OP_SUBDIVIDE || f != 0.0f) {
        const float newSize = subdivide_size(f, scale);
        const float o = __fadd_rn(offset, __fmul_rn(newSize, 0.5f));
        offset = __fadd_rn(offset, newSize);
        const int32_t nxt = succ_at(a, r.succBase + g);
        const DevRule sr = rule_at(a, (uint32_t)nxt);
        if (sr.op == PGA_OP_GENERATE) {
          z = y;
          put3(z.s, axis, newSize);
          translate_ref(z, y, ref, o);
          z.seed = seed_of(a, y.seed, g);
          z.entry = nxt;
          z.path = child_path(y.path, g, nxt);
          tidx = sr.nChildren;
          kind = kTerm;
        }
      }
    }
    emit_round<PAGED>(a, w, kind, z, tidx, 0u, link, g);
  }
}

// Emits a lane's new child: with LEAF, leaf children in place and the others
// as terminals or work items; without, everything as terminals or work items.
// LEAF is a separate instantiation of the persistent kernel, launched only for
// grammars that have leaf rules, so the others do not carry its registers.
template <bool PAGED, bool LEAF>
__device__ __forceinline__ void emit_new(const DeriveArgs& a, WarpOut& w, int kind, const Shape& y, uint32_t tidx,
                                         uint32_t link, uint32_t ordinal) {
  if (!LEAF) {
    emit_child<PAGED>(a, w, kind, y, tidx, link, ordinal);
    return;
  }
  bool leaf = false;
  if (kind == kNode) leaf = (rule_at(a, (uint32_t)y.entry).flags & kRuleLeaf) != 0;
  emit_child<PAGED>(a, w, leaf ? (int)kNone : kind, y, tidx, link, ordinal);
  if (__any_sync(kFull, leaf)) emit_leaf<PAGED>(a, w, leaf, y, link);
}

// Root shape of axiom i, as Grid::...::generateAxiom builds it (Grid.cuh:199-204).
__device__ __forceinline__ void axiom_shape(const DeriveArgs& a, uint32_t i, Shape& x) {
  const PgaAxiom* ax = a.axioms + i;
  frame_identity(x);
  x.t[0] = __ldg(&ax->position[0]); x.t[1] = __ldg(&ax->position[1]); x.t[2] = __ldg(&ax->position[2]);
  x.s[0] = __ldg(&ax->size[0]); x.s[1] = __ldg(&ax->size[1]); x.s[2] = __ldg(&ax->size[2]);
  x.seed = __ldg(&ax->seed);
  x.entry = (int32_t)__ldg(&ax->entry);
  x.kind = __ldg(&ax->shape);
  x.axiom = i;
  x.path = mix64((uint64_t)i + 0x9E3779B97F4A7C15ULL);
}

// Expands the work items first + 32 k + lane (k < K, item < hi) of one warp.
template <bool PAGED, bool LEAF, int AFF>
__device__ __forceinline__ void warp_items(const DeriveArgs& a, WarpOut& w, unsigned long long first,
                                           unsigned long long hi, uint32_t K) {
  const unsigned lane = threadIdx.x & 31u;
  for (uint32_t k = 0; k < K; k++) {
    const unsigned long long item = first + 32ull * k + lane;
    if (!__any_sync(kFull, item < hi)) break;
    Expander E;
    uint32_t c0 = 0, n = 0;
    bool valid = item < hi;
    PGA_GUARD(!valid || item < a.nodeCap, 10, valid = false);
    if (valid) {
      uint4 ext;
      load_node(a, item, E.base, ext);
      const int32_t e = E.base.entry;
      if (ext.x == kEmptyItem) {
        // an unused slot of an item page
      } else if (e < 0 || (uint32_t)e >= a.tab.numEntries) {
        raise_error(a.st, PGA_ERR_BAD_OPCODE, e);
      } else {
        E.r = rule_at(a, (uint32_t)e);
        E.base.kind = E.r.shape;
        const uint32_t all = expander_init<AFF>(a, E);
        const uint32_t c1 = min(ext.y, all);
        c0 = ext.x;
        if (c0 < c1) {
          expander_skip(a, E, c0);
          n = c1 - c0;
        }
      }
    }
    for (uint32_t c = 0; __any_sync(kFull, c < n); c++) {
      int kind = kNone;
      Shape y;
      uint32_t tidx = 0, ordinal = 0;
      if (c < n && expander_child<AFF>(a, E, c0 + c, y, ordinal)) kind = resolve<AFF>(a, y, tidx);
      emit_new<PAGED, LEAF>(a, w, kind, y, tidx, (uint32_t)item, ordinal);
    }
  }
}

// Seeds the axioms [first, first + count) with a warp-uniform grid-stride loop
// (the i-th seeded is axiomOrder[i] when an order is given).
template <bool PAGED, bool LEAF, int AFF>
__device__ void seed_axioms(const DeriveArgs& a, WarpOut& w, uint32_t first, uint32_t count) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long warpId = ((unsigned long long)blockIdx.x * kThreads + threadIdx.x) >> 5;
  const unsigned long long numWarps = ((unsigned long long)gridDim.x * kThreads) >> 5;
  const unsigned long long end = (unsigned long long)first + count;
  for (unsigned long long b = first + warpId * 32ull; b < end; b += numWarps * 32ull) {
    const unsigned long long i = b + lane;
    int kind = kNone;
    Shape y;
    uint32_t tidx = 0, ax = (uint32_t)i;
    if (i < end) {
      if (a.axiomOrder != nullptr) ax = __ldg(a.axiomOrder + i);
      axiom_shape(a, ax, y);
      kind = resolve<AFF>(a, y, tidx);
    }
    emit_new<PAGED, LEAF>(a, w, kind, y, tidx, kAxiomLink | ax, 0u);
  }
}

// Seeds the shapes deferred to this phase (multi-phase derivation): each is
// loaded as it was stored and resolved from the rule it was waiting at.
template <bool PAGED, bool LEAF, int AFF>
__device__ void seed_deferred(const DeriveArgs& a, WarpOut& w) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned long long warpId = ((unsigned long long)blockIdx.x * kThreads + threadIdx.x) >> 5;
  const unsigned long long numWarps = ((unsigned long long)gridDim.x * kThreads) >> 5;
  const unsigned long long end = a.numDeferIn;
  for (unsigned long long b = warpId * 32ull; b < end; b += numWarps * 32ull) {
    const unsigned long long i = b + lane;
    int kind = kNone;
    Shape y;
    uint32_t tidx = 0;
    if (i < end) {
      const float4* p = reinterpret_cast<const float4*>(a.deferIn + i);
      const float4 p0 = __ldcg(p), p1 = __ldcg(p + 1);
      const uint4 m = __ldcg(reinterpret_cast<const uint4*>(p + 2));
      y.t[0] = p0.x; y.t[1] = p0.y; y.t[2] = p0.z; y.s[0] = p0.w;
      y.s[1] = p1.x; y.s[2] = p1.y; y.seed = p1.z;
#if PGA_GENERAL_FRAMES
      const float4 r0 = __ldcg(a.deferRotIn + 2 * i), r1 = __ldcg(a.deferRotIn + 2 * i + 1);
      y.R[0] = r0.x; y.R[1] = r0.y; y.R[2] = r0.z; y.R[3] = r0.w;
      y.R[4] = r1.x; y.R[5] = r1.y; y.R[6] = r1.z; y.R[7] = r1.w;
      y.R[8] = p1.w;
#else
      y.frame = __float_as_uint(p1.w);
#endif
      y.entry = (int32_t)m.x;
      y.axiom = m.y;
      y.path = ((uint64_t)m.w << 32) | m.z;
      y.kind = ((uint32_t)y.entry < a.tab.numEntries) ? rule_at(a, (uint32_t)y.entry).shape : 0u;
      kind = resolve<AFF>(a, y, tidx);
    }
    emit_new<PAGED, LEAF>(a, w, kind, y, tidx, kAxiomLink | y.axiom, 0u);
  }
}

// The share of a wide level the dynamic instantiation hands out from the
// level's counter: 1 / this.
#ifndef PGA_DERIVE_DYNAMIC_SHARE
#define PGA_DERIVE_DYNAMIC_SHARE 4
#endif

// All items of one level [lo, hi): warp chunks of 32 K items in a static
// grid-stride order (no shared work counter).  DYN (PGA_FLAG_DYNAMIC_CHUNKS; a
// separate instantiation, so that the static one keeps its register
// allocation): on a level of at least four rounds of chunks the static order
// covers whole rounds up to the last quarter of the level (at least two
// rounds of chunks are left); warps then take the rest one chunk at a time
// from the level's cursor, which the level snapshot set to lo.
template <bool PAGED, bool LEAF, int AFF, bool DYN = false>
__device__ __forceinline__ void expand_level(const DeriveArgs& a, WarpOut& w, unsigned long long lo,
                                             unsigned long long hi, uint32_t K) {
  const unsigned long long warpId = ((unsigned long long)blockIdx.x * kThreads + threadIdx.x) >> 5;
  const unsigned long long numWarps = ((unsigned long long)gridDim.x * kThreads) >> 5;
  if constexpr (!DYN) {
    for (unsigned long long b = lo + warpId * 32ull * K; b < hi; b += numWarps * 32ull * K)
      warp_items<PAGED, LEAF, AFF>(a, w, b, hi, K);
  } else {
    const unsigned long long chunk = 32ull * K, stride = numWarps * chunk;
    unsigned long long dynLo = hi;  // items from dynLo on come from the cursor
    if (hi - lo >= 4 * stride) {
      const unsigned long long n = hi - lo, rest = max(n / PGA_DERIVE_DYNAMIC_SHARE, 2 * stride);
      dynLo = lo + ((n - rest) / stride) * stride;
    }
    // one call site of warp_items for both orders (a second inlined copy costs
    // the kernel its register allocation)
    for (unsigned long long b = lo + warpId * chunk;; b += stride) {
      if (b >= dynLo) {
        if (dynLo >= hi) break;
        unsigned long long c = 0;
        if ((threadIdx.x & 31u) == 0) c = atomicAdd(&a.st->cursor, chunk);
        b = dynLo + (__shfl_sync(kFull, c, 0) - lo);  // the loop step never lands below dynLo again
        if (b >= hi) break;
      }
      warp_items<PAGED, LEAF, AFF>(a, w, b, hi, K);
    }
  }
}

// Copies the rule table into shared memory when it fits (decided at engine
// creation, which sized the dynamic shared memory for it) and fixes the block's
// table pointers.
__device__ __forceinline__ void setup_block(const DeriveArgs& a, Smem& sm) {
  uint32_t dynBytes;
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dynBytes));
  const size_t tableBytes = (size_t)a.tab.numEntries * sizeof(DevRule) + (size_t)a.numParams * sizeof(DevParam) +
                            (size_t)a.numSucc * sizeof(int32_t);
  if (a.tableInSmem && sizeof(Smem) + tableBytes <= dynBytes) {
    DevRule* rules = reinterpret_cast<DevRule*>(smem_raw + sizeof(Smem));
    DevParam* params = reinterpret_cast<DevParam*>(rules + a.tab.numEntries);
    int32_t* succ = reinterpret_cast<int32_t*>(params + a.numParams);
    for (uint32_t i = threadIdx.x; i < a.tab.numEntries; i += kThreads) rules[i] = a.tab.rules[i];
    for (uint32_t i = threadIdx.x; i < a.numParams; i += kThreads) params[i] = a.tab.params[i];
    for (uint32_t i = threadIdx.x; i < a.numSucc; i += kThreads) succ[i] = a.tab.succ[i];
    if (threadIdx.x == 0) {
      sm.rules = rules;
      sm.params = params;
      sm.succ = succ;
    }
  } else if (threadIdx.x == 0) {
    sm.rules = a.tab.rules;
    sm.params = a.tab.params;
    sm.succ = a.tab.succ;
  }
  __syncthreads();
}

// ---------------------------------------------------- bounded grid barrier

// Thread 0 of every block arrives; the last arriver runs `leader()` and
// releases the others.  Waits are bounded by spinLimit; a timeout raises
// PGA_ERR_TIMEOUT and makes the caller leave the kernel.
template <typename Leader>
__device__ bool grid_barrier(const DeriveArgs& a, Leader leader) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    DevState* st = a.st;
    volatile uint32_t* gen = &st->barrierGen;
    uint32_t g = *gen;
    __threadfence();
    uint32_t prev = atomicAdd(&st->barrierArrive, 1u);
    if (prev == gridDim.x - 1) {
      atomicExch(&st->barrierArrive, 0u);
      leader();
      __threadfence();
      atomicAdd(&st->barrierGen, 1u);
    } else {
      uint32_t spins = 0;
      while (*gen == g) {
        if (++spins > a.spinLimit) {
          raise_error(st, PGA_ERR_TIMEOUT, -1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

__device__ __forceinline__ void level_snapshot(const DeriveArgs& a, uint32_t level) {
  DevState* st = a.st;
  volatile DevState* vs = st;
  unsigned long long lo = vs->levelHi;
  unsigned long long hi = atomicAdd(&st->nodePages, 0ull) * kNodePage;
  if (hi > a.nodeCap) hi = a.nodeCap;
  vs->nodeNext = hi;
  vs->levelLo = lo;
  vs->levelHi = hi;
  vs->cursor = lo;
  if (level + 1 <= a.maxLevels) {
    a.levelStart[level + 1] = hi;
    unsigned long long now;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
    a.levelClock[level] = now;
  }
  unsigned long long sz = hi - lo;
  if (sz > vs->maxLevelNodes) vs->maxLevelNodes = sz;
  bool more = hi > lo;
  if (more && level >= a.maxLevels) {
    raise_error(st, PGA_ERR_DEPTH, (int)level);
    more = false;
  }
  vs->levels = level;
  vs->stop = (!more || vs->status != 0) ? 1u : 0u;
}

// Exclusive prefix sum of x[0, n) in place (shared memory, whole block);
// x[n] receives the total.  Every thread takes a contiguous run.
__device__ void block_exclusive_scan(uint32_t* x, uint32_t n) {
  __shared__ uint32_t warpSum[kWarps];
  const unsigned lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
  const uint32_t per = (n + kThreads - 1) / kThreads;
  const uint32_t b = min(n, threadIdx.x * per), e = min(n, b + per);
  uint32_t sum = 0;
  for (uint32_t i = b; i < e; i++) sum += x[i];
  uint32_t total;
  const uint32_t pre = warp_excl_scan(sum, total);
  if (lane == 0) warpSum[wid] = total;
  __syncthreads();
  uint32_t off = 0, all = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) {
    off += (k < (int)wid) ? warpSum[k] : 0u;
    all += warpSum[k];
  }
  uint32_t run = off + pre;
  for (uint32_t i = b; i < e; i++) {
    const uint32_t v = x[i];
    x[i] = run;
    run += v;
  }
  if (threadIdx.x == 0) x[n] = all;
  __syncthreads();
}

// Shared-memory bytes the compaction needs for W warps.
__host__ __device__ constexpr size_t compact_smem_bytes(uint32_t W) {
  return ((sizeof(Smem) + 15) & ~size_t(15)) + 8ull * W + 4ull * (W + 1) + 4ull * (W + 2);
}

// Compaction of the terminal output after the last level.  Every warp's last
// terminal page may be partly filled, so with G pages handed out and `holes`
// unused slots in them, N = G * kTermPage - holes terminals exist and some lie
// at positions >= N.  Holes below N and filled slots at or above N are equally
// many; the k-th hole (warps in index order) receives the k-th such record
// (positions in increasing order).  Only the pages from the one holding N to
// the last can hold records >= N: fewer than W + 1 pages, all full except the
// partial pages among them.  After one grid barrier every block rebuilds both
// enumerations in shared memory from the W published partial pages (no sort,
// no further barrier) and moves its share of the records.
__device__ void compact_terminals(const DeriveArgs& a, WarpOut& w) {
  const unsigned lane = threadIdx.x & 31u;
  const uint32_t W = a.numWarps;
  const unsigned long long gw = ((unsigned long long)blockIdx.x * kThreads + threadIdx.x) >> 5;
  unsigned long long* part = a.scratch;  // W entries: page << 9 | fill, or ~0
  DevState* st = a.st;
  unsigned long long mine = ~0ull;
  if (w.tPage != ~0ull && w.tFill < kTermPage) mine = (w.tPage << 9) | w.tFill;
  if (lane == 0 && gw < W) part[gw] = mine;
  if (!grid_barrier(a, [] {})) return;
  uint32_t dynBytes;  // the same in every thread of the launch
  asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dynBytes));
  if (dynBytes < compact_smem_bytes(W)) {
    if (threadIdx.x == 0) raise_error(st, PGA_ERR_INTERNAL, 11);
    return;
  }
  unsigned long long* ps = reinterpret_cast<unsigned long long*>(smem_raw + ((sizeof(Smem) + 15) & ~size_t(15)));
  uint32_t* hPre = reinterpret_cast<uint32_t*>(ps + W);  // W + 1: holes below N per warp, then prefix
  uint32_t* sPre = hPre + W + 1;                        // W + 2: records >= N per page, then prefix
  __shared__ unsigned long long blockHoles[kWarps];
  unsigned long long holes = 0;
  for (uint32_t i = threadIdx.x; i < W; i += kThreads) {
    const unsigned long long e = __ldcg(&part[i]);
    ps[i] = e;
    if (e != ~0ull) holes += kTermPage - (e & 511ull);
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) holes += __shfl_xor_sync(kFull, holes, d);
  if (lane == 0) blockHoles[threadIdx.x >> 5] = holes;
  __syncthreads();
  holes = 0;
#pragma unroll
  for (int k = 0; k < kWarps; k++) holes += blockHoles[k];
  // One thread decides for the block, so that every thread takes the same path
  // through the block-wide steps below.
  __shared__ unsigned long long blockPages;
  __shared__ int blockGo;
  if (threadIdx.x == 0) {
    volatile DevState* vs = st;
    const unsigned long long G = vs->termPages;
    const unsigned long long N = G * kTermPage - holes;
    if (blockIdx.x == 0) vs->termCount = N;
    int go = (vs->status == 0 && N <= a.cap && holes != 0) ? 1 : 0;
    // G * kTermPage - N = holes < W * kTermPage, so at most W + 1 pages hold records >= N.
    if (go && (G <= N / kTermPage || G - N / kTermPage > W + 1)) {
      raise_error(st, PGA_ERR_INTERNAL, 11);
      go = 0;
    }
    blockPages = G;
    blockGo = go;
  }
  __syncthreads();
  if (!blockGo) return;
  const unsigned long long G = blockPages;
  const unsigned long long N = G * kTermPage - holes;
  const unsigned long long qN = N / kTermPage;
  const uint32_t P = (uint32_t)(G - qN);  // pages qN .. G-1
  for (uint32_t q = threadIdx.x; q < P; q += kThreads) sPre[q] = kTermPage;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < W; i += kThreads) {
    const unsigned long long e = ps[i];
    uint32_t h = 0;
    if (e != ~0ull) {
      const unsigned long long page = e >> 9, start = page * kTermPage + (e & 511ull);
      if (page >= qN) sPre[page - qN] = (uint32_t)(e & 511ull);
      if (start < N) h = (uint32_t)(min((page + 1) * kTermPage, N) - start);
    }
    hPre[i] = h;
  }
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < P; q += kThreads) {
    const unsigned long long base = (qN + q) * kTermPage, lo = max(base, N), end = base + sPre[q];
    sPre[q] = end > lo ? (uint32_t)(end - lo) : 0u;
  }
  __syncthreads();
  block_exclusive_scan(hPre, W);
  block_exclusive_scan(sPre, P);
  const uint32_t H = hPre[W];
  for (uint32_t k = blockIdx.x * kThreads + threadIdx.x; k < H; k += gridDim.x * kThreads) {
    uint32_t lo = 0, hi = W;  // last warp with hPre <= k
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (hPre[mid] <= k) lo = mid; else hi = mid;
    }
    const unsigned long long e = ps[lo];
    const unsigned long long dst = (e >> 9) * kTermPage + (e & 511ull) + (k - hPre[lo]);
    uint32_t slo = 0, shi = P;  // last page with sPre <= k
    while (shi - slo > 1) {
      const uint32_t mid = (slo + shi) >> 1;
      if (sPre[mid] <= k) slo = mid; else shi = mid;
    }
    const unsigned long long src = max((qN + slo) * kTermPage, N) + (k - sPre[slo]);
    PGA_GUARD(dst < N && src >= N && e != ~0ull, 12, continue);
    const bool inTail = src >= a.cap;
    if (inTail && src - a.cap >= a.tailCap) continue;
    const uint4* from = reinterpret_cast<const uint4*>(inTail ? a.tail + (src - a.cap) : a.out + src);
    uint4* to = reinterpret_cast<uint4*>(a.out + dst);
    uint4 r[4];
#pragma unroll
    for (int q = 0; q < 4; q++) r[q] = __ldcg(from + q);
#pragma unroll
    for (int q = 0; q < 4; q++) to[q] = r[q];
    if (a.termLinks != nullptr && dst < a.termLinkCap) {
      uint2 l = make_uint2(0u, 0u);
      if (inTail) {
        if (a.tailLinks != nullptr) l = a.tailLinks[src - a.cap];
      } else if (src < a.termLinkCap) {
        l = a.termLinks[src];
      }
      a.termLinks[dst] = l;
    }
  }
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long now;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
  return now;
}

// Resident blocks per SM the persistent kernel is compiled for (register budget).
#ifndef PGA_PERSISTENT_MIN_BLOCKS
#define PGA_PERSISTENT_MIN_BLOCKS 2
#endif

template <bool LEAF, int AFF, bool DYN = false>
__global__ void __launch_bounds__(kThreads, PGA_PERSISTENT_MIN_BLOCKS) k_derive_persistent(DeriveArgs a) {
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  if (blockIdx.x == 0 && threadIdx.x == 0) a.st->clockStart = global_ns();
  setup_block(a, sm);
  WarpOut w;
  warpout_init(a, w);
  if (AFF >= 2 && a.deferIn != nullptr) {
    warpout_level(a, w, a.numDeferIn);
    seed_deferred<true, LEAF, AFF>(a, w);
  } else {
    warpout_level(a, w, a.numAxioms - a.axiomBase);
    seed_axioms<true, LEAF, AFF>(a, w, a.axiomBase, a.numAxioms - a.axiomBase);
  }
  close_node_page(a, w);
  if (!grid_barrier(a, [&] {
        volatile DevState* vs = a.st;
        vs->levelHi = 0;
        a.levelStart[0] = 0;
        level_snapshot(a, 0);
      }))
    return;
  for (uint32_t level = 0;; level++) {
    volatile DevState* vs = a.st;
    if (vs->stop) break;
    const unsigned long long lo = vs->levelLo, hi = vs->levelHi;
    warpout_level(a, w, hi - lo);
    expand_level<true, LEAF, AFF, DYN>(a, w, lo, hi, a.itemsPerLane);
    close_node_page(a, w);
    if (!grid_barrier(a, [&] { level_snapshot(a, level + 1); })) return;
  }
  compact_terminals(a, w);
  if (blockIdx.x == 0 && threadIdx.x == 0 && a.outCount != nullptr) *a.outCount = ((volatile DevState*)a.st)->termCount;
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&a.st->clockEnd, global_ns());
}

__global__ void __launch_bounds__(kThreads, 2) k_seed(DeriveArgs a, uint32_t first, uint32_t count) {
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  setup_block(a, sm);
  WarpOut w;
  warpout_init(a, w);
  seed_axioms<false, false, 1>(a, w, first, count);
}

__global__ void __launch_bounds__(kThreads, 2) k_expand_level(DeriveArgs a, unsigned long long lo,
                                                              unsigned long long hi) {
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  setup_block(a, sm);
  WarpOut w;
  warpout_init(a, w);
  expand_level<false, false, 1>(a, w, lo, hi, 1);
}

__global__ void k_write_count(const DevState* st, unsigned long long* out) { *out = st->termCount; }

// This build's kernels, for the host code.  AFF: 0 the split operators only,
// 1 also the 1 -> 1 affine and selection steps, 2 also phases, Collider and
// IfCollides (no leaf children in place there).  The general-frame build only
// has the AFF >= 1 instantiations.
inline FrameKernels frame_kernels() {
  FrameKernels k;
#if PGA_GENERAL_FRAMES
  k.persistent[0] = k.persistent[2] = (const void*)k_derive_persistent<false, 1>;
  k.persistent[1] = k.persistent[3] = (const void*)k_derive_persistent<true, 1>;
  k.persistentDyn[0] = k.persistentDyn[1] = (const void*)k_derive_persistent<false, 1, true>;
#else
  k.persistent[0] = (const void*)k_derive_persistent<false, 0>;
  k.persistent[1] = (const void*)k_derive_persistent<true, 0>;
  k.persistent[2] = (const void*)k_derive_persistent<false, 1>;
  k.persistent[3] = (const void*)k_derive_persistent<true, 1>;
  k.persistentDyn[0] = (const void*)k_derive_persistent<false, 0, true>;
  k.persistentDyn[1] = (const void*)k_derive_persistent<false, 1, true>;
#endif
  k.phased = (const void*)k_derive_persistent<false, 2>;
  k.seed = (const void*)k_seed;
  k.expand = (const void*)k_expand_level;
  k.adjoint = nullptr;  // set by the builds that include adjoint.cuh
  k.adjointWide = nullptr;
  return k;
}

}  // inline namespace PGA_FRAMES_NS
}  // namespace pga
