// The oracle: a CPU restatement of the reference's derivation-and-terminal-
// emission path, its LBVH construction and (in double precision) the same
// derivation for gradient checks.
//
// TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
// cpu_baseline / reference legs of bench.py may load this library, and only as
// the checker or as the timed CPU baseline -- never as a product code path.
//
// Compiled with -O2 -ffp-contract=off so that every float operation rounds as
// written, in the order the reference writes it (host build of the reference:
// no FMA contraction).  The restatement is pinned against the reference's own
// evaluator (oracle/_ref/ref_harness) by tests/test_oracle.py.
//
// Citations are to files of the reference project (pboechat/OperatorGraph).
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/pga_gb300.h"

namespace {

// ---------------------------------------------------------------- helpers

// Random::tausStep / lcgStep / hybridTaus / nextSeed / range
// (include/pga/core/Random.cuh:15-57, host branch).
inline unsigned int taus_step(unsigned int& z, int S1, int S2, int S3, unsigned int M) {
  unsigned b = (((z << S1) ^ z) >> S2);
  return z = (((z & M) << S3) ^ b);
}
inline unsigned int lcg_step(unsigned int& z, unsigned int A, unsigned int C) { return z = (A * z + C); }

// Host-side float -> unsigned truncation as the reference uses it for seeds and
// axis/mode indices.  Values are non-negative in every grammar; negative and
// out-of-range inputs are clamped the way the device conversion (round toward
// zero, saturating) treats them.
inline unsigned int f2u(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (unsigned int)x;
}

inline float next_seed(float base, unsigned int modifier) {
  unsigned int z = (f2u(base) * UINT_MAX) + (modifier * 41231278u) % UINT_MAX;
  unsigned int z1 = (z + 7873234u) % UINT_MAX;
  unsigned int z2 = (z1 + 1237217827u) % UINT_MAX;
  unsigned int z3 = (z2 + 87382u) % UINT_MAX;
  unsigned int z4 = (z3 + 1410022u) % UINT_MAX;
  return (float)(2.3283064365387e-10 * (taus_step(z1, 13, 19, 12, 4294967294UL) ^ taus_step(z2, 2, 25, 4, 4294967288UL) ^
                                        taus_step(z3, 3, 11, 17, 4294967280UL) ^ lcg_step(z4, 1664525, 1013904223UL)));
}

template <typename F>
inline F rand_range(float seed, F lo, F hi) {
  if (seed < 1.0f) return F(seed) * (hi - lo) + lo;
  return hi;
}

// Derivation-path hash (no reference counterpart): splitmix64 finaliser.
inline uint64_t mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xbf58476d1ce4e5b9ULL;
  z ^= z >> 27;
  z *= 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return z;
}
inline uint64_t root_path(uint32_t axiom) { return mix64((uint64_t)axiom + 0x9E3779B97F4A7C15ULL); }
inline uint64_t child_path(uint64_t parent, uint32_t ordinal, int32_t entry) {
  return mix64(parent ^ (((uint64_t)ordinal << 32) | (uint32_t)entry));
}

// math::matrix<T,4,4> product and the translate/scale factories
// (deps/math/include/math/matrix.h:776-782, 904-919): full 4x4 products,
// zero terms included, summed left to right.
template <typename F>
struct M4 {
  F a[4][4];
};
template <typename F>
inline M4<F> mul(const M4<F>& x, const M4<F>& y) {
  M4<F> r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      r.a[i][j] = x.a[i][0] * y.a[0][j] + x.a[i][1] * y.a[1][j] + x.a[i][2] * y.a[2][j] + x.a[i][3] * y.a[3][j];
  return r;
}
template <typename F>
inline M4<F> make(F a00, F a01, F a02, F a03, F a10, F a11, F a12, F a13, F a20, F a21, F a22, F a23) {
  M4<F> r = {{{a00, a01, a02, a03}, {a10, a11, a12, a13}, {a20, a21, a22, a23}, {F(0), F(0), F(0), F(1)}}};
  return r;
}
template <typename F>
inline M4<F> translate(F x, F y, F z) {
  return make<F>(F(1), F(0), F(0), x, F(0), F(1), F(0), y, F(0), F(0), F(1), z);
}
template <typename F>
inline M4<F> scale(F x, F y, F z) {
  return make<F>(x, F(0), F(0), F(0), F(0), y, F(0), F(0), F(0), F(0), z, F(0));
}

// math::float4x4::rotateXYZ (matrix.h:876-888) after Rotate's degree to radian
// conversion (Rotate.cuh:34-36), all in float: sines and cosines of the three
// angles, products left to right.
template <typename F>
inline M4<F> rotate_xyz(float x, float y, float z) {
  const float k = 3.1415926535897932384626434f / 180.0f;
  x *= k;
  y *= k;
  z *= k;
  const float sa = std::sin(x), sb = std::sin(y), sg = std::sin(z);
  const float ca = std::cos(x), cb = std::cos(y), cg = std::cos(z);
  const float r00 = cb * cg, r01 = cg * sa * sb - ca * sg, r02 = ca * cg * sb + sa * sg;
  const float r10 = cb * sg, r11 = ca * cg + sa * sb * sg, r12 = -cg * sa + ca * sb * sg;
  const float r20 = -sb, r21 = cb * sa, r22 = ca * cb;
  return make<F>(F(r00), F(r01), F(r02), F(0), F(r10), F(r11), F(r12), F(0), F(r20), F(r21), F(r22), F(0));
}

// Oriented-box overlap, the separating-axis test of Gottschalk, Lin and
// Manocha (OBBTree, 1996; the form in Ericson, Real-Time Collision Detection,
// 4.4.1) as Collision::check states it for Box/Box, Box/Quad and Quad/Quad
// (Collision.cuh:35-262, 263-490, 506-738): A's 3 face axes, B's 3, the 9 edge
// cross products, separated when |T . L| > ra + rb.  A quad has no thickness in
// the projected sums (its half-extent z there is 0, which drops the same terms
// the reference drops) but keeps size.z / 2 where an axis test reads its own
// half-extent (ra = a[i], rb = b[k]).  Float, left-to-right sums, as written.
struct Obb {
  float c[3];     // centre: model column 3
  float u[3][3];  // u[j]: model column j
  float e[3];     // size / 2
  float es[3];    // size / 2 in the projected sums (a quad: z = 0)
};

inline float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

inline Obb make_obb(const float m[12], const float size[3], bool quad) {
  Obb o;
  for (int r = 0; r < 3; r++) {
    o.c[r] = m[r * 4 + 3];
    for (int j = 0; j < 3; j++) o.u[j][r] = m[r * 4 + j];
  }
  for (int k = 0; k < 3; k++) o.e[k] = o.es[k] = size[k] * 0.5f;
  if (quad) o.es[2] = 0.0f;
  return o;
}

inline bool obb_overlap(const Obb& A, const Obb& B) {
  const float v[3] = {B.c[0] - A.c[0], B.c[1] - A.c[1], B.c[2] - A.c[2]};
  float T[3], R[3][3], AR[3][3];
  for (int i = 0; i < 3; i++) T[i] = dot3(v, A.u[i]);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      R[i][j] = dot3(A.u[i], B.u[j]);
      AR[i][j] = std::fabs(R[i][j]);
    }
  const float* a = A.es;
  const float* b = B.es;
  for (int i = 0; i < 3; i++)
    if (std::fabs(T[i]) > A.e[i] + (b[0] * AR[i][0] + b[1] * AR[i][1] + b[2] * AR[i][2])) return false;
  for (int k = 0; k < 3; k++)
    if (std::fabs(T[0] * R[0][k] + T[1] * R[1][k] + T[2] * R[2][k]) >
        (a[0] * AR[0][k] + a[1] * AR[1][k] + a[2] * AR[2][k]) + B.e[k])
      return false;
  // L = A_i x B_j: with (p, q) the other two axes of A and (r, s) those of B,
  // ra = a_p |R_qj| + a_q |R_pj|, rb = b_r |R_is| + b_s |R_ir|,
  // t = |T_q R_pj - T_p R_qj| in the order the reference lists them.
  static const int P[3][2] = {{1, 2}, {0, 2}, {0, 1}};
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      const int p = P[i][0], q = P[i][1], r = P[j][0], s2 = P[j][1];
      const float ra = a[p] * AR[q][j] + a[q] * AR[p][j];
      const float rb = b[r] * AR[i][s2] + b[s2] * AR[i][r];
      const float t = i == 1 ? std::fabs(T[p] * R[q][j] - T[q] * R[p][j]) : std::fabs(T[q] * R[p][j] - T[p] * R[q][j]);
      if (t > ra + rb) return false;
    }
  return true;
}

// IntermediateSymbol<Box / Quad> as Collider stores it (IntermediateSymbol.cuh,
// IntermediateSymbolsBufferAdapter.cuh:200-215): the shape and its int tag.
struct StoredCollider {
  Obb obb;
  bool quad;
  int tag;
};

// Shapes::Shape + Symbol<ShapeT> (Shape.cuh:16-22, Symbol.cuh:9-15): model
// (3x4, kept as 4x4 with the constant last row), size, seed, custom attribute,
// entry index; plus the shape kind, the axiom index and the path hash.
template <typename F>
struct Sym {
  M4<F> model;
  F size[3];
  float seed;
  F custom;
  int32_t entry;
  uint32_t shape;
  uint32_t axiom;
  uint64_t path;
};

struct StoredCollider;

struct Ctx {
  const PgaProc* procs;
  uint32_t nProcs;
  const PgaEntry* entries;
  uint32_t nEntries;
  const PgaAxiom* axioms;
  uint32_t blockStride;
  int status;
  int detail;
  // Phases (multi-phase derivation): the phase being run, the phase of the
  // edges into each entry, and the colliders of the phases before this one.
  uint32_t phase = 0;
  // Index of the batch's first axiom in a larger batch (root path hashes, as
  // the engine's axiomBase when it derives a batch in axiom ranges).
  uint64_t axiomBase = 0;
  std::vector<uint32_t> entryPhase;
  std::vector<StoredCollider>* colliders = nullptr;
  size_t visibleColliders = 0;
};

template <typename F>
struct Blocks {
  const float* f32;
  const double* f64;
  F get(size_t i) const { return f64 ? F(f64[i]) : F(f32[i]); }
};

inline void fail(Ctx& c, int status, int detail) {
  if (c.status == PGA_OK) {
    c.status = status;
    c.detail = detail;
  }
}

// Shape::at (Shape.cuh:120-171).
template <typename F>
inline F attr(const Sym<F>& s, unsigned int i) {
  if (i < 12) return s.model.a[i / 4][i % 4];
  if (i < 15) return s.size[i - 12];
  if (i == 15) return F(s.seed);
  if (i == 16) return s.custom;
  return F(0);
}

// PackUtils::unpackOperand / unpackFloat2 (include/pga/core/PackUtils.h:30-43).
inline void unpack_operand(float a, unsigned int& p, float& x) {
  unsigned int r;
  std::memcpy(&r, &a, 4);
  p = r >> 30;
  r <<= 2;
  std::memcpy(&x, &r, 4);
}
inline void unpack_float2(float a, float& x, float& y) {
  y = fmodf(a, 4096.0f) / (4096 - 1.0f);
  x = floorf(a / 4096.0f) / (4096 - 1.0f);
}

// EncExp<Stack<4>>::eval (Parameters.cuh:518-664): postfix evaluation of
// packed operands; b[0] holds the operand count.
template <typename F>
F eval_exp(Ctx& c, const Sym<F>& s, const float* b) {
  F stack[PGA_MAX_EXP_LEVELS];
  unsigned int top = 0;
  unsigned int size = (unsigned int)b[0];
  for (unsigned int i = 1; i <= size && i < PGA_MAX_NUM_PARAMETER_VALUES; i++) {
    unsigned int p;
    float x;
    unpack_operand(b[i], p, x);
    F v;
    if (p == 0) {
      v = F(x);
    } else if (p == 1) {
      float lo, hi;
      unpack_float2(x, lo, hi);
      v = rand_range<F>(s.seed, F(lo), F(hi));
    } else if (p == 2) {
      v = attr(s, (unsigned int)std::round(x));
    } else {
      unsigned int op = (unsigned int)std::round(x);
      if (top < 2) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return F(0); }
      F p2 = stack[--top];
      F p1 = stack[--top];
      switch (op) {
        case 0: v = p1 + p2; break;
        case 1: v = p1 - p2; break;
        case 2: v = p1 / p2; break;
        case 3: v = p1 * p2; break;
        case 4: v = F(p1 == p2); break;
        case 5: v = F(p1 != p2); break;
        case 6: v = F(p1 < p2); break;
        case 7: v = F(p1 > p2); break;
        case 8: v = F(p1 <= p2); break;
        case 9: v = F(p1 >= p2); break;
        case 10: v = F(p1 != F(0) && p2 != F(0)); break;
        case 11: v = F(p1 != F(0) || p2 != F(0)); break;
        default: v = F(0); break;
      }
    }
    if (top >= PGA_MAX_EXP_LEVELS) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return F(0); }
    stack[top++] = v;
  }
  if (top == 0) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return F(0); }
  return stack[--top];
}

// dynEval (Parameters.cuh:668-711) plus PGA_PT_BLOCK.
template <typename F>
F dyn_eval(Ctx& c, const Blocks<F>& blk, const Sym<F>& s, const PgaParameter& p) {
  switch (p.type) {
    case PGA_PT_SCALAR: return F(p.value[0]);
    case PGA_PT_RAND: return rand_range<F>(s.seed, F(p.value[0]), F(p.value[1]));
    case PGA_PT_SHAPE_ATTR: return attr(s, f2u(p.value[0]));
    case PGA_PT_EXP: return eval_exp(c, s, p.value);
    case PGA_PT_BLOCK: {
      if (!blk.f32 && !blk.f64) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return F(0); }
      size_t slot = f2u(p.value[0]);
      if (slot >= c.blockStride) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return F(0); }
      return blk.get((size_t)c.axioms[s.axiom].block * c.blockStride + slot);
    }
    default: return F(0);  // unknown types evaluate to 0 without invariant checking
  }
}

template <typename F>
struct Out {
  std::vector<Sym<F>> work;
  PgaTerminal* term;
  double* termM;
  uint64_t* termPath;
  uint64_t cap;
  uint64_t count;
  std::vector<struct OracleMesh>* meshes = nullptr;  // triangle meshes (float derivation only)
  std::vector<std::vector<Sym<F>>> deferred;          // symbols waiting for a later phase, per phase
};

// One triangle mesh as GenerationFunction<GenFuncFilter, 0> fills
// TriangleMeshData: 12 floats per vertex (position 4, normal 3, uv 2, 3 unused)
// and the triangles' vertex numbers, both in the order they were written.
struct OracleMesh {
  std::vector<float> vertices;
  std::vector<uint32_t> indices;
};

// ShapeGenerator<Box / Quad, false>::run (ShapeGenerator.cuh:377-512, 671-708),
// counter-clockwise build: each face's four corners model4 * (+-hx, +-hy, +-hz, 1)
// with hx = size * 0.5 (Shape.cuh:70-73), the face normal
// normalize(cross(v0 - v1, v2 - v1)) (vector.h:505-575: dot left to right,
// length = sqrt, normalize = v * (1 / length)), uvs (1,1) (0,1) (0,0) (1,0),
// triangles (v, v+1, v+2) and (v, v+2, v+3) per face.
inline void shape_mesh(const M4<float>& model, const float size[3], bool quad, OracleMesh& mesh) {
  static const int box[6][4][3] = {
      {{-1, 1, -1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1}},      // top
      {{-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {-1, -1, -1}},  // bottom
      {{-1, 1, -1}, {-1, 1, 1}, {-1, -1, 1}, {-1, -1, -1}},  // left
      {{1, 1, 1}, {1, 1, -1}, {1, -1, -1}, {1, -1, 1}},      // right
      {{-1, 1, 1}, {1, 1, 1}, {1, -1, 1}, {-1, -1, 1}},      // front
      {{1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}, {1, -1, -1}},  // back
  };
  static const int quadCorners[4][3] = {{-1, 1, 0}, {1, 1, 0}, {1, -1, 0}, {-1, -1, 0}};
  const float h[3] = {size[0] * 0.5f, size[1] * 0.5f, size[2] * 0.5f};
  const float uv[4][2] = {{1.0f, 1.0f}, {0.0f, 1.0f}, {0.0f, 0.0f}, {1.0f, 0.0f}};
  const int faces = quad ? 1 : 6;
  for (int f = 0; f < faces; f++) {
    float v[4][4];
    for (int c = 0; c < 4; c++) {
      const int* sg = quad ? quadCorners[c] : box[f][c];
      const float p[4] = {sg[0] * h[0], sg[1] * h[1], quad ? 0.0f : sg[2] * h[2], 1.0f};
      for (int i = 0; i < 4; i++)
        v[c][i] = model.a[i][0] * p[0] + model.a[i][1] * p[1] + model.a[i][2] * p[2] + model.a[i][3] * p[3];
    }
    const float a[3] = {v[0][0] - v[1][0], v[0][1] - v[1][1], v[0][2] - v[1][2]};
    const float b[3] = {v[2][0] - v[1][0], v[2][1] - v[1][1], v[2][2] - v[1][2]};
    const float n[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const float inv = 1.0f / std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    const uint32_t base = (uint32_t)(mesh.vertices.size() / 12);
    for (int c = 0; c < 4; c++) {
      const float vert[12] = {v[c][0], v[c][1], v[c][2], v[c][3], n[0] * inv, n[1] * inv, n[2] * inv,
                              uv[c][0], uv[c][1], 0.0f, 0.0f, 0.0f};
      mesh.vertices.insert(mesh.vertices.end(), vert, vert + 12);
    }
    const uint32_t tri[6] = {base, base + 1, base + 2, base, base + 2, base + 3};
    mesh.indices.insert(mesh.indices.end(), tri, tri + 6);
  }
}

// BaseSymbolManager::dispatchNonTerminal (CPUEvaluator.h:230-239): the symbol
// goes to the queue of its entry's procedure; a shape of the wrong type is
// rejected (CPUEvaluator.h:64-68).
template <typename F>
void dispatch(Ctx& c, Out<F>& o, const Sym<F>& s) {
  if (s.entry < 0 || (uint32_t)s.entry >= c.nEntries) { fail(c, PGA_ERR_BAD_OPCODE, s.entry); return; }
  int32_t code = c.entries[s.entry].operatorCode;
  if (code < 0 || (uint32_t)code >= c.nProcs || c.procs[code].shape != s.shape) { fail(c, PGA_ERR_BAD_OPCODE, s.entry); return; }
  // enqueue(symbol, phaseIdx) (CPUEvaluator.h:155-190): a symbol whose edge
  // names a later phase waits for that phase's queues.
  const uint32_t ph = c.entryPhase.empty() ? 0u : c.entryPhase[(size_t)s.entry];
  if (ph > c.phase) {
    if (o.deferred.size() <= ph) o.deferred.resize(ph + 1);
    o.deferred[ph].push_back(s);
    return;
  }
  o.work.push_back(s);
}

template <typename F>
inline bool successor(Ctx& c, const PgaEntry& e, uint32_t k, int32_t parentEntry, int32_t& out) {
  if (k >= e.numSuccessors || k >= PGA_MAX_NUM_SUCCESSORS) { fail(c, PGA_ERR_BAD_OPCODE, parentEntry); return false; }
  out = e.successors[k].entryIndex;
  return true;
}

template <typename F>
inline bool param_ok(Ctx& c, const PgaEntry& e, uint32_t k, int32_t entry) {
  if (k >= e.numParameters) { fail(c, PGA_ERR_BAD_PARAM, entry); return false; }
  return true;
}

template <typename F>
inline bool axis_of(Ctx& c, F v, int32_t entry, unsigned int& axis) {
  axis = f2u(float(v));
  if (axis > 2) { fail(c, PGA_ERR_BAD_PARAM, entry); return false; }
  return true;
}

template <typename F>
void execute(Ctx& c, const Blocks<F>& blk, Out<F>& o, Sym<F> s) {
  const PgaEntry& e = c.entries[s.entry];
  const PgaProc& proc = c.procs[e.operatorCode];
  const F zero = F(0);
  switch (proc.op) {
    case PGA_OP_SUBDIVIDE: {
      // Subdivide<DynParams>::execute (Subdivide.cuh:177-236).  The symbol is
      // updated in place, so factors are evaluated on the previous child.
      if (!param_ok<F>(c, e, 0, s.entry)) return;
      unsigned int axis;
      if (!axis_of<F>(c, dyn_eval(c, blk, s, e.parameters[0]), s.entry, axis)) return;
      uint32_t n = e.numParameters;
      F totalSize = s.size[axis];
      F offset = totalSize * F(-0.5f);
      F absSum = zero, relSum = zero, scale = zero;
      for (uint32_t i = 1; i < n; i++) {
        F f = dyn_eval(c, blk, s, e.parameters[i]);
        absSum += F(f > zero) * f;
        relSum += F(f < zero) * (f * F(-1.0f));
      }
      if (relSum == zero) scale = zero;
      else scale = (totalSize - absSum) / relSum;
      if (scale < zero) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      float baseSeed = s.seed;
      F baseSize[3] = {s.size[0], s.size[1], s.size[2]};
      M4<F> baseModel = s.model;
      uint64_t basePath = s.path;
      int32_t self = s.entry;
      for (uint32_t i = 1, j = 0; i < n; j = i, i++) {
        F f = dyn_eval(c, blk, s, e.parameters[i]);
        F newSize = ((F(f < zero) * scale * f * F(-1.0f)) + (F(f > zero) * f));
        F off[3] = {zero, zero, zero};
        off[axis] = offset + (newSize * F(0.5f));
        s.size[0] = baseSize[0]; s.size[1] = baseSize[1]; s.size[2] = baseSize[2];
        s.size[axis] = newSize;
        s.model = mul(baseModel, translate<F>(off[0], off[1], off[2]));
        s.seed = next_seed(baseSeed, j);
        int32_t nxt;
        if (!successor<F>(c, e, j, self, nxt)) return;
        s.entry = nxt;
        s.path = child_path(basePath, j, nxt);
        dispatch(c, o, s);
        offset += newSize;
      }
      return;
    }
    case PGA_OP_SUBDIVIDE_STATIC: {
      // Subdivide<AxisT, Pair<Factor, DCall<k>>...>::execute (Subdivide.cuh:45-156):
      // factor k = DynParam<k+1>, successor k, seed modifier k, zero factors skipped.
      uint32_t K = proc.numChildren;
      if (!param_ok<F>(c, e, K, s.entry)) return;
      unsigned int axis;
      if (!axis_of<F>(c, dyn_eval(c, blk, s, e.parameters[0]), s.entry, axis)) return;
      F totalSize = s.size[axis];
      F offset = totalSize * F(-0.5f);
      F absSum = zero, relSum = zero, scale = zero;
      for (uint32_t k = 0; k < K; k++) {
        F f = dyn_eval(c, blk, s, e.parameters[k + 1]);
        absSum += F(f > zero) * f;
        relSum += F(f < zero) * (f * F(-1.0f));
      }
      if (relSum == zero) scale = zero;
      else scale = (totalSize - absSum) / relSum;
      Sym<F> child = s;
      for (uint32_t k = 0; k < K; k++) {
        F f = dyn_eval(c, blk, s, e.parameters[k + 1]);
        if (f != zero) {
          F newSize = ((F(f < zero) * scale * f * F(-1.0f)) + (F(f > zero) * f));
          F size3[3] = {s.size[0], s.size[1], s.size[2]};
          F off[3] = {zero, zero, zero};
          off[axis] = offset + (newSize * F(0.5f));
          size3[axis] = newSize;
          child.model = mul(s.model, translate<F>(off[0], off[1], off[2]));
          child.size[0] = size3[0]; child.size[1] = size3[1]; child.size[2] = size3[2];
          child.seed = next_seed(s.seed, f2u((float)k));
          int32_t nxt;
          if (!successor<F>(c, e, k, s.entry, nxt)) return;
          child.entry = nxt;
          child.path = child_path(s.path, k, nxt);
          dispatch(c, o, child);
          offset += newSize;
        }
      }
      return;
    }
    case PGA_OP_REPEAT: {
      // Repeat<false, Axis, Extent, Mode, Next>::execute (Repeat.cuh:70-191).
      if (!param_ok<F>(c, e, 2, s.entry)) return;
      unsigned int axis;
      if (!axis_of<F>(c, dyn_eval(c, blk, s, e.parameters[0]), s.entry, axis)) return;
      unsigned int mode = f2u(float(dyn_eval(c, blk, s, e.parameters[2])));
      F ext = dyn_eval(c, blk, s, e.parameters[1]);
      // getNewExtent (Repeat.cuh:28-31); abs() resolves to the float overload.
      F extent = ((F(ext < zero) * s.size[axis] * F(std::fabs(ext))) + (F(ext > zero) * ext));
      if (extent <= zero) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      F total = s.size[axis];
      if (total < zero) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      F division = total / extent;
      unsigned int reps;
      F e1, e2, e3;
      if (mode == 0 || mode == 1) {
        F rest = F(std::fmod(total, extent));
        bool exact = (rest == zero);
        reps = f2u(float(std::ceil(division)));
        e1 = F(exact) * extent + F(!exact) * rest;
        e2 = e3 = extent;
      } else if (mode == 2) {
        reps = f2u(float(std::floor(division)));
        if (reps > 0) e1 = e2 = e3 = total / F((float)reps);
        else e1 = e2 = e3 = zero;
      } else {
        fail(c, PGA_ERR_BAD_PARAM, s.entry);
        return;
      }
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      bool start = (mode == 0);
      F startExtent = F(start) * e1 + F(!start) * e3;
      Sym<F> child = s;
      child.entry = nxt;
      F newSize[3] = {s.size[0], s.size[1], s.size[2]};
      newSize[axis] = startExtent;
      child.size[0] = newSize[0]; child.size[1] = newSize[1]; child.size[2] = newSize[2];
      F off[3] = {zero, zero, zero};
      F halfStart = startExtent * F(0.5f);
      off[axis] = (total * F(-0.5f)) + halfStart;
      child.model = mul(s.model, translate<F>(off[0], off[1], off[2]));
      child.seed = next_seed(s.seed, 1u);
      child.path = child_path(s.path, 1u, nxt);
      dispatch(c, o, child);
      off[axis] += halfStart;
      F halfMid = e2 * F(0.5f);
      newSize[axis] = e2;
      for (unsigned int i = 2; i < reps; i++) {
        off[axis] += halfMid;
        child.size[0] = newSize[0]; child.size[1] = newSize[1]; child.size[2] = newSize[2];
        child.model = mul(s.model, translate<F>(off[0], off[1], off[2]));
        child.seed = next_seed(s.seed, i);
        child.path = child_path(s.path, i, nxt);
        dispatch(c, o, child);
        off[axis] += halfMid;
      }
      if (reps > 1) {
        F endExtent = F(start) * e3 + F(!start) * e1;
        off[axis] += endExtent * F(0.5f);
        newSize[axis] = endExtent;
        child.size[0] = newSize[0]; child.size[1] = newSize[1]; child.size[2] = newSize[2];
        child.model = mul(s.model, translate<F>(off[0], off[1], off[2]));
        child.seed = next_seed(s.seed, reps);
        child.path = child_path(s.path, reps, nxt);
        dispatch(c, o, child);
      }
      return;
    }
    case PGA_OP_COMPONENT_SPLIT: {
      // ComponentSplit<false, Top, Bottom, Sides>::execute (ComponentSplit.cuh:238-255)
      // with FaceSplitter<Box> (ComponentSplit.cuh:85-172).
      int32_t top, bottom, sides;
      if (!successor<F>(c, e, 0, s.entry, top) || !successor<F>(c, e, 1, s.entry, bottom) ||
          !successor<F>(c, e, 2, s.entry, sides))
        return;
      const M4<F>& model = s.model;
      F hx = s.size[0] * F(0.5f), hy = s.size[1] * F(0.5f), hz = s.size[2] * F(0.5f);
      const F one = F(1), mone = F(-1);
      Sym<F> face = s;
      face.shape = PGA_SHAPE_QUAD;
      for (unsigned int fi = 0; fi < 4; fi++) {
        switch (fi) {
          case 0:  // back
            face.model = mul(mul(model, translate<F>(zero, zero, -hz)),
                             make<F>(mone, zero, zero, zero, zero, one, zero, zero, zero, zero, mone, zero));
            face.size[0] = s.size[0]; face.size[1] = s.size[1];
            break;
          case 1:  // front
            face.model = mul(model, translate<F>(zero, zero, hz));
            face.size[0] = s.size[0]; face.size[1] = s.size[1];
            break;
          case 2:  // left
            face.model = mul(mul(model, translate<F>(-hx, zero, zero)),
                             make<F>(zero, zero, mone, zero, zero, one, zero, zero, one, zero, zero, zero));
            face.size[0] = s.size[2]; face.size[1] = s.size[1];
            break;
          default:  // right
            face.model = mul(mul(model, translate<F>(hx, zero, zero)),
                             make<F>(zero, zero, one, zero, zero, one, zero, zero, mone, zero, zero, zero));
            face.size[0] = s.size[2]; face.size[1] = s.size[1];
            break;
        }
        face.size[2] = one;
        face.seed = next_seed(s.seed, f2u(fi + 2.0f));
        face.entry = sides;
        face.path = child_path(s.path, fi + 2, sides);
        dispatch(c, o, face);
      }
      // bottom
      face.model = mul(mul(model, translate<F>(zero, -hy, zero)),
                       make<F>(one, zero, zero, zero, zero, zero, mone, zero, zero, one, zero, zero));
      face.size[0] = s.size[0]; face.size[1] = s.size[2]; face.size[2] = one;
      face.seed = next_seed(s.seed, 1u);
      face.entry = bottom;
      face.path = child_path(s.path, 1u, bottom);
      dispatch(c, o, face);
      // top
      face.model = mul(mul(model, translate<F>(zero, hy, zero)),
                       make<F>(one, zero, zero, zero, zero, zero, one, zero, zero, mone, zero, zero));
      face.size[0] = s.size[0]; face.size[1] = s.size[2]; face.size[2] = one;
      face.seed = next_seed(s.seed, 0u);
      face.entry = top;
      face.path = child_path(s.path, 0u, top);
      dispatch(c, o, face);
      return;
    }
    case PGA_OP_EXTRUDE: {
      // Extrude<Axis, Extent, Next>::execute (Extrude.cuh:29-56): Quad -> Box.
      if (!param_ok<F>(c, e, 1, s.entry)) return;
      F extent = dyn_eval(c, blk, s, e.parameters[1]);
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      Sym<F> box = s;
      box.shape = PGA_SHAPE_BOX;
      box.model = mul(s.model, make<F>(F(1), zero, zero, zero, zero, zero, F(-1), zero, zero, F(1), zero, zero));
      box.size[0] = s.size[0]; box.size[1] = extent; box.size[2] = s.size[1];
      box.seed = next_seed(s.seed, 0u);
      box.custom = s.custom;
      box.entry = nxt;
      box.path = child_path(s.path, 0u, nxt);
      dispatch(c, o, box);
      return;
    }
    case PGA_OP_IF_SIZE_LESS: {
      // IfSizeLess<Axis, Size, True, False>::execute (If.cuh:65-89): in place.
      if (!param_ok<F>(c, e, 1, s.entry)) return;
      unsigned int axis;
      if (!axis_of<F>(c, dyn_eval(c, blk, s, e.parameters[0]), s.entry, axis)) return;
      F size = dyn_eval(c, blk, s, e.parameters[1]);
      uint32_t branch = (s.size[axis] < size) ? 0u : 1u;
      int32_t nxt;
      if (!successor<F>(c, e, branch, s.entry, nxt)) return;
      s.entry = nxt;
      s.path = child_path(s.path, branch, nxt);
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_GENERATE_MESH:
    case PGA_OP_GENERATE: {
      // Generate<false, 1, TerminalIdx>::execute (Generate.cuh:30-34) ->
      // GenerationFunction<.., 1>::perShape (GenerationFunctions.cuh:158-188).
      if (!param_ok<F>(c, e, 0, s.entry)) return;
      unsigned int tidx = f2u(float(dyn_eval(c, blk, s, e.parameters[0])));
      if (tidx > 127u) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      M4<F> M = mul(s.model, scale<F>(s.size[0], s.size[1], s.size[2]));
      uint64_t k = o.count++;
      if (k < o.cap) {
        if (o.term) {
          PgaTerminal& t = o.term[k];
          for (int r = 0; r < 3; r++)
            for (int q = 0; q < 4; q++) t.m[r * 4 + q] = float(M.a[r][q]);
          t.rule = ((uint32_t)s.entry & 0xFFFFFFu) | (tidx << 24) | (s.shape == PGA_SHAPE_QUAD ? 0x80000000u : 0u);
          t.custom = float(s.custom);
          t.path = s.path;
        }
        if (o.termM)
          for (int r = 0; r < 3; r++)
            for (int q = 0; q < 4; q++) o.termM[k * 12 + r * 4 + q] = double(M.a[r][q]);
        if (o.termPath) o.termPath[k] = s.path;
      }
      if (proc.op == PGA_OP_GENERATE_MESH && o.meshes) {
        // Generate<false, 0, TerminalIdx>: the terminal's triangle mesh (float derivation only).
        if (tidx >= o.meshes->size()) o.meshes->resize(tidx + 1);
        M4<float> model;
        float size[3];
        for (int r = 0; r < 4; r++)
          for (int q = 0; q < 4; q++) model.a[r][q] = float(s.model.a[r][q]);
        for (int k2 = 0; k2 < 3; k2++) size[k2] = float(s.size[k2]);
        shape_mesh(model, size, s.shape == PGA_SHAPE_QUAD, (*o.meshes)[tidx]);
      }
      return;
    }
    case PGA_OP_TRANSLATE: {
      // Translate<X, Y, Z, Next>::execute (Translate.cuh:24-43): setModel(model * translate(x, y, z)),
      // then the successor on the same symbol.
      if (!param_ok<F>(c, e, 2, s.entry)) return;
      F x = dyn_eval(c, blk, s, e.parameters[0]), y = dyn_eval(c, blk, s, e.parameters[1]),
        z = dyn_eval(c, blk, s, e.parameters[2]);
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      s.model = mul(s.model, translate<F>(x, y, z));
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_SCALE: {
      // Scale<X, Y, Z, Next>::execute (Scale.cuh:23-45): size component by component as
      // ((v < 0) * size * v * -1) + ((v > 0) * v), then the successor.
      if (!param_ok<F>(c, e, 2, s.entry)) return;
      F v[3] = {dyn_eval(c, blk, s, e.parameters[0]), dyn_eval(c, blk, s, e.parameters[1]),
                dyn_eval(c, blk, s, e.parameters[2])};
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      for (int k = 0; k < 3; k++) s.size[k] = F(v[k] < F(0)) * s.size[k] * v[k] * F(-1) + F(v[k] > F(0)) * v[k];
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_RANDOM_RULE: {
      // RandomRule<DynParams>::execute (RandomRule.cuh:121-150): chance = frac(p0) in
      // float; weights summed in order; the first successor whose running
      // normalised share reaches the chance, none if rounding leaves it short.
      if (e.numParameters < 2) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      float c0 = float(dyn_eval(c, blk, s, e.parameters[0]));
      float chance = c0 - std::floor(c0);
      F sum = F(0);
      for (uint32_t i = 1; i < e.numParameters; i++) sum += dyn_eval(c, blk, s, e.parameters[i]);
      F acc = F(0);
      for (uint32_t i = 1; i < e.numParameters; i++) {
        acc += dyn_eval(c, blk, s, e.parameters[i]) / sum;
        if (F(chance) <= acc) {
          int32_t nxt;
          if (!successor<F>(c, e, i - 1, s.entry, nxt)) return;
          s.entry = nxt;
          s.path = child_path(s.path, i - 1, nxt);
          dispatch(c, o, s);
          return;
        }
      }
      return;
    }
    case PGA_OP_IF: {
      // If<Expression, True, False>::execute (If.cuh:22-49): the first
      // successor when the value is nonzero, else the second.
      if (!param_ok<F>(c, e, 0, s.entry)) return;
      const bool yes = dyn_eval(c, blk, s, e.parameters[0]) != F(0);
      int32_t nxt;
      if (!successor<F>(c, e, yes ? 0 : 1, s.entry, nxt)) return;
      s.path = child_path(s.path, yes ? 0u : 1u, nxt);
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_SWAP_SIZE: {
      // SwapSize<X, Y, Z, Next>::execute (SwapSize.cuh:20-38): the size's
      // components re-read along the three axes (host truncation).
      if (!param_ok<F>(c, e, 2, s.entry)) return;
      unsigned ax[3];
      for (int k = 0; k < 3; k++) {
        const float v = float(dyn_eval(c, blk, s, e.parameters[k]));
        ax[k] = v > 0.0f ? static_cast<unsigned>(v) : 0u;
        if (ax[k] > 2) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      }
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      const F sz[3] = {s.size[ax[0]], s.size[ax[1]], s.size[ax[2]]};
      for (int k = 0; k < 3; k++) s.size[k] = sz[k];
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_COLLIDER: {
      // Collider<Tag, Next>::execute (Collider.cuh:20-45): a positive tag stores
      // the shape with it (visible to IfCollides from the next phase on).
      if (!param_ok<F>(c, e, 0, s.entry)) return;
      const unsigned tag = f2u(float(dyn_eval(c, blk, s, e.parameters[0])));
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      if (tag > 0 && c.colliders) {
        float m[12], size[3];
        for (int r = 0; r < 3; r++)
          for (int q = 0; q < 4; q++) m[r * 4 + q] = float(s.model.a[r][q]);
        for (int k2 = 0; k2 < 3; k2++) size[k2] = float(s.size[k2]);
        c.colliders->push_back(StoredCollider{make_obb(m, size, s.shape == PGA_SHAPE_QUAD), s.shape == PGA_SHAPE_QUAD,
                                              (int)tag});
      }
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_IF_COLLIDES: {
      // IfCollides<Tag, True, False>::execute (IfCollides.cuh:18-36): true when
      // a stored shape with the tag (compared as the unsigned char rule tag,
      // BVHTraversal.cuh:16) overlaps this one (Collision::check(stored,
      // shape)).  The reference prunes with a BVH; the answer is the same
      // "any" over the stored shapes, which is what this loop computes.
      if (!param_ok<F>(c, e, 0, s.entry)) return;
      const unsigned char tag = (unsigned char)f2u(float(dyn_eval(c, blk, s, e.parameters[0])));
      float m[12], size[3];
      for (int r = 0; r < 3; r++)
        for (int q = 0; q < 4; q++) m[r * 4 + q] = float(s.model.a[r][q]);
      for (int k2 = 0; k2 < 3; k2++) size[k2] = float(s.size[k2]);
      const bool quad = s.shape == PGA_SHAPE_QUAD;
      const Obb me = make_obb(m, size, quad);
      bool hit = false;
      for (size_t k = 0; c.colliders && k < c.visibleColliders && !hit; k++) {
        const StoredCollider& sc = (*c.colliders)[k];
        if (sc.tag != (int)tag) continue;
        // Collision::check(Quad, Box) is check(Box, Quad) (Collision.cuh:734-737)
        hit = (sc.quad && !quad) ? obb_overlap(me, sc.obb) : obb_overlap(sc.obb, me);
      }
      const uint32_t branch = hit ? 0u : 1u;
      int32_t nxt;
      if (!successor<F>(c, e, branch, s.entry, nxt)) return;
      s.path = child_path(s.path, branch, nxt);
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_RANDOM_RULE_STATIC: {
      // RandomRule<Chance, Pair<P, Next>...>::execute (RandomRule.cuh:33-99):
      // getProbabilitiesSum recurses as p1 + (p2 + (... + pn)); each pair's
      // normalised share is added to the running sum and the pair is taken
      // when the share is nonzero and the chance is within the sum; the last
      // pair is taken unconditionally.
      if (e.numParameters < 2) { fail(c, PGA_ERR_BAD_PARAM, s.entry); return; }
      float c0 = float(dyn_eval(c, blk, s, e.parameters[0]));
      float chance = c0 - std::floor(c0);
      const uint32_t n = e.numParameters - 1;
      F sum = dyn_eval(c, blk, s, e.parameters[n]);
      for (uint32_t i = n - 1; i >= 1; i--) sum = dyn_eval(c, blk, s, e.parameters[i]) + sum;
      F acc = F(0);
      for (uint32_t i = 1; i <= n; i++) {
        F share = dyn_eval(c, blk, s, e.parameters[i]) / sum;
        acc += share;
        if (i == n || (share != F(0) && F(chance) <= acc)) {
          int32_t nxt;
          if (!successor<F>(c, e, i - 1, s.entry, nxt)) return;
          s.entry = nxt;
          s.path = child_path(s.path, i - 1, nxt);
          dispatch(c, o, s);
          return;
        }
      }
      return;
    }
    case PGA_OP_ROTATE: {
      // Rotate<X, Y, Z, Next>::execute (Rotate.cuh:24-41): the angles in
      // degrees, times pi / 180 in float, setModel(model * rotateXYZ(angles))
      // (matrix.h:876-888), then the successor on the same symbol.
      if (!param_ok<F>(c, e, 2, s.entry)) return;
      float x = float(dyn_eval(c, blk, s, e.parameters[0])), y = float(dyn_eval(c, blk, s, e.parameters[1])),
            z = float(dyn_eval(c, blk, s, e.parameters[2]));
      int32_t nxt;
      if (!successor<F>(c, e, 0, s.entry, nxt)) return;
      s.model = mul(s.model, rotate_xyz<F>(x, y, z));
      s.entry = nxt;
      dispatch(c, o, s);
      return;
    }
    case PGA_OP_REPLICATE: {
      // Replicate<DynParams>::execute (Replicate.cuh:95-110): the symbol, with
      // only its entry changed, dispatched once per successor.
      for (uint32_t i = 0; i < e.numSuccessors; i++) {
        int32_t nxt;
        if (!successor<F>(c, e, i, s.entry, nxt)) return;
        Sym<F> child = s;
        child.entry = nxt;
        child.path = child_path(s.path, i, nxt);
        dispatch(c, o, child);
      }
      return;
    }
    case PGA_OP_DISCARD:
      return;
    default:
      fail(c, PGA_ERR_BAD_OPCODE, s.entry);
      return;
  }
}

// The phase of every entry: the phaseIndex of the successor edges that lead to
// it (the engine requires them to agree; axioms start in phase 0).  Returns
// false, with BAD_PARAM, when two edges into one entry name different phases.
inline bool entry_phases(Ctx& c) {
  c.entryPhase.assign(c.nEntries, 0u);
  std::vector<int> seen(c.nEntries, -1);
  for (uint32_t i = 0; i < c.nEntries; i++) {
    const PgaEntry& e = c.entries[i];
    for (uint32_t k = 0; k < e.numSuccessors && k < PGA_MAX_NUM_SUCCESSORS; k++) {
      const int32_t t = e.successors[k].entryIndex;
      if (t < 0 || (uint32_t)t >= c.nEntries) continue;
      const int ph = e.successors[k].phaseIndex < 0 ? 0 : e.successors[k].phaseIndex;
      if (seen[t] >= 0 && seen[t] != ph) {
        fail(c, PGA_ERR_BAD_PARAM, (int)i);
        return false;
      }
      seen[t] = ph;
      c.entryPhase[t] = (uint32_t)ph;
    }
  }
  return true;
}

template <typename F>
int derive(Ctx& c, const Blocks<F>& blk, const double* axiomSizes, Out<F>& o, uint32_t nAxioms) {
  std::vector<StoredCollider> colliders;
  c.colliders = &colliders;
  c.phase = 0;
  c.visibleColliders = 0;
  if (!entry_phases(c)) return c.status;
  for (uint32_t id = 0; id < nAxioms && c.status == PGA_OK; id++) {
    // Axiom generation as Grid::...::generateAxiom (Grid.cuh:199-204) then
    // dispatchAxiom (CPUEvaluator.h:255-266).
    const PgaAxiom& a = c.axioms[id];
    Sym<F> s;
    s.model = make<F>(F(1), F(0), F(0), F(a.position[0]), F(0), F(1), F(0), F(a.position[1]), F(0), F(0), F(1),
                      F(a.position[2]));
    for (int k = 0; k < 3; k++) s.size[k] = axiomSizes ? F(axiomSizes[id * 3 + k]) : F(a.size[k]);
    s.seed = a.seed;
    s.custom = F(a.custom);
    s.entry = (int32_t)a.entry;
    s.shape = a.shape;
    s.axiom = id;
    s.path = root_path((uint32_t)(c.axiomBase + id));
    dispatch(c, o, s);
    while (!o.work.empty() && c.status == PGA_OK) {
      Sym<F> cur = o.work.back();
      o.work.pop_back();
      execute(c, blk, o, cur);
    }
  }
  // Later phases: MultiPhaseEvaluator::execute (CPUEvaluator.h:330-352) runs
  // the phases in order; the colliders stored so far are what IfCollides sees.
  for (uint32_t ph = 1; ph < o.deferred.size() && c.status == PGA_OK; ph++) {
    c.phase = ph;
    c.visibleColliders = colliders.size();
    std::vector<Sym<F>> start;
    start.swap(o.deferred[ph]);
    for (size_t k = 0; k < start.size() && c.status == PGA_OK; k++) {
      o.work.push_back(start[k]);
      while (!o.work.empty() && c.status == PGA_OK) {
        Sym<F> cur = o.work.back();
        o.work.pop_back();
        execute(c, blk, o, cur);
      }
    }
  }
  c.colliders = nullptr;
  return c.status;
}

// ----------------------------------------------------------------- LBVH

// spread / morton30 (include/pga/core/GPUBVHConstructor.cuh:44-64).
inline unsigned int spread(unsigned int v) {
  v = (v | (v << 16)) & 0x030000FF;
  v = (v | (v << 8)) & 0x0300F00F;
  v = (v | (v << 4)) & 0x030C30C3;
  v = (v | (v << 2)) & 0x09249249;
  return v;
}
// Device float -> unsigned conversion (round toward zero, saturating, NaN -> 0).
inline unsigned int f2u_rz_sat(float x) {
  if (!(x > 0.0f)) return 0u;
  if (x >= 4294967296.0f) return 0xFFFFFFFFu;
  return (unsigned int)x;
}
inline unsigned int morton30(const float* bmin, const float* bsize, const float* centre) {
  unsigned int code = 0;
  for (int k = 0; k < 3; k++) {
    float nc = (centre[k] - bmin[k]) / bsize[k];
    unsigned int v = f2u_rz_sat(nc * 1023);
    code |= spread(v) << k;
  }
  return code;
}

inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

}  // namespace

extern "C" {

// Triangle meshes of the last oracle_derive call (its triangle-mesh terminals).
static std::vector<OracleMesh> g_meshes;

uint32_t oracle_mesh_count(void) { return (uint32_t)g_meshes.size(); }

// obb_overlap on n pairs laid out as the reference harness reads them: kinds
// (uint32 0 box / 1 quad) of A and B, then A's row-major 3x4 model and size,
// then B's (128 bytes a pair); one result byte per pair.
void oracle_collide(const void* pairs, uint64_t n, uint8_t* out) {
  const uint8_t* p = static_cast<const uint8_t*>(pairs);
  for (uint64_t k = 0; k < n; k++, p += 128) {
    uint32_t kind[2];
    float f[30];
    std::memcpy(kind, p, 8);
    std::memcpy(f, p + 8, 120);
    const Obb a = make_obb(f, f + 12, kind[0] == 1), b = make_obb(f + 15, f + 27, kind[1] == 1);
    // Collision::check(Quad, Box) is check(Box, Quad) (Collision.cuh:734-737)
    out[k] = (kind[0] == 1 && kind[1] == 0) ? obb_overlap(b, a) : obb_overlap(a, b);
  }
}

void oracle_mesh_sizes(uint32_t mesh, uint32_t* numVertices, uint32_t* numIndices) {
  *numVertices = mesh < g_meshes.size() ? (uint32_t)(g_meshes[mesh].vertices.size() / 12) : 0u;
  *numIndices = mesh < g_meshes.size() ? (uint32_t)g_meshes[mesh].indices.size() : 0u;
}

void oracle_mesh_copy(uint32_t mesh, float* vertices, uint32_t* indices) {
  if (mesh >= g_meshes.size()) return;
  std::copy(g_meshes[mesh].vertices.begin(), g_meshes[mesh].vertices.end(), vertices);
  std::copy(g_meshes[mesh].indices.begin(), g_meshes[mesh].indices.end(), indices);
}

// oracle_derive for a shard of a larger batch: axiom k of this call hashes its
// root path as axiom axiomBase + k (the records are those the whole batch gives
// for these axioms).
int oracle_derive_base(const PgaProc* procs, uint32_t nProcs, const PgaEntry* entries, uint32_t nEntries,
                       const PgaAxiom* axioms, uint32_t nAxioms, const float* blocks, uint32_t blockStride,
                       PgaTerminal* out, uint64_t cap, uint64_t* count, int32_t* detail, uint64_t axiomBase) {
  Ctx c = {procs, nProcs, entries, nEntries, axioms, blockStride, PGA_OK, 0};
  c.axiomBase = axiomBase;
  Blocks<float> blk = {blocks, nullptr};
  Out<float> o;
  g_meshes.clear();
  o.meshes = &g_meshes;
  o.term = out;
  o.termM = nullptr;
  o.termPath = nullptr;
  o.cap = cap;
  o.count = 0;
  o.work.reserve(1024);
  derive<float>(c, blk, nullptr, o, nAxioms);
  *count = o.count;
  if (detail) *detail = c.detail;
  if (c.status == PGA_OK && o.count > cap) return PGA_ERR_OUTPUT_OVERFLOW;
  return c.status;
}

int oracle_derive(const PgaProc* procs, uint32_t nProcs, const PgaEntry* entries, uint32_t nEntries,
                  const PgaAxiom* axioms, uint32_t nAxioms, const float* blocks, uint32_t blockStride,
                  PgaTerminal* out, uint64_t cap, uint64_t* count, int32_t* detail) {
  return oracle_derive_base(procs, nProcs, entries, nEntries, axioms, nAxioms, blocks, blockStride, out, cap, count,
                            detail, 0);
}

// The same derivation carried out in double precision (seeds stay float, as
// they are discrete).  blocks64 / axiomSizes64 override the float inputs when
// given; used for central finite differences of the adjoint.
int oracle_derive_f64(const PgaProc* procs, uint32_t nProcs, const PgaEntry* entries, uint32_t nEntries,
                      const PgaAxiom* axioms, uint32_t nAxioms, const double* blocks64, uint32_t blockStride,
                      const double* axiomSizes64, double* outM, uint64_t* outPath, uint64_t cap, uint64_t* count) {
  Ctx c = {procs, nProcs, entries, nEntries, axioms, blockStride, PGA_OK, 0};
  Blocks<double> blk = {nullptr, blocks64};
  Out<double> o;
  o.term = nullptr;
  o.termM = outM;
  o.termPath = outPath;
  o.cap = cap;
  o.count = 0;
  derive<double>(c, blk, axiomSizes64, o, nAxioms);
  *count = o.count;
  if (c.status == PGA_OK && o.count > cap) return PGA_ERR_OUTPUT_OVERFLOW;
  return c.status;
}

// LBVH over terminal boxes.  Restates GPUBVHConstructor.cuh:66-261 with three
// documented changes: the Morton key's tie-break is the derivation path
// (key = morton30 << 34 | path >> 30, ties resolved on the full path) instead
// of the nondeterministic emission index; the Karras codes are
// morton30 << 32 | sorted position; AABBs start from -FLT_MAX (the reference
// starts _max at FLT_MIN, AABB.cuh:20, BoundingVolumeConstructor.cuh:24,58).
int oracle_lbvh(const PgaTerminal* t, uint64_t n, const float* bounds6, int32_t* nodes, uint32_t* leafParents,
                float* aabbs, uint32_t* leafTerminal, uint64_t* keysOut) {
  if (n < 2) return PGA_ERR_INVALID_ARGUMENT;
  const float bmin[3] = {bounds6[0], bounds6[1], bounds6[2]};
  const float bsize[3] = {bounds6[3] - bounds6[0], bounds6[4] - bounds6[1], bounds6[5] - bounds6[2]};
  std::vector<uint64_t> key(n);
  std::vector<uint32_t> idx(n);
  for (uint64_t i = 0; i < n; i++) {
    const float centre[3] = {t[i].m[3], t[i].m[7], t[i].m[11]};
    key[i] = ((uint64_t)morton30(bmin, bsize, centre) << 34) | (t[i].path >> 30);
    idx[i] = (uint32_t)i;
  }
  std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
    if (key[a] != key[b]) return key[a] < key[b];
    return t[a].path < t[b].path;
  });
  std::vector<uint64_t> codes(n);
  for (uint64_t i = 0; i < n; i++) {
    leafTerminal[i] = idx[i];
    keysOut[i] = key[idx[i]];
    codes[i] = ((key[idx[i]] >> 34) << 32) | (uint64_t)i;
  }
  const int64_t N = (int64_t)n;
  auto delta = [&](int64_t a, int64_t b) -> int { return clz64(codes[a] ^ codes[b]); };
  // buildRadixTree (GPUBVHConstructor.cuh:88-213), one internal node per i.
  for (int64_t i = 0; i < N - 1; i++) {
    int64_t d, len;
    if (i == 0) {
      d = 1;
      len = N - 1;
    } else {
      int t1 = delta(i, i - 1), t2 = delta(i, i + 1);
      int dmin = std::min(t1, t2);
      d = (t2 - t1 >= 0) ? 1 : -1;
      int64_t step = 128, j;
      while ((j = i + d * step) >= 0 && j < N && delta(i, j) > dmin) step <<= 2;
      len = 0;
      for (step >>= 1; step > 0; step >>= 1) {
        j = i + (len + step) * d;
        if (j < 0 || j >= N) continue;
        if (delta(i, j) > dmin) len += step;
      }
    }
    int64_t j = i + len * d;
    int dnode = delta(i, j);
    int64_t step = (int64_t)1 << std::max(0, 31 - clz32((uint32_t)len));
    step >>= (step == len);
    int64_t s = 0;
    for (; step > 0; step >>= 1) {
      int64_t k = i + (s + step) * d;
      if (k < 0 || k >= N) continue;  // out of the array: the test cannot pass
      if (delta(i, k) > dnode) s += step;
    }
    int64_t gamma = i + s * d + std::min<int64_t>(d, 0);
    int64_t left = (std::min(i, j) == gamma) ? gamma : -gamma;
    int64_t right = (std::max(i, j) == gamma + 1) ? (gamma + 1) : -(gamma + 1);
    nodes[i * 3 + 1] = (int32_t)left;
    nodes[i * 3 + 2] = (int32_t)right;
    if (left < 0) nodes[(-left) * 3 + 0] = (int32_t)i;
    else leafParents[left] = (uint32_t)i;
    if (right < 0) nodes[(-right) * 3 + 0] = (int32_t)i;
    else leafParents[right] = (uint32_t)i;
  }
  nodes[0] = -1;  // the root has no parent
  // Bottom-up refit (propagateBVH, GPUBVHConstructor.cuh:215-261): min/max are
  // exact, so the result does not depend on the visiting order.
  std::vector<float> leaf(n * 6);
  for (uint64_t i = 0; i < n; i++) {
    const PgaTerminal& tt = t[idx[i]];
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    bool quad = (tt.rule >> 31) != 0;
    for (int cz = 0; cz < (quad ? 1 : 2); cz++)
      for (int cy = 0; cy < 2; cy++)
        for (int cx = 0; cx < 2; cx++) {
          float x = cx ? 0.5f : -0.5f, y = cy ? 0.5f : -0.5f, z = quad ? 0.0f : (cz ? 0.5f : -0.5f);
          for (int r = 0; r < 3; r++) {
            // (model3x4 * float4(x, y, z, 1)) with the scale folded into m
            // (matrix.h:261-266 for the 3x4 * 4-vector product).
            float p = tt.m[r * 4 + 0] * x + tt.m[r * 4 + 1] * y + tt.m[r * 4 + 2] * z + tt.m[r * 4 + 3] * 1.0f;
            mn[r] = std::min(mn[r], p);
            mx[r] = std::max(mx[r], p);
          }
        }
    for (int r = 0; r < 3; r++) {
      leaf[i * 6 + r] = mn[r];
      leaf[i * 6 + 3 + r] = mx[r];
    }
  }
  // Post-order over internal nodes with an explicit stack.
  std::vector<int64_t> stack;
  std::vector<uint8_t> visited(n, 0);
  stack.push_back(0);
  while (!stack.empty()) {
    int64_t i = stack.back();
    int32_t l = nodes[i * 3 + 1], r = nodes[i * 3 + 2];
    if (!visited[i]) {
      visited[i] = 1;
      if (r < 0) stack.push_back(-r);
      if (l < 0) stack.push_back(-l);
      continue;
    }
    stack.pop_back();
    const float* a = l < 0 ? &aabbs[(size_t)(-l) * 6] : &leaf[(size_t)l * 6];
    const float* b = r < 0 ? &aabbs[(size_t)(-r) * 6] : &leaf[(size_t)r * 6];
    for (int k = 0; k < 3; k++) {
      aabbs[i * 6 + k] = std::min(a[k], b[k]);
      aabbs[i * 6 + 3 + k] = std::max(a[3 + k], b[3 + k]);
    }
  }
  return PGA_OK;
}

}  // extern "C"
