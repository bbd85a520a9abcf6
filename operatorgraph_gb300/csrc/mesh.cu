// Triangle-mesh generation from terminal records (pga_generate_meshes).
//
// The reference generates triangle meshes inside the derivation: Generate<false,
// 0, TerminalIdx> calls ShapeGenerator<Box / Quad>::run with
// GenerationFunction<GenFuncFilter, 0> (include/pga/core/ShapeGenerator.cuh:377-512,
// 671-708; include/pga/rendering/GenerationFunctions.cuh:41-153), which takes
// vertex and index space with one atomic per terminal and writes
// model4 * corner, the face normal and the uv of every vertex.  Here the
// derivation writes a 64-byte record for every terminal as for instanced
// meshes, and one streaming pass expands the records of triangle-mesh rules.
//
// The positions come out bit for bit: a record holds m = R * s column by
// column (R the rotation, s the size), and the reference's corner
// model4 * (+-s_x / 2, +-s_y / 2, +-s_z / 2, 1) is, per row,
// ((R_i0 x + R_i1 y) + R_i2 z) + t_i with fl(R_ij * s_j / 2) = m_ij / 2 exactly
// (halving commutes with rounding) and the signs exact.  The normal is
// normalize(cross(v0 - v1, v2 - v1)) of the face's first three positions with
// the reference's operation order (vector.h: cross, dot, length = sqrt,
// normalize = v * (1 / length)); sqrt and the division are correctly rounded
// on both sides.
//
// Work layout: a warp takes 32 consecutive records; the lanes of each mesh
// found among them reserve one contiguous range of vertices and one of
// indices with a single atomic pair per mesh, then the warp writes the range
// together: every lane writes whole 16-byte vertex pieces and 4-byte indices at
// consecutive addresses, so the stores are coalesced whatever mix of boxes (24
// vertices, 36 indices) and quads (4, 6) the warp holds.
#include <cuda_runtime.h>

#include "engine_host.h"

namespace pga {
namespace {

constexpr int kMeshThreads = 256;

// Corner signs of the vertices ShapeGenerator<Box, false>::run writes
// (counter-clockwise build): faces top, bottom, left, right, front, back, four
// corners each; bit 4 * face + corner is set where the coordinate is +s/2.
constexpr uint32_t kBoxSignX = 0x6u | (0x6u << 4) | (0x0u << 8) | (0xFu << 12) | (0x6u << 16) | (0x9u << 20);
constexpr uint32_t kBoxSignY = 0xFu | (0x0u << 4) | (0x3u << 8) | (0x3u << 12) | (0x3u << 16) | (0x3u << 20);
constexpr uint32_t kBoxSignZ = 0xCu | (0x3u << 4) | (0x6u << 8) | (0x9u << 12) | (0xFu << 16) | (0x0u << 20);
// ShapeGenerator<Quad, false>::run: (-x, +y), (+x, +y), (+x, -y), (-x, -y), z = 0.
constexpr uint32_t kQuadSignX = 0x6u;
constexpr uint32_t kQuadSignY = 0x3u;

struct Rec {
  float a[3][3];  // R_ij * s_j / 2
  float t[3];
  bool quad;
};

// Position of corner c of face f: ((R_i0 x + R_i1 y) + R_i2 z) + t_i.
__device__ __forceinline__ void corner(const Rec& r, uint32_t f, uint32_t c, float p[3]) {
  const uint32_t bit = 4u * f + c;
  const float sx = ((r.quad ? kQuadSignX : kBoxSignX) >> bit) & 1u ? 1.0f : -1.0f;
  const float sy = ((r.quad ? kQuadSignY : kBoxSignY) >> bit) & 1u ? 1.0f : -1.0f;
  const float sz = (kBoxSignZ >> bit) & 1u ? 1.0f : -1.0f;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    // a quad's z term is R_i2 * 0: a signed zero
    const float z = r.quad ? __fmul_rn(r.a[i][2], 0.0f) : __fmul_rn(sz, r.a[i][2]);
    p[i] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(sx, r.a[i][0]), __fmul_rn(sy, r.a[i][1])), z), r.t[i]);
  }
}

// normalize(cross(v0 - v1, v2 - v1)) (ShapeGenerator.cuh:401, vector.h:505-575).
__device__ __forceinline__ void face_normal(const Rec& r, uint32_t f, float n[3]) {
  float v0[3], v1[3], v2[3];
  corner(r, f, 0, v0);
  corner(r, f, 1, v1);
  corner(r, f, 2, v2);
  const float a0 = __fsub_rn(v0[0], v1[0]), a1 = __fsub_rn(v0[1], v1[1]), a2 = __fsub_rn(v0[2], v1[2]);
  const float b0 = __fsub_rn(v2[0], v1[0]), b1 = __fsub_rn(v2[1], v1[1]), b2 = __fsub_rn(v2[2], v1[2]);
  const float c0 = __fsub_rn(__fmul_rn(a1, b2), __fmul_rn(a2, b1));
  const float c1 = __fsub_rn(__fmul_rn(a2, b0), __fmul_rn(a0, b2));
  const float c2 = __fsub_rn(__fmul_rn(a0, b1), __fmul_rn(a1, b0));
  const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(c0, c0), __fmul_rn(c1, c1)), __fmul_rn(c2, c2)));
  const float inv = __fdiv_rn(1.0f, len);
  n[0] = __fmul_rn(c0, inv);
  n[1] = __fmul_rn(c1, inv);
  n[2] = __fmul_rn(c2, inv);
}

// Exclusive prefix of faces over lanes below L among the group's boxes (6
// faces) and quads (1 face).
__device__ __forceinline__ uint32_t faces_below(uint32_t boxes, uint32_t quads, uint32_t lane) {
  const uint32_t lt = (lane >= 32u) ? 0xFFFFFFFFu : ((1u << lane) - 1u);
  return 6u * __popc(boxes & lt) + __popc(quads & lt);
}

__global__ void __launch_bounds__(kMeshThreads) k_meshes(const PgaTerminal* __restrict__ terms, unsigned long long n,
                                                          const DevRule* __restrict__ rules, uint32_t numEntries,
                                                          PgaTriangleMesh* meshes, uint32_t numMeshes, DevState* st) {
  const uint32_t lane = threadIdx.x & 31u;
  const unsigned long long warp = ((unsigned long long)blockIdx.x * kMeshThreads + threadIdx.x) >> 5;
  const unsigned long long warps = ((unsigned long long)gridDim.x * kMeshThreads) >> 5;
  for (unsigned long long base = warp * 32ull; base < n; base += warps * 32ull) {
    const unsigned long long i = base + lane;
    int mesh = -1;
    Rec r;
    if (i < n) {
      const float4* p = reinterpret_cast<const float4*>(terms + i);
      const float4 r0 = __ldcs(p), r1 = __ldcs(p + 1), r2 = __ldcs(p + 2);
      const uint4 meta = __ldcs(reinterpret_cast<const uint4*>(p + 3));
      const uint32_t entry = meta.x & 0xFFFFFFu, tidx = (meta.x >> 24) & 0x7Fu;
      if (entry < numEntries && (__ldg(&rules[entry].flags) & kRuleMesh)) {
        if (tidx < numMeshes) {
          mesh = (int)tidx;
        } else if (atomicCAS(&st->status, 0, PGA_ERR_BAD_PARAM) == 0) {
          atomicExch(&st->detail, (int)entry);
        }
      }
      const float row[3][4] = {{r0.x, r0.y, r0.z, r0.w}, {r1.x, r1.y, r1.z, r1.w}, {r2.x, r2.y, r2.z, r2.w}};
#pragma unroll
      for (int a = 0; a < 3; a++) {
#pragma unroll
        for (int b = 0; b < 3; b++) r.a[a][b] = __fmul_rn(row[a][b], 0.5f);
        r.t[a] = row[a][3];
      }
      r.quad = (meta.x >> 31) != 0;
    }
    uint32_t pending = __ballot_sync(0xFFFFFFFFu, mesh >= 0);
    while (pending) {
      const uint32_t leader = __ffs(pending) - 1u;
      const int m = __shfl_sync(0xFFFFFFFFu, mesh, leader);
      const uint32_t group = __ballot_sync(0xFFFFFFFFu, mesh == m) & pending;
      pending &= ~group;
      const uint32_t quads = __ballot_sync(0xFFFFFFFFu, r.quad) & group;
      const uint32_t boxes = group & ~quads;
      const uint32_t faces = 6u * __popc(boxes) + __popc(quads);
      uint32_t vb = 0, ib = 0;
      bool fits = false;
      PgaVertex* verts = nullptr;
      uint32_t* idx = nullptr;
      if (lane == leader) {
        PgaTriangleMesh* M = meshes + m;
        vb = atomicAdd(&M->numVertices, 4u * faces);
        ib = atomicAdd(&M->numIndices, 6u * faces);
        fits = (unsigned long long)vb + 4u * faces <= M->maxNumVertices &&
               (unsigned long long)ib + 6u * faces <= M->maxNumIndices;
        verts = M->vertices;
        idx = M->indices;
        if (!fits && atomicCAS(&st->status, 0, PGA_ERR_OUTPUT_OVERFLOW) == 0) atomicExch(&st->detail, m);
      }
      vb = __shfl_sync(0xFFFFFFFFu, vb, leader);
      ib = __shfl_sync(0xFFFFFFFFu, ib, leader);
      fits = __shfl_sync(0xFFFFFFFFu, fits, leader);
      verts = reinterpret_cast<PgaVertex*>(__shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(verts), leader));
      idx = reinterpret_cast<uint32_t*>(__shfl_sync(0xFFFFFFFFu, reinterpret_cast<unsigned long long>(idx), leader));
      if (!fits) continue;
      // Vertices: 3 float4 pieces per vertex, 4 vertices per face.
      float4* vdst = reinterpret_cast<float4*>(verts + vb);
      const uint32_t pieces = 12u * faces;
      for (uint32_t s0 = 0; s0 < pieces; s0 += 32u) {
        const uint32_t s = s0 + lane;
        const uint32_t fi = s / 12u;  // face of the group
        // the member lane whose faces contain fi: the largest lane L with faces_below(L) <= fi
        uint32_t lo = 0, hi = 32;
        while (hi - lo > 1) {
          const uint32_t mid = (lo + hi) >> 1;
          if (faces_below(boxes, quads, mid) <= fi) lo = mid; else hi = mid;
        }
        const uint32_t owner = lo;
        Rec o;
#pragma unroll
        for (int a = 0; a < 3; a++) {
#pragma unroll
          for (int b = 0; b < 3; b++) o.a[a][b] = __shfl_sync(0xFFFFFFFFu, r.a[a][b], owner);
          o.t[a] = __shfl_sync(0xFFFFFFFFu, r.t[a], owner);
        }
        o.quad = __shfl_sync(0xFFFFFFFFu, (int)r.quad, owner) != 0;
        if (s < pieces) {
          const uint32_t f = o.quad ? 0u : fi - faces_below(boxes, quads, owner);
          const uint32_t c = (s / 3u) & 3u, piece = s % 3u;
          const float uvx = (c == 0u || c == 3u) ? 1.0f : 0.0f, uvy = (c <= 1u) ? 1.0f : 0.0f;
          float4 out;
          if (piece == 0u) {
            float p[3];
            corner(o, f, c, p);
            out = make_float4(p[0], p[1], p[2], 1.0f);
          } else if (piece == 1u) {
            float nrm[3];
            face_normal(o, f, nrm);
            out = make_float4(nrm[0], nrm[1], nrm[2], uvx);
          } else {
            out = make_float4(uvy, 0.0f, 0.0f, 0.0f);
          }
          __stcs(vdst + s, out);
        }
      }
      // Indices: two triangles per face, (v, v+1, v+2) and (v, v+2, v+3).
      const uint32_t nidx = 6u * faces;
      for (uint32_t s = lane; s < nidx; s += 32u) {
        const uint32_t fi = s / 6u, k = s % 6u;
        const uint32_t off = (k == 0u || k == 3u) ? 0u : (k == 1u ? 1u : (k == 2u || k == 4u) ? 2u : 3u);
        __stcs(idx + ib + s, vb + 4u * fi + off);
      }
    }
  }
}

}  // namespace
}  // namespace pga

using namespace pga;

extern "C" PgaStatus pga_generate_meshes(PgaEngine* e, const PgaTerminal* dTerminals, uint64_t numTerminals,
                                         PgaTriangleMesh* dMeshes, uint32_t numMeshes, void* stream) {
  if (!e || (numTerminals && (!dTerminals || !dMeshes))) {
    set_error("pga_generate_meshes: null engine, terminals or meshes");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (numTerminals == 0) return PGA_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned long long warpsNeeded = (numTerminals + 31) / 32;
  const unsigned long long maxBlocks = (unsigned long long)e->numSMs * 8ull;
  unsigned long long blocks = (warpsNeeded + (kMeshThreads / 32) - 1) / (kMeshThreads / 32);
  if (blocks > maxBlocks) blocks = maxBlocks;
  if (blocks < 1) blocks = 1;
  k_meshes<<<(unsigned)blocks, kMeshThreads, 0, s>>>(dTerminals, numTerminals, e->dRules, e->numEntries, dMeshes,
                                                     numMeshes, e->dState);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_status(err, "pga_generate_meshes launch");
  return PGA_OK;
}
