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
// Work layout: a block takes a tile of 1024 consecutive records.  The lanes of
// each mesh in a warp's 32 records take a contiguous run of the tile's faces
// with one shared-memory atomic; then one global atomic pair per mesh reserves
// the tile's vertex and index space (a few per tile instead of one per warp:
// same-address atomics serialise); then each warp writes its runs together:
// every lane writes whole 16-byte vertex pieces and 4-byte indices at
// consecutive addresses, so the stores are coalesced whatever mix of boxes (24
// vertices, 36 indices) and quads (4, 6) the warp holds.
#include <cuda_runtime.h>

#include "engine_host.h"

namespace pga {
namespace {

constexpr int kMeshThreads = 128;

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

// normalize(cross(v0 - v1, v2 - v1)) of a face's corners (ShapeGenerator.cuh:401,
// vector.h:505-575).
__device__ __forceinline__ void face_normal(const float v[4][3], float n[3]) {
  const float* v0 = v[0];
  const float* v1 = v[1];
  const float* v2 = v[2];
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

// A record's mesh (-1: not a triangle-mesh terminal) and shape; raises
// BAD_PARAM for a mesh index beyond the mesh array.
__device__ __forceinline__ int record_mesh(const PgaTerminal* terms, unsigned long long i, unsigned long long n,
                                           const DevRule* rules, uint32_t numEntries, uint32_t numMeshes,
                                           DevState* st, bool raise, Rec& r) {
  r.quad = false;
  if (i >= n) return -1;
  const float4* p = reinterpret_cast<const float4*>(terms + i);
  const float4 r0 = __ldg(p), r1 = __ldg(p + 1), r2 = __ldg(p + 2);
  const uint4 meta = __ldg(reinterpret_cast<const uint4*>(p + 3));
  const float row[3][4] = {{r0.x, r0.y, r0.z, r0.w}, {r1.x, r1.y, r1.z, r1.w}, {r2.x, r2.y, r2.z, r2.w}};
#pragma unroll
  for (int a = 0; a < 3; a++) {
#pragma unroll
    for (int b = 0; b < 3; b++) r.a[a][b] = __fmul_rn(row[a][b], 0.5f);
    r.t[a] = row[a][3];
  }
  r.quad = (meta.x >> 31) != 0;
  const uint32_t entry = meta.x & 0xFFFFFFu, tidx = (meta.x >> 24) & 0x7Fu;
  if (entry >= numEntries || !(__ldg(&rules[entry].flags) & kRuleMesh)) return -1;
  if (tidx < numMeshes) return (int)tidx;
  if (raise && atomicCAS(&st->status, 0, PGA_ERR_BAD_PARAM) == 0) atomicExch(&st->detail, (int)entry);
  return -1;
}

// Records per block tile: 4 warps x 32 lanes x kMeshBatches.
constexpr int kMeshBatches = 8;
constexpr uint32_t kMaxMeshes = 128;  // terminal indices are 7 bits

__global__ void __launch_bounds__(kMeshThreads, 6) k_meshes(const PgaTerminal* __restrict__ terms, unsigned long long n,
                                                          const DevRule* __restrict__ rules, uint32_t numEntries,
                                                          PgaTriangleMesh* meshes, uint32_t numMeshes, DevState* st) {
  __shared__ uint32_t sFaces[kMaxMeshes];   // faces of each mesh in this tile
  __shared__ uint32_t sVBase[kMaxMeshes];   // the tile's first vertex / index in each mesh
  __shared__ uint32_t sIBase[kMaxMeshes];
  __shared__ uint32_t sFits[kMaxMeshes];
  __shared__ float4 sStage[kMeshThreads / 32][32 * 12];  // per warp: 32 faces x 4 vertices x 48 B
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const unsigned long long tileRecords = (unsigned long long)kMeshThreads * kMeshBatches;
  for (unsigned long long tile = blockIdx.x; tile * tileRecords < n; tile += gridDim.x) {
    for (uint32_t m = threadIdx.x; m < numMeshes; m += kMeshThreads) sFaces[m] = 0;
    __syncthreads();
    // 1. Faces per mesh in the tile: each warp group of one mesh takes a
    //    contiguous run of the tile's faces with one shared-memory atomic.
    uint32_t myFace[kMeshBatches];
#pragma unroll
    for (int b = 0; b < kMeshBatches; b++) {
      const unsigned long long i = tile * tileRecords + (unsigned long long)(warp * kMeshBatches + b) * 32ull + lane;
      Rec r;
      const int mesh = record_mesh(terms, i, n, rules, numEntries, numMeshes, st, true, r);
      myFace[b] = 0;
      uint32_t pending = __ballot_sync(0xFFFFFFFFu, mesh >= 0);
      while (pending) {
        const uint32_t leader = __ffs(pending) - 1u;
        const int m = __shfl_sync(0xFFFFFFFFu, mesh, leader);
        const uint32_t group = __ballot_sync(0xFFFFFFFFu, mesh == m) & pending;
        pending &= ~group;
        const uint32_t quads = __ballot_sync(0xFFFFFFFFu, r.quad) & group;
        const uint32_t boxes = group & ~quads;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&sFaces[m], 6u * __popc(boxes) + __popc(quads));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if ((group >> lane) & 1u) myFace[b] = base + faces_below(boxes, quads, lane);
      }
    }
    __syncthreads();
    // 2. One atomic pair per mesh and tile for the global vertex / index space.
    for (uint32_t m = threadIdx.x; m < numMeshes; m += kMeshThreads) {
      const uint32_t faces = sFaces[m];
      if (faces == 0) continue;
      PgaTriangleMesh* M = meshes + m;
      const uint32_t vb = atomicAdd(&M->numVertices, 4u * faces);
      const uint32_t ib = atomicAdd(&M->numIndices, 6u * faces);
      const bool fits = (unsigned long long)vb + 4u * faces <= M->maxNumVertices &&
                        (unsigned long long)ib + 6u * faces <= M->maxNumIndices;
      if (!fits && atomicCAS(&st->status, 0, PGA_ERR_OUTPUT_OVERFLOW) == 0) atomicExch(&st->detail, (int)m);
      sVBase[m] = vb;
      sIBase[m] = ib;
      sFits[m] = fits ? 1u : 0u;
    }
    __syncthreads();
    // 3. Each warp group writes its contiguous run together: 16-byte vertex
    //    pieces and 4-byte indices at consecutive addresses.
#pragma unroll
    for (int b = 0; b < kMeshBatches; b++) {
      const unsigned long long i = tile * tileRecords + (unsigned long long)(warp * kMeshBatches + b) * 32ull + lane;
      Rec r;
      const int mesh = record_mesh(terms, i, n, rules, numEntries, numMeshes, st, false, r);
      uint32_t pending = __ballot_sync(0xFFFFFFFFu, mesh >= 0);
      while (pending) {
        const uint32_t leader = __ffs(pending) - 1u;
        const int m = __shfl_sync(0xFFFFFFFFu, mesh, leader);
        const uint32_t group = __ballot_sync(0xFFFFFFFFu, mesh == m) & pending;
        pending &= ~group;
        if (!sFits[m]) continue;
        const uint32_t quads = __ballot_sync(0xFFFFFFFFu, r.quad) & group;
        const uint32_t boxes = group & ~quads;
        const uint32_t faces = 6u * __popc(boxes) + __popc(quads);
        const uint32_t face0 = __shfl_sync(0xFFFFFFFFu, myFace[b], leader);
        const uint32_t vb = sVBase[m] + 4u * face0, ib = sIBase[m] + 6u * face0;
        float4* vdst = reinterpret_cast<float4*>(meshes[m].vertices + vb);
        uint32_t* idst = meshes[m].indices + ib;
        // Vertices: a lane builds one face (4 vertices, 12 float4) in its
        // warp's shared-memory stage; the warp then copies the stage out with
        // consecutive 16-byte stores.
        float4* stage = sStage[warp];
        for (uint32_t f0 = 0; f0 < faces; f0 += 32u) {
          const uint32_t fi = f0 + lane;  // face of the group
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
            for (int c = 0; c < 3; c++) o.a[a][c] = __shfl_sync(0xFFFFFFFFu, r.a[a][c], owner);
            o.t[a] = __shfl_sync(0xFFFFFFFFu, r.t[a], owner);
          }
          o.quad = __shfl_sync(0xFFFFFFFFu, (int)r.quad, owner) != 0;
          if (fi < faces) {
            const uint32_t f = o.quad ? 0u : fi - faces_below(boxes, quads, owner);
            float v[4][3];
#pragma unroll
            for (uint32_t c = 0; c < 4; c++) corner(o, f, c, v[c]);
            float nrm[3];
            face_normal(v, nrm);
#pragma unroll
            for (uint32_t c = 0; c < 4; c++) {
              const float uvx = (c == 0u || c == 3u) ? 1.0f : 0.0f, uvy = (c <= 1u) ? 1.0f : 0.0f;
              stage[lane * 12u + 3u * c + 0u] = make_float4(v[c][0], v[c][1], v[c][2], 1.0f);
              stage[lane * 12u + 3u * c + 1u] = make_float4(nrm[0], nrm[1], nrm[2], uvx);
              stage[lane * 12u + 3u * c + 2u] = make_float4(uvy, 0.0f, 0.0f, 0.0f);
            }
          }
          __syncwarp();
          const uint32_t pieces = 12u * min(32u, faces - f0);
          for (uint32_t p = lane; p < pieces; p += 32u) __stcs(vdst + 12u * f0 + p, stage[p]);
          __syncwarp();
        }
        // Indices: two triangles per face, (v, v+1, v+2) and (v, v+2, v+3).
        const uint32_t nidx = 6u * faces;
        for (uint32_t s = lane; s < nidx; s += 32u) {
          const uint32_t fi = s / 6u, k = s % 6u;
          const uint32_t off = (k == 0u || k == 3u) ? 0u : (k == 1u ? 1u : (k == 2u || k == 4u) ? 2u : 3u);
          __stcs(idst + s, vb + 4u * fi + off);
        }
      }
    }
    __syncthreads();
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
  if (numMeshes > kMaxMeshes) numMeshes = kMaxMeshes;  // terminal indices are 7 bits
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned long long tiles = (numTerminals + (unsigned long long)kMeshThreads * kMeshBatches - 1) /
                                   ((unsigned long long)kMeshThreads * kMeshBatches);
  const unsigned long long maxBlocks = (unsigned long long)e->numSMs * 6ull;  // resident at 80 registers
  const unsigned blocks = (unsigned)(tiles < maxBlocks ? tiles : maxBlocks);
  k_meshes<<<blocks, kMeshThreads, 0, s>>>(dTerminals, numTerminals, e->dRules, e->numEntries, dMeshes, numMeshes,
                                          e->dState);
  const cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return cuda_status(err, "pga_generate_meshes launch");
  return PGA_OK;
}
