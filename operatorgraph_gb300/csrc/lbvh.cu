// LBVH over terminal boxes: Morton keys, radix sort, Karras topology, refit.
//
// Restates ContextSensitivity::GPU::BVHConstructor::construct
// (include/pga/core/GPUBVHConstructor.cuh:44-331) for the terminal records of
// a derivation, with three changes:
//  * key = morton30 << 34 | path >> 30: equal Morton codes are ordered by the
//    derivation-path hash (ties on those 34 bits resolved on the full hash)
//    instead of the emission index, which depends on queue order;
//  * the Karras codes are morton30 << 32 | sorted position, as the reference's
//    `(code << 32) | j` with j replaced by that deterministic position;
//  * AABBs start from -FLT_MAX instead of FLT_MIN (AABB.cuh:20) and a fence
//    orders each node's AABB store before its parent's arrival counter.
#include <cuda_runtime.h>

#include <cfloat>
#include <cub/device/device_radix_sort.cuh>
#include <mutex>
#include <string>

#include "engine_host.h"

namespace pga {

constexpr int kLbvhThreads = 256;

// spread / morton30 (GPUBVHConstructor.cuh:44-64).
__device__ __forceinline__ uint32_t spread(uint32_t v) {
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

struct Bounds {
  float mn[3];
  float sz[3];
};

// generateMortonCodes (GPUBVHConstructor.cuh:66-86) on terminal centres.
__global__ void __launch_bounds__(kLbvhThreads) k_morton(const PgaTerminal* __restrict__ t, unsigned long long n,
                                                         Bounds b, unsigned long long* __restrict__ keys,
                                                         uint32_t* __restrict__ vals) {
  unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4* p = reinterpret_cast<const float4*>(t + i);
  float4 r0 = __ldg(p + 0), r1 = __ldg(p + 1), r2 = __ldg(p + 2);
  uint4 meta = __ldg(reinterpret_cast<const uint4*>(p + 3));
  float c[3] = {r0.w, r1.w, r2.w};
  uint32_t code = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float nc = __fdiv_rn(__fsub_rn(c[k], b.mn[k]), b.sz[k]);
    code |= spread(__float2uint_rz(__fmul_rn(nc, 1023.0f))) << k;
  }
  uint64_t path = ((uint64_t)meta.w << 32) | meta.z;
  keys[i] = ((unsigned long long)code << 34) | (path >> 30);
  vals[i] = (uint32_t)i;
}

__device__ __forceinline__ uint64_t term_path(const PgaTerminal* t, uint32_t i) {
  const uint2 v = __ldg(reinterpret_cast<const uint2*>(&t[i].path));
  return ((uint64_t)v.y << 32) | v.x;
}

// Orders runs of equal keys by the full path hash (then terminal index).
__global__ void k_fix_ties(const unsigned long long* __restrict__ keys, uint32_t* __restrict__ vals,
                           const PgaTerminal* __restrict__ t, unsigned long long n) {
  unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i + 1 >= n) return;
  unsigned long long k = keys[i];
  if (keys[i + 1] != k || (i > 0 && keys[i - 1] == k)) return;
  unsigned long long j = i + 1;
  while (j < n && keys[j] == k) j++;
  for (unsigned long long a = i + 1; a < j; a++) {
    uint32_t v = vals[a];
    uint64_t pv = term_path(t, v);
    unsigned long long b = a;
    while (b > i) {
      uint32_t u = vals[b - 1];
      uint64_t pu = term_path(t, u);
      if (pu < pv || (pu == pv && u < v)) break;
      vals[b] = u;
      b--;
    }
    vals[b] = v;
  }
}

__device__ __forceinline__ unsigned long long karras_code(const unsigned long long* keys, long long j) {
  return ((keys[j] >> 34) << 32) | (unsigned long long)j;
}

// buildRadixTree (GPUBVHConstructor.cuh:88-213), one thread per internal node,
// with bounds checks on every probe.
__global__ void __launch_bounds__(kLbvhThreads) k_karras(const unsigned long long* __restrict__ keys, long long n,
                                                         int32_t* __restrict__ nodes, uint32_t* __restrict__ leafParents,
                                                         uint32_t* __restrict__ sortedVals, const uint32_t* __restrict__ vals) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sortedVals[i] = vals[i];
  if (i >= n - 1) return;
  const unsigned long long ci = karras_code(keys, i);
  auto delta = [&](long long j) -> int { return __clzll(ci ^ karras_code(keys, j)); };
  long long d, len;
  if (i == 0) {
    d = 1;
    len = n - 1;
  } else {
    int t1 = delta(i - 1), t2 = delta(i + 1);
    int dmin = min(t1, t2);
    d = (t2 - t1 >= 0) ? 1 : -1;
    long long step = 128, j;
    while ((j = i + d * step) >= 0 && j < n && delta(j) > dmin) step <<= 2;
    len = 0;
    for (step >>= 1; step > 0; step >>= 1) {
      j = i + (len + step) * d;
      if (j < 0 || j >= n) continue;
      if (delta(j) > dmin) len += step;
    }
  }
  long long j = i + len * d;
  int dnode = delta(j);
  long long step = 1ll << max(0, 31 - __clz((unsigned)len));
  step >>= (step == len);
  long long s = 0;
  for (; step > 0; step >>= 1) {
    long long k = i + (s + step) * d;
    if (k < 0 || k >= n) continue;
    if (delta(k) > dnode) s += step;
  }
  long long gamma = i + s * d + min(d, 0ll);
  long long left = (min(i, j) == gamma) ? gamma : -gamma;
  long long right = (max(i, j) == gamma + 1) ? (gamma + 1) : -(gamma + 1);
  nodes[i * 3 + 1] = (int32_t)left;
  nodes[i * 3 + 2] = (int32_t)right;
  if (left < 0) nodes[(-left) * 3 + 0] = (int32_t)i;
  else leafParents[left] = (uint32_t)i;
  if (right < 0) nodes[(-right) * 3 + 0] = (int32_t)i;
  else leafParents[right] = (uint32_t)i;
  if (i == 0) nodes[0] = -1;
}

// Leaf AABB: corners of the terminal box (8) or quad (4), as
// BoundingVolumeConstructor<AABB>::construct (BoundingVolumeConstructor.cuh:22-76)
// with the scale folded into the terminal matrix.
__device__ __forceinline__ void leaf_aabb(const PgaTerminal* t, uint32_t idx, float mn[3], float mx[3]) {
  const float4* p = reinterpret_cast<const float4*>(t + idx);
  float4 r[3] = {__ldg(p + 0), __ldg(p + 1), __ldg(p + 2)};
  uint32_t rule = __ldg(reinterpret_cast<const uint32_t*>(p + 3));
  bool quad = (rule >> 31) != 0;
#pragma unroll
  for (int k = 0; k < 3; k++) { mn[k] = FLT_MAX; mx[k] = -FLT_MAX; }
  for (int cz = 0; cz < (quad ? 1 : 2); cz++)
#pragma unroll
    for (int cy = 0; cy < 2; cy++)
#pragma unroll
      for (int cx = 0; cx < 2; cx++) {
        float x = cx ? 0.5f : -0.5f, y = cy ? 0.5f : -0.5f, z = quad ? 0.0f : (cz ? 0.5f : -0.5f);
#pragma unroll
        for (int k = 0; k < 3; k++) {
          float v = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(r[k].x, x), __fmul_rn(r[k].y, y)), __fmul_rn(r[k].z, z)), r[k].w);
          mn[k] = fminf(mn[k], v);
          mx[k] = fmaxf(mx[k], v);
        }
      }
}

// propagateBVH (GPUBVHConstructor.cuh:215-261): the second thread to reach a
// node merges its children and climbs on.
__global__ void __launch_bounds__(kLbvhThreads) k_refit(const PgaTerminal* __restrict__ t, long long n,
                                                        const int32_t* __restrict__ nodes,
                                                        const uint32_t* __restrict__ leafParents,
                                                        const uint32_t* __restrict__ sortedVals,
                                                        uint32_t* __restrict__ arrival, float* __restrict__ aabbs) {
  long long leaf = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (leaf >= n) return;
  long long cur = leafParents[leaf];
  for (long long guard = 0; guard < n; guard++) {
    __threadfence();
    if (atomicAdd(&arrival[cur], 1u) == 0) return;
    __threadfence();
    int32_t l = __ldcg(&nodes[cur * 3 + 1]), r = __ldcg(&nodes[cur * 3 + 2]);
    float amn[3], amx[3], bmn[3], bmx[3];
    if (l < 0) {
      for (int k = 0; k < 3; k++) { amn[k] = __ldcg(&aabbs[(long long)(-l) * 6 + k]); amx[k] = __ldcg(&aabbs[(long long)(-l) * 6 + 3 + k]); }
    } else {
      leaf_aabb(t, sortedVals[l], amn, amx);
    }
    if (r < 0) {
      for (int k = 0; k < 3; k++) { bmn[k] = __ldcg(&aabbs[(long long)(-r) * 6 + k]); bmx[k] = __ldcg(&aabbs[(long long)(-r) * 6 + 3 + k]); }
    } else {
      leaf_aabb(t, sortedVals[r], bmn, bmx);
    }
    for (int k = 0; k < 3; k++) {
      __stcg(&aabbs[cur * 6 + k], fminf(amn[k], bmn[k]));
      __stcg(&aabbs[cur * 6 + 3 + k], fmaxf(amx[k], bmx[k]));
    }
    if (cur == 0) return;
    cur = __ldcg(&nodes[cur * 3 + 0]);
    if (cur < 0) return;
  }
}

}  // namespace pga

using namespace pga;

extern "C" size_t pga_lbvh_temp_bytes(uint64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (uint32_t*)nullptr, (uint32_t*)nullptr, (int64_t)(n ? n : 1), 0, 64);
  return bytes ? bytes : 16;
}

extern "C" PgaStatus pga_lbvh_build(PgaEngine* e, const PgaTerminal* dTerminals, uint64_t n, const PgaBounds* bounds,
                                    const PgaLbvh* out, void* stream) {
  if (!e || !dTerminals || !bounds || !out || !out->nodes || !out->leafParents || !out->aabbs || !out->leafTerminal ||
      !out->keys) {
    set_error("pga_lbvh_build: null argument");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (n < 2 || n > e->cfg.maxTerminals || n > 0x7FFFFFFFull) {
    set_error("pga_lbvh_build: need 2 <= n <= maxTerminals (and < 2^31)");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  Bounds b;
  for (int k = 0; k < 3; k++) {
    b.mn[k] = bounds->min[k];
    b.sz[k] = bounds->max[k] - bounds->min[k];
  }
  unsigned blocks = (unsigned)((n + kLbvhThreads - 1) / kLbvhThreads);
  k_morton<<<blocks, kLbvhThreads, 0, s>>>(dTerminals, n, b, e->dKeysA, e->dValsA);
  PGA_CUDA_TRY(cudaGetLastError());
  size_t temp = e->sortTempBytes;
  PGA_CUDA_TRY(cub::DeviceRadixSort::SortPairs(e->dSortTemp, temp, e->dKeysA, (unsigned long long*)out->keys,
                                               e->dValsA, e->dValsB, (int64_t)n, 0, 64, s));
  k_fix_ties<<<blocks, kLbvhThreads, 0, s>>>((const unsigned long long*)out->keys, e->dValsB, dTerminals, n);
  PGA_CUDA_TRY(cudaGetLastError());
  k_karras<<<blocks, kLbvhThreads, 0, s>>>((const unsigned long long*)out->keys, (long long)n, out->nodes,
                                           out->leafParents, out->leafTerminal, e->dValsB);
  PGA_CUDA_TRY(cudaGetLastError());
  PGA_CUDA_TRY(cudaMemsetAsync(e->dArrival, 0, (n - 1) * sizeof(uint32_t), s));
  k_refit<<<blocks, kLbvhThreads, 0, s>>>(dTerminals, (long long)n, out->nodes, out->leafParents, out->leafTerminal,
                                          e->dArrival, out->aabbs);
  PGA_CUDA_TRY(cudaGetLastError());
  return PGA_OK;
}

// ---------------------------------------------------------------------------
// pga_lbvh_build_static: the same LBVH build with every piece of scratch taken
// from one fixed device array of this file instead of an engine's buffers.
//
// Some callers cannot allocate device memory when they build a hierarchy: a
// host process whose device-memory budget was handed out in full at start-up,
// a plug-in running inside an application that owns the allocator, or code
// that must not hit the driver's allocator inside a latency-critical loop.
// They pass only their inputs and outputs; the scratch lives in
// g_lbvhStaticScratch, which every GPU that loads this library holds until
// the process exits.
//
// The array's name denotes a host-side stand-in in host code, not a device
// address, so the device address is looked up once per device with
// cudaGetSymbolAddress (with that device current) on the first call made on
// it; make that first call before any stream capture.  All calls share the
// array and it keeps the last call's contents: the arrival counters that must
// start at zero are cleared on every call, and calls that overlap on the GPU
// (on different streams, or from different threads) race on it.

namespace pga {

constexpr size_t kStaticScratchBytes = 6u << 20;  // 6 MiB
static __device__ __align__(256) unsigned char g_lbvhStaticScratch[kStaticScratchBytes];

static std::mutex g_staticMutex;
static void* g_staticAddr[64];  // device address of g_lbvhStaticScratch per device ordinal

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace pga

extern "C" PgaStatus pga_lbvh_build_static(const PgaTerminal* dTerminals, uint64_t n, const PgaBounds* bounds,
                                           const PgaLbvh* out, void* stream) {
  if (!dTerminals || !bounds || !out || !out->nodes || !out->leafParents || !out->aabbs || !out->leafTerminal ||
      !out->keys) {
    set_error("pga_lbvh_build_static: null argument");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (n < 2 || n > PGA_LBVH_STATIC_MAX_LEAVES) {
    set_error("pga_lbvh_build_static: n must be in [2, " + std::to_string(PGA_LBVH_STATIC_MAX_LEAVES) +
              "] (the fixed scratch holds at most that many leaves); use pga_lbvh_build for larger sets");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  int dev = 0;
  PGA_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("pga_lbvh_build_static: device ordinal out of range");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  unsigned char* base = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_staticMutex);
    if (!g_staticAddr[dev]) {
      void* p = nullptr;
      cudaError_t err = cudaGetSymbolAddress(&p, g_lbvhStaticScratch);
      if (err != cudaSuccess) return cuda_status(err, "pga_lbvh_build_static: cudaGetSymbolAddress");
      g_staticAddr[dev] = p;
    }
    base = static_cast<unsigned char*>(g_staticAddr[dev]);
  }
  // Carve the scratch: keys, two value arrays, arrival counters, sort temp.
  size_t temp = pga_lbvh_temp_bytes(n);
  size_t off = 0;
  unsigned long long* keysA = reinterpret_cast<unsigned long long*>(base + off);
  off += align256(n * sizeof(unsigned long long));
  uint32_t* valsA = reinterpret_cast<uint32_t*>(base + off);
  off += align256(n * sizeof(uint32_t));
  uint32_t* valsB = reinterpret_cast<uint32_t*>(base + off);
  off += align256(n * sizeof(uint32_t));
  uint32_t* arrival = reinterpret_cast<uint32_t*>(base + off);
  off += align256(n * sizeof(uint32_t));
  void* sortTemp = base + off;
  off += align256(temp);
  if (off > kStaticScratchBytes) {
    set_error("pga_lbvh_build_static: fixed scratch too small for the radix sort of " + std::to_string(n) + " keys");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  Bounds b;
  for (int k = 0; k < 3; k++) {
    b.mn[k] = bounds->min[k];
    b.sz[k] = bounds->max[k] - bounds->min[k];
  }
  const unsigned blocks = (unsigned)((n + kLbvhThreads - 1) / kLbvhThreads);
  k_morton<<<blocks, kLbvhThreads, 0, s>>>(dTerminals, n, b, keysA, valsA);
  PGA_CUDA_TRY(cudaGetLastError());
  PGA_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sortTemp, temp, keysA, (unsigned long long*)out->keys, valsA, valsB,
                                               (int64_t)n, 0, 64, s));
  k_fix_ties<<<blocks, kLbvhThreads, 0, s>>>((const unsigned long long*)out->keys, valsB, dTerminals, n);
  PGA_CUDA_TRY(cudaGetLastError());
  k_karras<<<blocks, kLbvhThreads, 0, s>>>((const unsigned long long*)out->keys, (long long)n, out->nodes,
                                           out->leafParents, out->leafTerminal, valsB);
  PGA_CUDA_TRY(cudaGetLastError());
  PGA_CUDA_TRY(cudaMemsetAsync(arrival, 0, (n - 1) * sizeof(uint32_t), s));
  k_refit<<<blocks, kLbvhThreads, 0, s>>>(dTerminals, (long long)n, out->nodes, out->leafParents, out->leafTerminal,
                                          arrival, out->aabbs);
  PGA_CUDA_TRY(cudaGetLastError());
  return PGA_OK;
}
