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
// The reference sorts with thrust::sort (GPUBVHConstructor.cuh:311-312); here
// the sort is this file's own onesweep radix sort (see k_onesweep).
#include <cuda_runtime.h>

#include <cfloat>
#include <algorithm>
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

// Leaf AABB: corners of the terminal box (8) or quad (4), as
// BoundingVolumeConstructor<AABB>::construct (BoundingVolumeConstructor.cuh:22-76)
// with the scale folded into the terminal matrix.
__device__ __forceinline__ void leaf_aabb(const float4 r[3], bool quad, float mn[3], float mx[3]) {
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

// Leaf count of a build: the host value `n`, or, when the count lives on the
// device (dN != nullptr), min(*dN, n) with `n` the capacity the launches and
// the sort were sized for.
__device__ __forceinline__ unsigned long long leaf_count(const unsigned long long* dN, unsigned long long n) {
  return dN ? min(*dN, n) : n;
}

// The radix sort orders the keys' top bits [kSortLowBit, 64) only (the Morton
// code and the path hash's top 10 bits): four passes of 10-bit digits.
constexpr int kSortLowBit = 24;
constexpr int kRadixBits = 10;
constexpr uint32_t kBins = 1u << kRadixBits;
constexpr int kSortPasses = (64 - kSortLowBit) / kRadixBits;
static_assert(kSortLowBit + kSortPasses * kRadixBits == 64, "the passes cover bits [kSortLowBit, 64)");

// Histogram of one digit of a warp's 32 keys into shared memory: one add for
// the whole warp when every lane has the same digit (the Morton code's high
// digits, for neighbouring terminals), else one add per lane.
__device__ __forceinline__ void hist_add(uint32_t* h, uint32_t d, bool valid) {
  const uint32_t d0 = __shfl_sync(0xFFFFFFFFu, d, 0);
  const unsigned same = __ballot_sync(0xFFFFFFFFu, valid && d == d0);
  if (same == 0xFFFFFFFFu) {
    if ((threadIdx.x & 31u) == 0) atomicAdd(h + d0, 32u);
  } else if (valid) {
    atomicAdd(h + d, 1u);
  }
}

// generateMortonCodes (GPUBVHConstructor.cuh:66-86) on terminal centres.
// Also writes each terminal's AABB (6 floats, terminal order) while its record
// is in registers.  The sort's values start as the terminal index, which its
// first pass generates, so none are written here.
// With a device count, the keys in [count, capacity) are padding: all ones,
// after every real key in the stable radix sort (a real key can equal it only
// in the sorted top bits, and it comes first there by input order).
__global__ void __launch_bounds__(kLbvhThreads) k_morton(const PgaTerminal* __restrict__ t, unsigned long long cap,
                                                         const unsigned long long* __restrict__ dN, Bounds b,
                                                         unsigned long long* __restrict__ keys,
                                                         float* __restrict__ leafBox) {
  unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap) return;
  if (i >= leaf_count(dN, cap)) {
    keys[i] = ~0ull;
    return;
  }
  const float4* p = reinterpret_cast<const float4*>(t + i);
  float4 r[3] = {__ldg(p + 0), __ldg(p + 1), __ldg(p + 2)};
  uint4 meta = __ldg(reinterpret_cast<const uint4*>(p + 3));
  float mn[3], mx[3];
  leaf_aabb(r, (meta.x >> 31) != 0, mn, mx);
  float2* lb = reinterpret_cast<float2*>(leafBox + i * 6);
  lb[0] = make_float2(mn[0], mn[1]);
  lb[1] = make_float2(mn[2], mx[0]);
  lb[2] = make_float2(mx[1], mx[2]);
  float c[3] = {r[0].w, r[1].w, r[2].w};
  uint32_t code = 0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float nc = __fdiv_rn(__fsub_rn(c[k], b.mn[k]), b.sz[k]);
    code |= spread(__float2uint_rz(__fmul_rn(nc, 1023.0f))) << k;
  }
  uint64_t path = ((uint64_t)meta.w << 32) | meta.z;
  keys[i] = ((unsigned long long)code << 34) | (path >> 30);
}

// The four digit histograms of keys [0, n) (kSortPasses x kBins, zeroed
// before the launch): each block counts a contiguous run of keys into shared
// memory, kHistUnroll keys per thread in flight, then adds its nonzero bins.
constexpr int kHistThreads = 512;
constexpr int kHistUnroll = 4;
__global__ void __launch_bounds__(kHistThreads) k_digit_hist(const unsigned long long* __restrict__ keys,
                                                             unsigned long long n, uint32_t* __restrict__ hist) {
  __shared__ uint32_t sh[kSortPasses * kBins];
  for (uint32_t k = threadIdx.x; k < kSortPasses * kBins; k += kHistThreads) sh[k] = 0u;
  __syncthreads();
  const unsigned long long per = (n + gridDim.x - 1) / gridDim.x;
  const unsigned long long lo = min(n, (unsigned long long)blockIdx.x * per), hi = min(n, lo + per);
  // every lane of a warp runs the same iterations (hist_add is warp-wide)
  for (unsigned long long i0 = lo; i0 < hi; i0 += (unsigned long long)kHistThreads * kHistUnroll) {
    unsigned long long key[kHistUnroll];
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) {
      const unsigned long long i = i0 + (unsigned long long)u * kHistThreads + threadIdx.x;
      key[u] = i < hi ? __ldcs(keys + i) : 0ull;
    }
#pragma unroll
    for (int u = 0; u < kHistUnroll; u++) {
      const bool valid = i0 + (unsigned long long)u * kHistThreads + threadIdx.x < hi;
#pragma unroll
      for (int q = 0; q < kSortPasses; q++)
        hist_add(sh + q * kBins, (uint32_t)(key[u] >> (kSortLowBit + q * kRadixBits)) & (kBins - 1u), valid);
    }
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < kSortPasses * kBins; k += kHistThreads)
    if (sh[k] != 0u) atomicAdd(hist + k, sh[k]);
}

// Exclusive scans of the four digit histograms: gBase[q][d] = where digit d's
// keys start in pass q's output.  One block of kBins threads.
__global__ void __launch_bounds__(kBins) k_sort_bases(const uint32_t* __restrict__ hist, uint32_t* __restrict__ gBase) {
  __shared__ uint32_t warpSum[kBins / 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (int q = 0; q < kSortPasses; q++) {
    const uint32_t v = hist[q * kBins + threadIdx.x];
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= (uint32_t)d) x += y;
    }
    if (lane == 31) warpSum[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) before += warpSum[w];
    gBase[q * kBins + threadIdx.x] = before + x - v;
    __syncthreads();
  }
}

// One pass of the radix sort ("onesweep", Adinets & Merrill 2022), stable:
// keys and values of [0, n) ordered by digit (key >> shift) & (kBins - 1).
// A block takes the next tile of kSortTile keys from an atomic counter, so a
// tile's predecessors were taken by blocks that started earlier.  Its warps
// rank their keys by digit in input order (warp-private 16-bit histograms;
// the lanes sharing a digit found with one ballot per digit bit) and the tile
// goes to shared memory in digit order.  Thread t owns bins 2t and 2t + 1 and
// publishes their counts as one 64-bit word (each half carries the flag), so
// one walk serves both bins: decoupled look-back over the earlier tiles'
// words until one carries an inclusive prefix.  Keys then go out in
// contiguous runs per digit.  valsIn == nullptr means the identity (value =
// index).  A look-back wait gives up after spinLimit polls, raising
// PGA_ERR_TIMEOUT in *err (the order is then unspecified).
constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 10;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;
constexpr uint32_t kHistStride = kBins + 16;  // u16 per warp histogram; bin kBins counts keys past n
constexpr uint32_t kFlagAggregate = 1u << 30, kFlagPrefix = 2u << 30, kCountMask = (1u << 30) - 1u;
constexpr int kLookback = 16;  // predecessor words loaded at once by a look-back step
static_assert(kBins == 2 * kSortThreads, "each thread owns two bins");
constexpr size_t kOnesweepSmem =
    (size_t)kSortTile * 8 + (size_t)kSortTile * 4 + (size_t)kSortWarps * kHistStride * 2 + (size_t)kBins * 8;

__device__ __forceinline__ void st_relaxed64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long pair_word(uint32_t flag, uint32_t c0, uint32_t c1) {
  return ((unsigned long long)(flag | c1) << 32) | (flag | c0);
}

__global__ void __launch_bounds__(kSortThreads, 2)
    k_onesweep(const unsigned long long* __restrict__ keysIn, const uint32_t* __restrict__ valsIn,
               unsigned long long* __restrict__ keysOut, uint32_t* __restrict__ valsOut, unsigned long long n,
               uint32_t shift, const uint32_t* __restrict__ gBase, unsigned long long* status,
               uint32_t* tileCounter, int* err, uint32_t spinLimit) {
  extern __shared__ __align__(16) unsigned char smem_sort[];
  unsigned long long* sKeys = reinterpret_cast<unsigned long long*>(smem_sort);
  uint32_t* sVals = reinterpret_cast<uint32_t*>(sKeys + kSortTile);
  uint16_t* sHist = reinterpret_cast<uint16_t*>(sVals + kSortTile);
  uint32_t* sStart = reinterpret_cast<uint32_t*>(sHist + kSortWarps * kHistStride);
  int32_t* sDst = reinterpret_cast<int32_t*>(sStart + kBins);
  __shared__ uint32_t sTile;
  __shared__ uint32_t sWarpSum[kSortWarps];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) sTile = atomicAdd(tileCounter, 1u);
  uint16_t* hist = sHist + warp * kHistStride;
  for (uint32_t k = lane; k < kHistStride / 2; k += 32) reinterpret_cast<uint32_t*>(hist)[k] = 0u;
  __syncthreads();
  const uint32_t tile = sTile;
  const unsigned long long tileBase = (unsigned long long)tile * kSortTile;
  const unsigned long long warpBase = tileBase + (unsigned long long)warp * (32u * kSortItems);
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  unsigned long long key[kSortItems];
  uint32_t val[kSortItems];
  uint32_t rank[kSortItems];
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const unsigned long long i = warpBase + (unsigned)k * 32u + lane;
    key[k] = i < n ? __ldcs(keysIn + i) : 0ull;
    val[k] = valsIn == nullptr ? (uint32_t)i : (i < n ? __ldcs(valsIn + i) : 0u);
  }
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const unsigned long long i = warpBase + (unsigned)k * 32u + lane;
    const bool valid = i < n;
    const uint32_t d = valid ? (uint32_t)(key[k] >> shift) & (kBins - 1u) : kBins;
    // the lanes with the same digit (and validity): one ballot per digit bit
    unsigned peers = __ballot_sync(0xFFFFFFFFu, valid);
    if (!valid) peers = ~peers;
#pragma unroll
    for (int bit = 0; bit < kRadixBits; bit++) {
      const unsigned on = __ballot_sync(0xFFFFFFFFu, (d >> bit) & 1u);
      peers &= ((d >> bit) & 1u) ? on : ~on;
    }
    const int leader = __ffs(peers) - 1;
    uint32_t old = 0;
    if ((int)lane == leader) {
      old = hist[d];
      hist[d] = (uint16_t)(old + __popc(peers));
    }
    old = __shfl_sync(0xFFFFFFFFu, old, leader);
    rank[k] = old + __popc(peers & lt);
    __syncwarp();
  }
  __syncthreads();
  // Thread t owns bins 2t and 2t + 1: the warps' exclusive prefixes in place,
  // the tile's count of each bin, published for the later tiles.
  uint32_t tot[2];
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const uint32_t d = 2u * threadIdx.x + q;
    uint32_t run = 0;
    for (int w = 0; w < kSortWarps; w++) {
      uint16_t* h = sHist + w * kHistStride;
      const uint32_t c = h[d];
      h[d] = (uint16_t)run;
      run += c;
    }
    tot[q] = run;
  }
  unsigned long long* st = status + (size_t)tile * (kBins / 2) + threadIdx.x;
  st_relaxed64(st, pair_word(tile == 0 ? kFlagPrefix : kFlagAggregate, tot[0], tot[1]));
  // The tile's bin starts: an exclusive scan of the bins in order.
  {
    const uint32_t v = tot[0] + tot[1];
    uint32_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= (uint32_t)d) x += y;
    }
    if (lane == 31) sWarpSum[warp] = x;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) before += sWarpSum[w];
    sStart[2u * threadIdx.x] = before + x - v;
    sStart[2u * threadIdx.x + 1] = before + x - v + tot[0];
  }
  __syncthreads();
  // The tile in digit order in shared memory (before the look-back: it needs
  // only the tile's own counts).
#pragma unroll
  for (int k = 0; k < kSortItems; k++) {
    const unsigned long long i = warpBase + (unsigned)k * 32u + lane;
    if (i < n) {
      const uint32_t d = (uint32_t)(key[k] >> shift) & (kBins - 1u);
      const uint32_t pos = sStart[d] + hist[d] + rank[k];
      sKeys[pos] = key[k];
      sVals[pos] = val[k];
    }
  }
  // Decoupled look-back: both bins' counts over the earlier tiles.  The words
  // of kLookback predecessors are loaded at once (independent loads), then
  // summed nearest first up to the first inclusive prefix; a word not yet
  // published stops the sum there and is polled again.
  uint32_t prefix0 = 0, prefix1 = 0;
  if (tile > 0) {
    long long p = (long long)tile - 1;
    uint32_t spins = 0;
    while (p >= 0) {
      unsigned long long w[kLookback];
#pragma unroll
      for (int k = 0; k < kLookback; k++)
        w[k] = p - k >= 0 ? ld_relaxed64(status + (size_t)(p - k) * (kBins / 2) + threadIdx.x)
                          : pair_word(kFlagPrefix, 0u, 0u);
      int used = 0;
      bool done = false, stalled = false;
#pragma unroll
      for (int k = 0; k < kLookback; k++) {
        if (done || stalled) continue;
        const uint32_t lo = (uint32_t)w[k], hi = (uint32_t)(w[k] >> 32);
        if ((lo >> 30) == 0u) {
          stalled = true;
          continue;
        }
        prefix0 += lo & kCountMask;
        prefix1 += hi & kCountMask;
        used++;
        if ((lo & kFlagPrefix) != 0u) done = true;
      }
      if (done) break;
      p -= used;
      if (stalled) {
        if (++spins > spinLimit) {
          atomicCAS(err, 0, (int)PGA_ERR_TIMEOUT);
          break;
        }
        __nanosleep(32);
      }
    }
    st_relaxed64(st, pair_word(kFlagPrefix, prefix0 + tot[0], prefix1 + tot[1]));
  }
  sDst[2u * threadIdx.x] = (int32_t)(__ldg(gBase + 2u * threadIdx.x) + prefix0);
  sDst[2u * threadIdx.x + 1] = (int32_t)(__ldg(gBase + 2u * threadIdx.x + 1) + prefix1);
  __syncthreads();
  // Out: consecutive positions of one digit go to consecutive places.
  const uint32_t count = (uint32_t)min((unsigned long long)kSortTile, n - tileBase);
  for (uint32_t p = threadIdx.x; p < count; p += kSortThreads) {
    const unsigned long long kk = sKeys[p];
    const uint32_t d = (uint32_t)(kk >> shift) & (kBins - 1u);
    const long long o = (long long)sDst[d] + (long long)(p - sStart[d]);
    if (o < 0 || (unsigned long long)o >= n) continue;  // only after a look-back that gave up
    keysOut[o] = kk;
    valsOut[o] = sVals[p];
  }
}

__device__ __forceinline__ uint64_t term_path(const PgaTerminal* t, uint32_t i) {
  const uint2 v = __ldg(reinterpret_cast<const uint2*>(&t[i].path));
  return ((uint64_t)v.y << 32) | v.x;
}

// The radix sort orders the keys' top bits [kSortLowBit, 64) only, which
// leaves runs of equal top bits in input order (terminals in one Morton cell
// whose path hashes share their top 10 bits: short runs, but about half of
// the keys of a crowded scene lie in one).  The final order inside a run is
// by the whole key (the Morton code and the path hash's top 34 bits), then,
// for equal keys, by the full path hash, then by terminal index:
// lexicographic in (Morton code, path hash, terminal), the order a full
// 64-bit sort plus tie fix gives.  Each member of a run counts the members
// that come before it and writes its key and value at run start + that count
// into tieKeys / tieVals; one bit per position in tieMask marks the members.
// The Karras pass takes a marked position's value from tieVals and the refit
// writes its key from tieKeys, so the keys' top bits, all the Karras codes
// read, do not change while a later kernel reads them.
//
// A warp ranks its 32 keys inside a window of kTieReach keys either side
// (lane l holds window positions l and 32 + l): run boundaries from two
// ballots of "equal to the left neighbour", and each member compares the low
// 32 bits of its key (the rest is equal inside a run) with those of its run's
// members, staged in shared memory.  A run that reaches the window's edge, or
// that holds equal keys (then the paths decide), is ranked by the member
// alone in global memory, reading a terminal record only for equal keys.
constexpr int kTieReach = 16;
__device__ __noinline__ void tie_rank_global(const unsigned long long* __restrict__ keys,
                                             const uint32_t* __restrict__ vals, const PgaTerminal* __restrict__ t,
                                             unsigned long long n, unsigned long long i,
                                             unsigned long long* __restrict__ tieKeys,
                                             uint32_t* __restrict__ tieVals) {
  const unsigned long long ki = keys[i], k = ki >> kSortLowBit;
  unsigned long long s = i, e = i + 1;
  while (s > 0 && (keys[s - 1] >> kSortLowBit) == k) s--;
  while (e < n && (keys[e] >> kSortLowBit) == k) e++;
  const uint32_t vi = vals[i];
  bool havePath = false;
  uint64_t pi = 0;
  unsigned long long before = 0;
  for (unsigned long long b = s; b < e; b++) {
    const unsigned long long kb = keys[b];
    if (kb != ki) {
      before += kb < ki;
    } else if (b != i) {
      if (!havePath) {
        pi = term_path(t, vi);
        havePath = true;
      }
      const uint32_t vb = vals[b];
      const uint64_t pb = term_path(t, vb);
      before += pb < pi || (pb == pi && vb < vi);
    }
  }
  tieKeys[s + before] = ki;
  tieVals[s + before] = vi;
}

__global__ void __launch_bounds__(kLbvhThreads) k_tie_rank(const unsigned long long* __restrict__ keys,
                                                           const uint32_t* __restrict__ vals,
                                                           const PgaTerminal* __restrict__ t, unsigned long long cap,
                                                           const unsigned long long* __restrict__ dN,
                                                           unsigned long long* __restrict__ tieKeys,
                                                           uint32_t* __restrict__ tieVals,
                                                           uint32_t* __restrict__ tieMask) {
  constexpr unsigned kAll = 0xFFFFFFFFu;
  __shared__ uint32_t sWin[kLbvhThreads / 32 * 64];
  const long long n = (long long)leaf_count(dN, cap);
  const int lane = (int)(threadIdx.x & 31u);
  const long long w0 = ((long long)blockIdx.x * kLbvhThreads + threadIdx.x) & ~31ll;
  if (w0 >= n) return;  // the whole warp
  // window position q <-> key w0 - kTieReach + q; lane holds q = lane (a) and q = 32 + lane (b)
  const long long ga = w0 - kTieReach + lane, gb = ga + 32;
  const bool va = ga >= 0 && ga < n, vb = gb < n;
  const unsigned long long ka = va ? keys[ga] : 0ull, kb = vb ? keys[gb] : 0ull;
  const unsigned long long ta = ka >> kSortLowBit, tb = kb >> kSortLowBit;
  // left neighbours: a's is lane - 1's a; b's is lane - 1's b, lane 0's is lane 31's a
  const unsigned long long la = __shfl_up_sync(kAll, ta, 1);
  const int lva = __shfl_up_sync(kAll, (int)va, 1);
  const int src = (lane + 31) & 31;
  const unsigned long long lb = __shfl_sync(kAll, lane == 31 ? ta : tb, src);
  const int lvb = __shfl_sync(kAll, lane == 31 ? (int)va : (int)vb, src);
  const bool eqa = lane > 0 && va && lva && la == ta;
  const bool eqb = vb && lvb && lb == tb;
  const unsigned long long eq = (unsigned long long)__ballot_sync(kAll, eqa) |
                                ((unsigned long long)__ballot_sync(kAll, eqb) << 32);
  // this lane's key sits at window position p (eq bit q: q and q - 1 in one run)
  const int p = kTieReach + lane;
  const long long i = w0 + lane;
  const bool inRun = i < n && (((eq >> p) & 1ull) || ((eq >> (p + 1)) & 1ull));
  const unsigned members = __ballot_sync(kAll, inRun);
  if (lane == 0) tieMask[w0 >> 5] = members;
  if (members == 0u) return;  // the whole warp
  const unsigned long long upto = (2ull << p) - 1ull;  // positions [0, p]
  const int s = 63 - __clzll(~eq & upto);              // eq bit 0 is clear: the run's first position
  const unsigned long long past = ~eq & ~upto;
  const int e = past ? __ffsll((long long)past) - 2 : 63;  // the run's last position
  const bool inWindow = inRun && s > 0 && e < 63;
  // the window's low key halves in this warp's slice of shared memory
  uint32_t* win = sWin + (threadIdx.x >> 5) * 64;
  win[lane] = (uint32_t)ka;
  win[32 + lane] = (uint32_t)kb;
  __syncwarp();
  uint32_t before = 0;
  bool equal = false;
  if (inWindow) {
    const uint32_t li = win[p];
    for (int q = s; q <= e; q++) {
      const uint32_t v = win[q];
      before += v < li;
      equal |= v == li && q != p;
    }
  }
  if (!inRun) return;
  if (inWindow && !equal) {
    const long long dst = w0 - kTieReach + s + (long long)before;
    tieKeys[dst] = keys[i];
    tieVals[dst] = vals[i];
  } else {
    tie_rank_global(keys, vals, t, (unsigned long long)n, (unsigned long long)i, tieKeys, tieVals);
  }
}

__device__ __forceinline__ bool tie_member(const uint32_t* tieMask, unsigned long long i) {
  return (__ldg(tieMask + (i >> 5)) >> (i & 31u)) & 1u;
}

__device__ __forceinline__ unsigned long long karras_code(const unsigned long long* keys, long long j) {
  return ((keys[j] >> 34) << 32) | (unsigned long long)j;
}

// buildRadixTree (GPUBVHConstructor.cuh:88-213), one thread per internal node,
// with bounds checks on every probe.
// Also gathers the leaves' terminal indices (a tie-run member's from
// tieVals) and boxes into sorted order (one independent load per leaf here
// instead of a dependent one ahead of the refit's climb), writes the other
// end of each node's leaf range (one end is the node's own index) and clears
// the refit's arrival counters.  Fewer than two leaves make no tree.
__global__ void __launch_bounds__(kLbvhThreads) k_karras(const unsigned long long* __restrict__ keys, long long cap,
                                                         const unsigned long long* __restrict__ dN,
                                                         int32_t* __restrict__ nodes, uint32_t* __restrict__ leafParents,
                                                         uint32_t* __restrict__ sortedVals, const uint32_t* __restrict__ vals,
                                                         const uint32_t* __restrict__ tieMask,
                                                         const uint32_t* __restrict__ tieVals,
                                                         const float* __restrict__ leafBox,
                                                         float* __restrict__ sortedBox,
                                                         int32_t* __restrict__ nodeOther, uint32_t* __restrict__ arrival) {
  const long long n = (long long)leaf_count(dN, (unsigned long long)cap);
  if (n < 2) return;
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t v = tie_member(tieMask, (unsigned long long)i) ? tieVals[i] : vals[i];
    sortedVals[i] = v;
    const float2* src = reinterpret_cast<const float2*>(leafBox + (size_t)v * 6);
    float2* dst = reinterpret_cast<float2*>(sortedBox + (size_t)i * 6);
    const float2 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2);
    dst[0] = a;
    dst[1] = b;
    dst[2] = c;
  }
  if (i >= n - 1) return;
  arrival[i] = 0u;
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
  nodeOther[i] = (int32_t)j;
}

// Arrival counter bump at GPU scope with only the ordering the step needs.
// A climber publishes a box through memory only when it comes from an
// internal node (it stored that node's box itself): release.  A climber that
// goes on reads its sibling's box through memory only when the sibling is an
// internal node (stored by another thread): acquire.  Leaf boxes come from an
// earlier kernel and need neither, so a step between two leaves is relaxed.
__device__ __forceinline__ uint32_t arrive(uint32_t* p, bool release, bool acquire) {
  uint32_t old;
  if (release && acquire)
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  else if (release)
    asm volatile("atom.release.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  else if (acquire)
    asm volatile("atom.acquire.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  else
    asm volatile("atom.relaxed.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
  return old;
}

// The same for a node whose two climbers are threads of one block: the
// counter and the boxes live in shared memory, ordered at block scope.
__device__ __forceinline__ uint32_t arrive_block(uint32_t* p) {
  uint32_t old;
  asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;"
               : "=r"(old)
               : "r"((uint32_t)__cvta_generic_to_shared(p))
               : "memory");
  return old;
}

__device__ __forceinline__ void load_box(const float* p, float mn[3], float mx[3]) {
  const float2* q = reinterpret_cast<const float2*>(p);
  const float2 a = __ldcg(q), b = __ldcg(q + 1), c = __ldcg(q + 2);
  mn[0] = a.x; mn[1] = a.y; mn[2] = b.x; mx[0] = b.y; mx[1] = c.x; mx[2] = c.y;
}

// propagateBVH (GPUBVHConstructor.cuh:215-261): one thread per leaf climbs;
// the second thread to reach a node merges its children and goes on.  The
// climber keeps the box of the child it comes from in registers and reads
// only the sibling's; the union is min/max(left, right) in that order.
//
// Two kernels.  In k_refit_local thread j handles sorted leaf j, so a block
// holds leaves [B, B + 256).  Its threads first stage their leaves' boxes and
// the records of internal nodes [B, B + 256) (links and the other end of the
// leaf range) in shared memory: one round of independent, coalesced loads.
// A node whose leaf range lies inside [B, B + 256) is reached only by threads
// of the block: its arrival counter and box sit in shared memory (index
// node - B; a Karras node's index is one end of its range) with block-scope
// ordering.  A climber that reaches a node whose range crosses the block's
// boundary (a few percent of the nodes; all their ancestors cross too) stops
// there and queues the child it comes from.  k_refit_global then carries the
// queued climbers up through those nodes with arrival counters at GPU scope,
// so no block of the first kernel waits on a long climb to the root.  Every
// node's box is also stored to aabbs, the output.  Each leaf's thread also
// writes the final key of a tie-run member.
__device__ __forceinline__ void load_box_ldg(const float* __restrict__ p, float mn[3], float mx[3]) {
  const float2* q = reinterpret_cast<const float2*>(p);
  const float2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  mn[0] = a.x; mn[1] = a.y; mn[2] = b.x; mx[0] = b.y; mx[1] = c.x; mx[2] = c.y;
}

__device__ __forceinline__ void store_box(float* p, const float mn[3], const float mx[3]) {
  float2* o = reinterpret_cast<float2*>(p);
  __stcg(o + 0, make_float2(mn[0], mn[1]));
  __stcg(o + 1, make_float2(mn[2], mx[0]));
  __stcg(o + 2, make_float2(mx[1], mx[2]));
}

// The union in (left, right) order of the climber's box (mn, mx; from the
// left child when fromLeft) and its sibling's.
__device__ __forceinline__ void merge_box(bool fromLeft, float mn[3], float mx[3], const float smn[3],
                                          const float smx[3]) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float lmn = fromLeft ? mn[k] : smn[k], rmn = fromLeft ? smn[k] : mn[k];
    const float lmx = fromLeft ? mx[k] : smx[k], rmx = fromLeft ? smx[k] : mx[k];
    mn[k] = fminf(lmn, rmn);
    mx[k] = fmaxf(lmx, rmx);
  }
}

__global__ void __launch_bounds__(kLbvhThreads) k_refit_local(const float* __restrict__ sortedBox, long long cap,
                                                              const unsigned long long* __restrict__ dN,
                                                              const int32_t* __restrict__ nodes,
                                                              const int32_t* __restrict__ nodeOther,
                                                              const uint32_t* __restrict__ leafParents,
                                                              float* __restrict__ aabbs,
                                                              int32_t* __restrict__ queue, uint32_t* __restrict__ queued,
                                                              const uint32_t* __restrict__ tieMask,
                                                              const unsigned long long* __restrict__ tieKeys,
                                                              unsigned long long* __restrict__ keys) {
  __shared__ uint32_t blockArrive[kLbvhThreads];
  __shared__ float blockBox[kLbvhThreads * 6];  // internal nodes [B, E)
  __shared__ float sLeafBox[kLbvhThreads * 6];  // leaves [B, E)
  __shared__ int4 sNode[kLbvhThreads];          // internal nodes [B, E): parent, left, right, other end
  const long long n = (long long)leaf_count(dN, (unsigned long long)cap);
  if (n < 2) return;
  const long long B = (long long)blockIdx.x * kLbvhThreads;
  if (B >= n) return;  // the whole block
  const long long E = min(B + kLbvhThreads, n);
  const long long leaf = B + threadIdx.x;
  blockArrive[threadIdx.x] = 0u;
  float mn[3], mx[3];
  long long cur = -1;
  if (leaf < n) {
    if (tie_member(tieMask, (unsigned long long)leaf)) keys[leaf] = tieKeys[leaf];
    load_box_ldg(sortedBox + (size_t)leaf * 6, mn, mx);
    float* q = &sLeafBox[threadIdx.x * 6];
    q[0] = mn[0]; q[1] = mn[1]; q[2] = mn[2]; q[3] = mx[0]; q[4] = mx[1]; q[5] = mx[2];
    cur = __ldg(leafParents + leaf);
  }
  if (leaf < n - 1)
    sNode[threadIdx.x] = make_int4(__ldg(nodes + leaf * 3 + 0), __ldg(nodes + leaf * 3 + 1),
                                   __ldg(nodes + leaf * 3 + 2), __ldg(nodeOther + leaf));
  __syncthreads();
  if (leaf >= n) return;
  int32_t from = (int32_t)leaf;  // child id as the node table stores it: leaf j -> j, internal k -> -k
  for (int level = 0; level < kLbvhThreads; level++) {
    bool local = cur >= B && cur < E;
    int4 rec = make_int4(0, 0, 0, 0);
    if (local) {
      rec = sNode[cur - B];
      local = min(cur, (long long)rec.w) >= B && max(cur, (long long)rec.w) < E;
    }
    if (!local) {  // the node's range crosses the block's boundary: k_refit_global goes on from here
      queue[atomicAdd(queued, 1u)] = from;
      return;
    }
    if (arrive_block(&blockArrive[cur - B]) == 0) return;
    const bool fromLeft = rec.y == from;
    const int32_t sib = fromLeft ? rec.z : rec.y;  // inside [B, E): the node is local
    const float* q = sib >= 0 ? &sLeafBox[(sib - B) * 6] : &blockBox[(-(long long)sib - B) * 6];
    const float smn[3] = {q[0], q[1], q[2]}, smx[3] = {q[3], q[4], q[5]};
    merge_box(fromLeft, mn, mx, smn, smx);
    store_box(aabbs + (size_t)cur * 6, mn, mx);
    float* o = &blockBox[(cur - B) * 6];
    o[0] = mn[0]; o[1] = mn[1]; o[2] = mn[2]; o[3] = mx[0]; o[4] = mx[1]; o[5] = mx[2];
    if (cur == 0) return;
    from = -(int32_t)cur;
    cur = rec.x;
  }
}

// The queued climbers (*queued of them, each the child it comes from) up
// through the nodes that cross block boundaries: arrival counters at GPU
// scope, the boxes of the children the first kernel finished read from
// aabbs / sortedBox (written before this launch), those of this kernel with
// release / acquire on the counter.  Grid-stride over the queue.
__global__ void __launch_bounds__(kLbvhThreads) k_refit_global(const float* __restrict__ sortedBox, long long cap,
                                                               const unsigned long long* __restrict__ dN,
                                                               const int32_t* __restrict__ nodes,
                                                               const uint32_t* __restrict__ leafParents,
                                                               uint32_t* __restrict__ arrival, float* aabbs,
                                                               const int32_t* __restrict__ queue,
                                                               const uint32_t* __restrict__ queued) {
  const long long n = (long long)leaf_count(dN, (unsigned long long)cap);
  if (n < 2) return;
  const uint32_t count = *queued;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    int32_t from = queue[k];
    float mn[3], mx[3];
    long long cur;
    if (from >= 0) {
      load_box_ldg(sortedBox + (size_t)from * 6, mn, mx);
      cur = leafParents[from];
    } else {
      load_box(aabbs + (size_t)(-(long long)from) * 6, mn, mx);
      cur = nodes[(size_t)(-(long long)from) * 3 + 0];
    }
    bool published = false;  // the climber's box was stored by this kernel
    for (long long guard = 0; guard < n && cur >= 0; guard++) {
      const int32_t parent = __ldg(nodes + cur * 3 + 0), l = __ldg(nodes + cur * 3 + 1), r = __ldg(nodes + cur * 3 + 2);
      const bool fromLeft = l == from;
      const int32_t sib = fromLeft ? r : l;
      float smn[3], smx[3];
      if (sib >= 0) load_box_ldg(sortedBox + (size_t)sib * 6, smn, smx);
      if (arrive(&arrival[cur], published, sib < 0) == 0) break;
      if (sib < 0) load_box(aabbs + (size_t)(-(long long)sib) * 6, smn, smx);
      merge_box(fromLeft, mn, mx, smn, smx);
      store_box(aabbs + (size_t)cur * 6, mn, mx);
      published = true;
      if (cur == 0) break;
      from = -(int32_t)cur;
      cur = parent;
    }
  }
}

}  // namespace pga

using namespace pga;

// Sort scratch: the digit histograms, the passes' tile counters and look-back
// words (zeroed by one memset per build), then the digit bases.
static unsigned long long sort_tiles(unsigned long long n) { return (n + kSortTile - 1) / kSortTile; }

extern "C" size_t pga_lbvh_temp_bytes(uint64_t n) {
  const unsigned long long tiles = sort_tiles(n ? n : 1);
  return (size_t)(kSortPasses * kBins + 64 + (unsigned long long)kSortPasses * tiles * kBins + kSortPasses * kBins) *
         sizeof(uint32_t);
}

namespace pga {

// Scratch of one build: keys, two value arrays, arrival counters, leaf boxes
// (terminal and sorted order), the other ends of the node ranges, the radix sort's
// scratch, and the word a sort wait that gives up raises PGA_ERR_TIMEOUT in.
struct LbvhScratch {
  unsigned long long* keysA;
  uint32_t* valsA;
  uint32_t* valsB;
  uint32_t* arrival;
  float* leafBox;
  float* sortedBox;
  int32_t* nodeOther;
  void* sortTemp;
  size_t sortTempBytes;
  int* err;
};

// Polls of a look-back wait before it gives up (each followed by a 32 ns sleep).
constexpr uint32_t kSortSpinLimit = 1u << 22;

// The launches of a build over `cap` leaves, or over min(*dN, cap) when dN is
// a device count (then `cap` sizes the grids and the sort): Morton codes, the
// digit histograms and bases, four sort passes (keys ping-pong
// between out->keys and keysA, ending in out->keys), the tie-run ranks,
// Karras and the two refit kernels.
static PgaStatus launch_lbvh(const PgaTerminal* t, unsigned long long cap, const unsigned long long* dN,
                             const PgaBounds* bounds, const PgaLbvh* out, const LbvhScratch& w, cudaStream_t s) {
  Bounds b;
  for (int k = 0; k < 3; k++) {
    b.mn[k] = bounds->min[k];
    b.sz[k] = bounds->max[k] - bounds->min[k];
  }
  const unsigned long long tiles = sort_tiles(cap);
  if (pga_lbvh_temp_bytes(cap) > w.sortTempBytes) {
    set_error("LBVH: sort scratch too small for " + std::to_string(cap) + " keys");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  uint32_t* hist = static_cast<uint32_t*>(w.sortTemp);
  uint32_t* counters = hist + kSortPasses * kBins;
  uint32_t* status = counters + 64;
  uint32_t* gBase = status + (size_t)kSortPasses * tiles * kBins;
  PGA_CUDA_TRY(cudaMemsetAsync(hist, 0, (size_t)(gBase - hist) * sizeof(uint32_t), s));
  int dev = 0, sms = 0;
  PGA_CUDA_TRY(cudaGetDevice(&dev));
  PGA_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const unsigned blocks = (unsigned)((cap + kLbvhThreads - 1) / kLbvhThreads);
  unsigned long long* keys = (unsigned long long*)out->keys;
  k_morton<<<blocks, kLbvhThreads, 0, s>>>(t, cap, dN, b, keys, w.leafBox);
  PGA_CUDA_TRY(cudaGetLastError());
  const unsigned histBlocks =
      (unsigned)std::min<unsigned long long>((cap + kHistThreads - 1) / kHistThreads, (unsigned long long)sms * 4);
  k_digit_hist<<<histBlocks, kHistThreads, 0, s>>>(keys, cap, hist);
  PGA_CUDA_TRY(cudaGetLastError());
  k_sort_bases<<<1, kBins, 0, s>>>(hist, gBase);
  PGA_CUDA_TRY(cudaGetLastError());
  PGA_CUDA_TRY(cudaFuncSetAttribute(k_onesweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOnesweepSmem));
  // The first pass reads the identity values (terminal index); the values
  // then ping-pong valsB -> valsA -> valsB -> valsA.
  unsigned long long* kIn = keys;
  unsigned long long* kOut = w.keysA;
  uint32_t* vIn = nullptr;
  uint32_t* vOut = w.valsB;
  unsigned long long* words = reinterpret_cast<unsigned long long*>(status);
  for (int q = 0; q < kSortPasses; q++) {
    k_onesweep<<<(unsigned)tiles, kSortThreads, kOnesweepSmem, s>>>(
        kIn, vIn, kOut, vOut, cap, (uint32_t)(kSortLowBit + q * kRadixBits), gBase + q * kBins,
        words + (size_t)q * tiles * (kBins / 2), counters + q, w.err, kSortSpinLimit);
    PGA_CUDA_TRY(cudaGetLastError());
    std::swap(kIn, kOut);
    vIn = vOut;
    vOut = vOut == w.valsB ? w.valsA : w.valsB;
  }
  static_assert(kSortPasses % 2 == 0, "an even number of passes ends in out->keys and valsA");
  // The tie runs' order goes to keysA / valsB (free after the sort), the
  // member bits over the look-back words (free too; tiles * kBins * passes
  // words >= cap / 32).
  uint32_t* tieMask = status;
  k_tie_rank<<<blocks, kLbvhThreads, 0, s>>>(keys, w.valsA, t, cap, dN, w.keysA, w.valsB, tieMask);
  PGA_CUDA_TRY(cudaGetLastError());
  k_karras<<<blocks, kLbvhThreads, 0, s>>>(keys, (long long)cap, dN, out->nodes, out->leafParents, out->leafTerminal,
                                           w.valsA, tieMask, w.valsB, w.leafBox, w.sortedBox, w.nodeOther, w.arrival);
  PGA_CUDA_TRY(cudaGetLastError());
  // The refit's queue of climbers that leave their block goes to valsB (free
  // after Karras), its length to the sort scratch's counter word kSortPasses.
  uint32_t* queued = counters + kSortPasses;
  k_refit_local<<<blocks, kLbvhThreads, 0, s>>>(w.sortedBox, (long long)cap, dN, out->nodes, w.nodeOther,
                                                out->leafParents, out->aabbs, reinterpret_cast<int32_t*>(w.valsB),
                                                queued, tieMask, w.keysA, keys);
  PGA_CUDA_TRY(cudaGetLastError());
  const unsigned globalBlocks = std::min<unsigned>(blocks, (unsigned)sms * (2048 / kLbvhThreads));
  k_refit_global<<<globalBlocks, kLbvhThreads, 0, s>>>(w.sortedBox, (long long)cap, dN, out->nodes,
                                                       out->leafParents, w.arrival, out->aabbs,
                                                       reinterpret_cast<const int32_t*>(w.valsB), queued);
  PGA_CUDA_TRY(cudaGetLastError());
  return PGA_OK;
}

static LbvhScratch engine_scratch(PgaEngine* e) {
  return LbvhScratch{e->dKeysA,     e->dValsA,     e->dValsB,    e->dArrival,      e->dLeafAabb,
                     e->dLeafAabbSorted, e->dNodeOther, e->dSortTemp, e->sortTempBytes, &e->dState->status};
}

static bool lbvh_out_ok(const PgaLbvh* out) {
  return out && out->nodes && out->leafParents && out->aabbs && out->leafTerminal && out->keys;
}

}  // namespace pga

extern "C" PgaStatus pga_lbvh_build(PgaEngine* e, const PgaTerminal* dTerminals, uint64_t n, const PgaBounds* bounds,
                                    const PgaLbvh* out, void* stream) {
  if (!e || !dTerminals || !bounds || !lbvh_out_ok(out)) {
    set_error("pga_lbvh_build: null argument");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (n < 2 || n > e->cfg.maxTerminals || n >= (1ull << 30)) {
    set_error("pga_lbvh_build: need 2 <= n <= maxTerminals (and < 2^30)");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  return launch_lbvh(dTerminals, n, nullptr, bounds, out, engine_scratch(e), (cudaStream_t)stream);
}

extern "C" PgaStatus pga_lbvh_build_counted(PgaEngine* e, const PgaTerminal* dTerminals, const uint64_t* dCount,
                                            uint64_t capacity, const PgaBounds* bounds, const PgaLbvh* out,
                                            void* stream) {
  if (!e || !dTerminals || !dCount || !bounds || !lbvh_out_ok(out)) {
    set_error("pga_lbvh_build_counted: null argument");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (capacity < 2 || capacity > e->cfg.maxTerminals || capacity >= (1ull << 30)) {
    set_error("pga_lbvh_build_counted: need 2 <= capacity <= maxTerminals (and < 2^30)");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  return launch_lbvh(dTerminals, capacity, (const unsigned long long*)dCount, bounds, out, engine_scratch(e),
                     (cudaStream_t)stream);
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
// it.  Under CUDA's lazy module loading the array itself is committed on the
// device only when this file's module first loads there -- at that lookup at
// the latest -- so a caller that hands out its device budget at start-up
// makes one call on each device first: a call with n = 0 (pointers may be
// null) does only this set-up.  Make it before any stream capture too.  The
// address is cached per device ordinal for the life of the process: the
// library assumes that each device's primary context lives as long as the
// process (after cudaDeviceReset the cached address is stale).  All calls
// share the array and it keeps the last call's contents: the arrival counters
// that must start at zero are cleared on every call, and calls that overlap
// on the GPU (on different streams, or from different threads) race on it.

namespace pga {

constexpr size_t kStaticScratchBytes = 6u << 20;  // 6 MiB
static __device__ __align__(256) unsigned char g_lbvhStaticScratch[kStaticScratchBytes];

static std::mutex g_staticMutex;
static void* g_staticAddr[64];  // device address of g_lbvhStaticScratch per device ordinal

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace pga

extern "C" PgaStatus pga_lbvh_build_static(const PgaTerminal* dTerminals, uint64_t n, const PgaBounds* bounds,
                                           const PgaLbvh* out, void* stream) {
  if (n != 0 && (!dTerminals || !bounds || !lbvh_out_ok(out))) {
    set_error("pga_lbvh_build_static: null argument");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (n == 1 || n > PGA_LBVH_STATIC_MAX_LEAVES) {
    set_error("pga_lbvh_build_static: n must be 0 (set-up only) or in [2, " +
              std::to_string(PGA_LBVH_STATIC_MAX_LEAVES) +
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
  if (n == 0) return PGA_OK;  // set-up only
  // Carve the scratch: keys, two value arrays, arrival counters, leaf boxes
  // (terminal and sorted order), the other ends of the node ranges, sort temp.
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
  float* leafBox = reinterpret_cast<float*>(base + off);
  off += align256(n * 6 * sizeof(float));
  float* sortedBox = reinterpret_cast<float*>(base + off);
  off += align256(n * 6 * sizeof(float));
  int32_t* nodeOther = reinterpret_cast<int32_t*>(base + off);
  off += align256(n * sizeof(int32_t));
  void* sortTemp = base + off;
  off += align256(temp);
  int* err = reinterpret_cast<int*>(base + off);  // a sort wait that gives up marks it (unreported)
  off += 256;
  if (off > kStaticScratchBytes) {
    set_error("pga_lbvh_build_static: fixed scratch too small for the radix sort of " + std::to_string(n) + " keys");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  const LbvhScratch w{keysA, valsA, valsB, arrival, leafBox, sortedBox, nodeOther, sortTemp, temp, err};
  return launch_lbvh(dTerminals, n, nullptr, bounds, out, w, (cudaStream_t)stream);
}
