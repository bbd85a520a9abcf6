// Derivation kernels and the engine's C ABI (creation, derive, report).
//
// Work model: level-synchronous expansion.  A level is the set of queued work
// items; an item is a shape whose rule branches (Subdivide, Repeat,
// ComponentSplit) together with a range of at most `subItem` of its children.
// One thread executes one item's operator and produces those children in
// order.  Each child is resolved in the same thread through its chain of
// 1 -> 1 rules (IfSizeLess, Extrude) and ends as a terminal (Generate: written
// out directly), a discard, or a branching shape that is queued as work items.
//
// A warp works on a chunk of 32 x itemsPerLane work items; warps take chunks
// in a static grid-stride order (no shared work counter, no block-wide barrier
// inside a level).  Output is paged per warp: a warp holds a page of kTermPage
// terminal slots and a page of kNodePage item slots, each taken with one
// atomic, and every emission round writes a contiguous run of its page in lane
// order.  A branching child is queued as ceil(children / S) work items, with S
// = narrowSubItem while the level being expanded is narrower than the grid and
// subItem otherwise.
//
// pga_derive runs every level of every axiom in ONE persistent cooperative
// launch: a bounded grid barrier between levels, item pages closed at each
// level end, and one compaction at the end that moves the records past the
// final count into the holes the warps' last terminal pages left.
// pga_derive_plain is the plain GPU form: one axiom at a time, one launch per
// level, the host reading each level's size back, one atomic per round.
//
// The reference executes the same operators from per-procedure queues in a
// Whippletree megakernel (deps/whippletree/include/techniqueMegakernel.cuh:374-473)
// or from std::deque queues on the host (include/pga/core/CPUEvaluator.h:38-76);
// the order in which shapes are processed is free in both, so outputs are
// compared as multisets.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine_host.h"
#include "derive_kernels.cuh"

namespace pga {

// ------------------------------------------------------------- host side

static thread_local std::string g_error;

void set_error(const std::string& msg) { g_error = msg; }

PgaStatus cuda_status(cudaError_t e, const char* what) {
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return PGA_ERR_CUDA;
}

DeriveArgs make_args(PgaEngine* e, const PgaAxiom* axioms, uint32_t numAxioms, const float* blocks, PgaTerminal* out,
                     unsigned long long cap, unsigned long long* count) {
  DeriveArgs a;
  a.tab.rules = e->dRules;
  a.tab.params = e->dParams;
  a.tab.succ = e->dSucc;
  a.tab.expPool = e->dExpPool;
  a.tab.numEntries = e->numEntries;
  a.axioms = axioms;
  a.numAxioms = numAxioms;
  a.axiomBase = 0;
  a.axiomOrder = nullptr;
  a.blocks = blocks;
  a.blockStride = e->cfg.blockStride;
  a.out = out;
  a.cap = cap;
  a.outCount = count;
  a.nodes = e->dNodes;
  a.nodeRot = e->dNodeRot;
  a.nodeCap = e->cfg.nodeCapacity;
  a.termLinks = e->dTermLinks;
  a.termLinkCap = e->dTermLinks ? e->cfg.maxTerminals : 0;
  a.levelStart = e->dLevelStart;
  a.levelClock = e->dLevelClock;
  a.maxLevels = e->cfg.maxLevels;
  a.spinLimit = e->cfg.spinLimit;
  a.subItem = e->cfg.subItem;
  a.useSeeds = e->useSeeds ? 1u : 0u;
  a.itemsPerLane = e->cfg.itemsPerLane;
  a.narrowSubItem = e->cfg.narrowSubItem;
  a.tail = e->dTail;
  a.tailLinks = e->dTailLinks;
  a.tailCap = e->tailCap;
  a.scratch = e->dScratch;
  a.numWarps = (uint32_t)e->persistentBlocks * (uint32_t)(e->threads / 32);
  a.tableInSmem = e->tableInSmem ? 1u : 0u;
  a.numParams = (uint32_t)e->hParams.size();
  a.numSucc = (uint32_t)e->hSucc.size();
  a.st = e->dState;
  a.phase = 0;
  a.deferIn = nullptr;
  a.deferRotIn = nullptr;
  a.numDeferIn = 0;
  a.deferOut = e->dDefer[0];
  a.deferRotOut = e->dDeferRot[0];
  a.deferCap = e->phased ? e->cfg.nodeCapacity : 0;
  a.phaseCounters = e->dPhaseCounters;
  a.colRec = e->dColRec;
  a.colShape = e->dColShape;
  a.colCap = e->colCap;
  a.colNodes = e->dColNodes;
  a.colAabbs = e->dColAabbs;
  a.colLeaf = e->dColLeaf;
  a.numColliders = 0;
  return a;
}

}  // namespace pga

using namespace pga;

namespace pga {
FrameKernels general_frame_kernels();  // derive_gen.cu
FrameKernels block_frame_kernels();    // derive_blk.cu
inline namespace PGA_FRAMES_NS {
inline const void* adjoint_kernel();       // this build's k_adjoint (adjoint.cuh, included below)
inline const void* adjoint_kernel_wide();  // and k_adjoint_wide
}
}

// The instantiation of the persistent kernel for an engine: its frame build,
// leaf children in place or not, with or without the 1 -> 1 affine steps.
static const void* persistent_kernel(const PgaEngine* e) {
  if (e->phased) return e->kernels.phased;
  if (!e->leafKernel && (e->cfg.flags & PGA_FLAG_DYNAMIC_CHUNKS)) return e->kernels.persistentDyn[e->affineKernel ? 1 : 0];
  return e->kernels.persistent[(e->leafKernel ? 1 : 0) + (e->affineKernel ? 2 : 0)];
}

// The persistent instantiations of a build: the four static ones, the phased
// one and the two with dynamic chunks.
static const void* persistent_at(const FrameKernels& k, int i) {
  return i < 4 ? k.persistent[i] : (i == 4 ? k.phased : k.persistentDyn[i - 5]);
}
constexpr int kPersistentKernels = 7;

// All kernels of the engine's build get the same dynamic shared memory limit;
// the launch uses the smallest of the persistent instantiations' occupancies,
// so any of them can run co-resident.
static cudaError_t set_kernel_smem(const FrameKernels& k, size_t bytes) {
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < kPersistentKernels && err == cudaSuccess; i++)
    err = cudaFuncSetAttribute(persistent_at(k, i), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err == cudaSuccess) err = cudaFuncSetAttribute(k.seed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (err == cudaSuccess) err = cudaFuncSetAttribute(k.expand, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return err;
}
static cudaError_t persistent_occupancy(const FrameKernels& k, int* perSM, int threads, size_t smem) {
  int best = 1 << 30;
  cudaError_t err = cudaSuccess;
  for (int i = 0; i < kPersistentKernels && err == cudaSuccess; i++) {
    int n = 0;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, persistent_at(k, i), threads, smem);
    best = std::min(best, n);
  }
  *perSM = best;
  return err;
}

// math::float4x4::rotateXYZ (deps/math/include/math/matrix.h:876-888) of
// Rotate's angles after its degree to radian conversion (Rotate.cuh:34-36),
// in float on the host as the reference computes it: the rotation part,
// row-major.  Built once per Rotate rule, whose angles are scalars.
static void rotate_xyz(float x, float y, float z, float q[9]) {
  const float k = 3.1415926535897932384626434f / 180.0f;
  x *= k;
  y *= k;
  z *= k;
  const float sa = std::sin(x), sb = std::sin(y), sg = std::sin(z);
  const float ca = std::cos(x), cb = std::cos(y), cg = std::cos(z);
  q[0] = cb * cg;
  q[1] = cg * sa * sb - ca * sg;
  q[2] = ca * cg * sb + sa * sg;
  q[3] = cb * sg;
  q[4] = ca * cg + sa * sb * sg;
  q[5] = -cg * sa + ca * sb * sg;
  q[6] = -sb;
  q[7] = cb * sa;
  q[8] = ca * cb;
}

static const PgaProc kDefaultProcs[40] = {
    {PGA_OP_SUBDIVIDE, PGA_SHAPE_BOX, 0, 1},        {PGA_OP_SUBDIVIDE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_SUBDIVIDE_STATIC, PGA_SHAPE_BOX, 3, 1}, {PGA_OP_SUBDIVIDE_STATIC, PGA_SHAPE_QUAD, 3, 1},
    {PGA_OP_REPEAT, PGA_SHAPE_BOX, 0, 1},           {PGA_OP_REPEAT, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_COMPONENT_SPLIT, PGA_SHAPE_BOX, 0, 1},  {PGA_OP_EXTRUDE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_IF_SIZE_LESS, PGA_SHAPE_BOX, 0, 1},     {PGA_OP_IF_SIZE_LESS, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_GENERATE, PGA_SHAPE_BOX, 0, 1},         {PGA_OP_GENERATE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_DISCARD, PGA_SHAPE_BOX, 0, 1},          {PGA_OP_DISCARD, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_TRANSLATE, PGA_SHAPE_BOX, 0, 1},        {PGA_OP_TRANSLATE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_SCALE, PGA_SHAPE_BOX, 0, 1},            {PGA_OP_SCALE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_RANDOM_RULE, PGA_SHAPE_BOX, 0, 1},      {PGA_OP_RANDOM_RULE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_ROTATE, PGA_SHAPE_BOX, 0, 1},           {PGA_OP_ROTATE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_REPLICATE, PGA_SHAPE_BOX, 0, 1},        {PGA_OP_REPLICATE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_BOX, 2, 1}, {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_QUAD, 2, 1},
    {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_BOX, 3, 1}, {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_QUAD, 3, 1},
    {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_BOX, 4, 1}, {PGA_OP_RANDOM_RULE_STATIC, PGA_SHAPE_QUAD, 4, 1},
    {PGA_OP_IF, PGA_SHAPE_BOX, 0, 1},               {PGA_OP_IF, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_SWAP_SIZE, PGA_SHAPE_BOX, 0, 1},        {PGA_OP_SWAP_SIZE, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_GENERATE_MESH, PGA_SHAPE_BOX, 0, 1},    {PGA_OP_GENERATE_MESH, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_COLLIDER, PGA_SHAPE_BOX, 0, 1},         {PGA_OP_COLLIDER, PGA_SHAPE_QUAD, 0, 1},
    {PGA_OP_IF_COLLIDES, PGA_SHAPE_BOX, 0, 1},      {PGA_OP_IF_COLLIDES, PGA_SHAPE_QUAD, 0, 1},
};

extern "C" {

const char* pga_version(void) { return "pga_gb300 0.1.0 (sm_103a)"; }

const char* pga_last_error(void) { return g_error.c_str(); }

const PgaProc* pga_default_procs(uint32_t* numProcs) {
  if (numProcs) *numProcs = 40;
  return kDefaultProcs;
}

static void free_engine(PgaEngine* e) {
  void* phasePtrs[] = {e->dDefer[0], e->dDefer[1], e->dDeferRot[0], e->dDeferRot[1], e->dColRec, e->dColShape,
                       e->dColNodes, e->dColParents, e->dColAabbs, e->dColLeaf, e->dColKeys, e->dPhaseCounters};
  for (void* p : phasePtrs)
    if (p) cudaFree(p);
  void* ptrs[] = {e->dRules, e->dParams, e->dSucc, e->dExpPool, e->dState, e->dNodes, e->dNodeRot, e->dLevelClock,
                  e->dTail, e->dTailLinks, e->dScratch,
                  e->dTermLinks, e->dLevelStart, e->dScratchCount, e->dSortTemp, e->dKeysA,
                  e->dValsA, e->dValsB, e->dArrival, e->dLeafAabb, e->dLeafAabbSorted, e->dNodeOther, e->dNodeGrad, e->dChildKey, e->dPageNext,
                  e->dSlots, e->dBlockSums, e->dGroupCount};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (e->dStageAxioms) cudaFree(e->dStageAxioms);
  if (e->dStageOut) cudaFree(e->dStageOut);
  if (e->dStageCount) cudaFree(e->dStageCount);
  if (e->copyStream) cudaStreamDestroy(e->copyStream);
  if (e->evDerived) cudaEventDestroy(e->evDerived);
  delete e;
}

size_t pga_lbvh_temp_bytes(uint64_t n);  // lbvh.cu

PgaStatus pga_engine_create(const PgaRuleTable* table, const PgaEngineConfig* config, PgaEngine** out) {
  if (!table || !out || !table->entries || !table->procs || table->numEntries == 0) {
    set_error("pga_engine_create: null table, procedure list or output pointer");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  PgaEngine* e = new PgaEngine();
  if (config) e->cfg = *config;
  PgaEngineConfig& c = e->cfg;
  if (c.nodeCapacity == 0) c.nodeCapacity = 1ull << 22;
  if (c.maxTerminals == 0) c.maxTerminals = 1ull << 22;
  if (c.threadsPerBlock == 0) c.threadsPerBlock = 256;
  if (c.spinLimit == 0) c.spinLimit = 1u << 24;
  if (c.maxLevels == 0) c.maxLevels = 4096;
  if (c.subItem == 0) c.subItem = 8;
  if (c.itemsPerLane == 0) c.itemsPerLane = 1;
  if (c.narrowSubItem == 0) c.narrowSubItem = c.subItem;
  if (c.subItem > 64 || c.narrowSubItem > 64) {
    set_error("pga_engine_create: subItem and narrowSubItem must be at most 64");
    delete e;
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (c.threadsPerBlock != 256) {
    set_error("pga_engine_create: threadsPerBlock must be 256");
    delete e;
    return PGA_ERR_INVALID_ARGUMENT;
  }
  e->threads = (int)c.threadsPerBlock;

  // Lower the dispatch table: one DevRule per entry, parameters and successors
  // packed, expression parameters' 16 values in a pool.
  e->numEntries = table->numEntries;
  for (uint32_t i = 0; i < table->numEntries; i++) {
    const PgaEntry& en = table->entries[i];
    DevRule r;
    memset(&r, 0, sizeof r);
    r.op = 0xFF;
    if (en.operatorCode >= 0 && (uint32_t)en.operatorCode < table->numProcs) {
      const PgaProc& p = table->procs[en.operatorCode];
      if (p.op <= PGA_OP_IF_COLLIDES && p.shape <= PGA_SHAPE_QUAD) {
        // A triangle-mesh Generate derives exactly like an instanced one; the
        // flag marks its records for pga_generate_meshes.
        r.op = (uint8_t)(p.op == PGA_OP_GENERATE_MESH ? PGA_OP_GENERATE : p.op);
        if (p.op == PGA_OP_GENERATE_MESH) r.flags = kRuleMesh;
        r.shape = (uint8_t)p.shape;
        r.nChildren = p.numChildren;
      }
    }
    if (en.numParameters > PGA_MAX_NUM_PARAMETERS || en.numSuccessors > PGA_MAX_NUM_SUCCESSORS) {
      set_error("pga_engine_create: entry " + std::to_string(i) + " exceeds MaxNumParameters/MaxNumSuccessors");
      delete e;
      return PGA_ERR_BAD_PARAM;
    }
    if (r.op == PGA_OP_SUBDIVIDE_STATIC && (r.nChildren > PGA_MAX_NUM_SUCCESSORS || r.nChildren == 0)) {
      set_error("pga_engine_create: static Subdivide with an invalid number of pairs");
      delete e;
      return PGA_ERR_BAD_PARAM;
    }
    r.nParams = (uint8_t)en.numParameters;
    r.nSucc = (uint8_t)en.numSuccessors;
    bool pure = true, scalar = true;
    for (uint32_t k = 0; k < en.numParameters; k++) {
      const PgaParameter& p = en.parameters[k];
      if (p.type != PGA_PT_SCALAR && p.type != PGA_PT_BLOCK) pure = false;
      if (p.type != PGA_PT_SCALAR) scalar = false;
      // Seeds are observable only through random ranges, expressions and the
      // seed attribute (Shape::at(15)); otherwise seed updates can be skipped.
      if (p.type == PGA_PT_RAND || p.type == PGA_PT_EXP) e->useSeeds = true;
      if (p.type == PGA_PT_SHAPE_ATTR && p.value[0] >= 15.0f && p.value[0] < 16.0f) e->useSeeds = true;
    }
    r.flags = (uint16_t)((r.flags & kRuleMesh) | (pure ? kRulePure : 0) | (scalar ? kRuleScalar : 0));
    // A scalar terminal index is decided here once (the device truncates it
    // toward zero like __float2uint_rz; only 0..127 are valid mesh indices).
    if (r.op == PGA_OP_GENERATE && en.numParameters >= 1 && en.parameters[0].type == PGA_PT_SCALAR &&
        en.parameters[0].value[0] >= 0.0f && en.parameters[0].value[0] < 128.0f) {
      r.flags |= kRuleConstTerminal;
      r.nChildren = (uint16_t)(uint32_t)en.parameters[0].value[0];
    }
    r.paramBase = (uint32_t)e->hParams.size();
    r.succBase = (uint32_t)e->hSucc.size();
    for (uint32_t k = 0; k < en.numParameters; k++) {
      const PgaParameter& p = en.parameters[k];
      DevParam d;
      d.type = p.type;
      d.v0 = p.value[0];
      d.v1 = p.value[1];
      d.aux = 0;
      if (p.type == PGA_PT_EXP) {
        d.aux = (uint32_t)e->hExpPool.size();
        e->hExpPool.insert(e->hExpPool.end(), p.value, p.value + PGA_MAX_NUM_PARAMETER_VALUES);
      }
      e->hParams.push_back(d);
    }
    if (r.op == PGA_OP_ROTATE) {
      // The rotation of scalar angles is built here, once; parameter 0's aux
      // points at its 9 entries in the expression pool.
      if (en.numParameters < 3 || en.parameters[0].type != PGA_PT_SCALAR || en.parameters[1].type != PGA_PT_SCALAR ||
          en.parameters[2].type != PGA_PT_SCALAR) {
        set_error("pga_engine_create: entry " + std::to_string(i) + ": Rotate takes three scalar angles");
        delete e;
        return PGA_ERR_BAD_PARAM;
      }
      float q[9];
      rotate_xyz(en.parameters[0].value[0], en.parameters[1].value[0], en.parameters[2].value[0], q);
      e->hParams[r.paramBase].aux = (uint32_t)e->hExpPool.size();
      e->hExpPool.insert(e->hExpPool.end(), q, q + 9);
    }
    for (uint32_t k = 0; k < en.numSuccessors; k++) e->hSucc.push_back(en.successors[k].entryIndex);
    e->hRules.push_back(r);
  }
  // Leaf rules: a Subdivide with shape-independent factors whose every child
  // successor is a Generate with a constant terminal index or a Discard, both
  // of the Subdivide's own shape (children keep the parent's shape kind).
  for (DevRule& r : e->hRules) {
    if ((r.op != PGA_OP_SUBDIVIDE && r.op != PGA_OP_SUBDIVIDE_STATIC) || !(r.flags & kRulePure)) continue;
    const uint32_t n = r.op == PGA_OP_SUBDIVIDE ? (r.nParams >= 1 ? r.nParams - 1u : 0u) : r.nChildren;
    if (n == 0 || n > r.nSucc || r.nParams < n + 1) continue;
    bool leaf = true;
    for (uint32_t k = 0; k < n && leaf; k++) {
      const int32_t s = e->hSucc[r.succBase + k];
      if (s < 0 || (size_t)s >= e->hRules.size()) {
        leaf = false;
        break;
      }
      const DevRule& sr = e->hRules[(size_t)s];
      leaf = sr.shape == r.shape &&
             ((sr.op == PGA_OP_GENERATE && (sr.flags & kRuleConstTerminal)) || sr.op == PGA_OP_DISCARD);
    }
    if (leaf) r.flags |= kRuleLeaf;
    // Leaf children are expanded in place, except with a tape (the adjoint
    // replays one work item per branching shape) or when disabled.
    if (leaf && !c.recordTape && !(c.flags & PGA_FLAG_NO_INLINE)) e->leafKernel = true;
  }
  // Phases: the phase of a rule is the phaseIndex of the successor edges that
  // lead to it (the reference queues a symbol in the phase its edge names,
  // CPUEvaluator.h:155-190); edges into one rule must agree.  A shape reaching
  // a rule of a later phase is deferred to that phase's launch.
  {
    std::vector<int> phaseOf(e->hRules.size(), -1);
    for (uint32_t i = 0; i < table->numEntries; i++) {
      const PgaEntry& en = table->entries[i];
      for (uint32_t k = 0; k < en.numSuccessors && k < PGA_MAX_NUM_SUCCESSORS; k++) {
        const int32_t t = en.successors[k].entryIndex;
        if (t < 0 || (uint32_t)t >= table->numEntries) continue;
        const int ph = en.successors[k].phaseIndex < 0 ? 0 : en.successors[k].phaseIndex;
        if (ph >= (int)kMaxPhases || (phaseOf[t] >= 0 && phaseOf[t] != ph)) {
          set_error("pga_engine_create: entry " + std::to_string(t) +
                    ": successor edges name different phases (or a phase >= 16)");
          delete e;
          return PGA_ERR_BAD_PARAM;
        }
        phaseOf[t] = ph;
      }
    }
    for (size_t t = 0; t < e->hRules.size(); t++) {
      if (phaseOf[t] > 0) {
        e->hRules[t].flags = (uint16_t)(e->hRules[t].flags | (phaseOf[t] << kRulePhaseShift));
        e->phased = true;
      }
    }
  }
  for (const DevRule& r : e->hRules) {
    if (r.op == PGA_OP_COLLIDER || r.op == PGA_OP_IF_COLLIDES) e->phased = true;
    if (r.op == PGA_OP_TRANSLATE || r.op == PGA_OP_SCALE || r.op == PGA_OP_RANDOM_RULE || r.op == PGA_OP_ROTATE ||
        r.op == PGA_OP_REPLICATE || r.op == PGA_OP_RANDOM_RULE_STATIC || r.op == PGA_OP_IF || r.op == PGA_OP_SWAP_SIZE)
      e->affineKernel = true;
    if (r.op == PGA_OP_ROTATE) e->generalFrames = true;
  }
  if (e->phased) {
    // phase checks, Collider and IfCollides live in the AFF instantiations;
    // leaf children in place would skip the phase check of their Generates
    e->affineKernel = true;
    e->leafKernel = false;
    for (DevRule& r : e->hRules) r.flags = (uint16_t)(r.flags & ~kRuleLeaf);
  }
  if (e->phased && c.recordTape) {
    set_error("pga_engine_create: the adjoint (recordTape) does not cover phases and colliders");
    delete e;
    return PGA_ERR_BAD_PARAM;
  }
  // Tables with block parameters (and no Rotate) run the build that reads
  // them inline; the others keep this file's kernels.
  bool blockParams = false;
  for (const DevParam& p : e->hParams) blockParams = blockParams || p.type == PGA_PT_BLOCK;
  if (e->generalFrames) {
    e->kernels = general_frame_kernels();
  } else if (blockParams) {
    e->kernels = block_frame_kernels();
  } else {
    e->kernels = frame_kernels();
    e->kernels.adjoint = adjoint_kernel();
    e->kernels.adjointWide = adjoint_kernel_wide();
  }
  // Large tapes take the 3-blocks-per-SM adjoint (see k_adjoint_wide).
  if (c.maxTerminals >= kWideAdjointTerminals && e->kernels.adjointWide) e->kernels.adjoint = e->kernels.adjointWide;
  if (e->hParams.empty()) e->hParams.push_back(DevParam{0, 0.f, 0.f, 0});
  if (e->hSucc.empty()) e->hSucc.push_back(-1);
  if (e->hExpPool.empty()) e->hExpPool.push_back(0.f);

  auto fail = [&](PgaStatus s) {
    free_engine(e);
    return s;
  };
  cudaError_t err;
#define ALLOC(ptr, bytes)                                                      \
  do {                                                                         \
    err = cudaMalloc((void**)&(ptr), (bytes));                                 \
    if (err != cudaSuccess) return fail(cuda_status(err, "cudaMalloc " #ptr)); \
  } while (0)
  ALLOC(e->dRules, e->hRules.size() * sizeof(DevRule));
  ALLOC(e->dParams, e->hParams.size() * sizeof(DevParam));
  ALLOC(e->dSucc, e->hSucc.size() * sizeof(int32_t));
  ALLOC(e->dExpPool, e->hExpPool.size() * sizeof(float));
  ALLOC(e->dState, sizeof(DevState));
  ALLOC(e->dNodes, c.nodeCapacity * sizeof(Node));
  if (e->generalFrames) ALLOC(e->dNodeRot, c.nodeCapacity * 2 * sizeof(float4));
  if (e->phased) {
    // deferred shapes (two buffers: the phase's input and its output),
    // colliders (records, oriented boxes) and the colliders' LBVH
    for (int k = 0; k < 2; k++) {
      ALLOC(e->dDefer[k], c.nodeCapacity * sizeof(Node));
      if (e->generalFrames) ALLOC(e->dDeferRot[k], c.nodeCapacity * 2 * sizeof(float4));
    }
    e->colCap = std::min<uint64_t>(c.nodeCapacity, c.maxTerminals);
    ALLOC(e->dColRec, e->colCap * sizeof(PgaTerminal));
    ALLOC(e->dColShape, e->colCap * 5 * sizeof(float4));
    ALLOC(e->dColNodes, std::max<uint64_t>(e->colCap, 2) * 3 * sizeof(int32_t));
    ALLOC(e->dColParents, e->colCap * sizeof(uint32_t));
    ALLOC(e->dColAabbs, std::max<uint64_t>(e->colCap, 2) * 6 * sizeof(float));
    ALLOC(e->dColLeaf, e->colCap * sizeof(uint32_t));
    ALLOC(e->dColKeys, e->colCap * sizeof(uint64_t));
    ALLOC(e->dPhaseCounters, 4 * sizeof(unsigned long long));
  }
  ALLOC(e->dLevelStart, (c.maxLevels + 2) * sizeof(unsigned long long));
  ALLOC(e->dLevelClock, (c.maxLevels + 2) * sizeof(unsigned long long));
  ALLOC(e->dScratchCount, sizeof(unsigned long long));
  ALLOC(e->dGroupCount, (e->hRules.size() + 1) * sizeof(uint32_t));
  if (c.recordTape) {
    // The reverse pass tags work-item indices with bit 31 and counts child
    // slots in 32 bits; a work item has at most max(subItem, narrowSubItem)
    // children, which bounds the slots.
    if (c.nodeCapacity >= 0x7FFFFFFFull) {
      set_error("pga_engine_create: recordTape needs nodeCapacity < 2^31 - 1");
      return fail(PGA_ERR_INVALID_ARGUMENT);
    }
    e->slotCap = std::min<unsigned long long>(c.nodeCapacity * std::max(c.subItem, c.narrowSubItem), 0xFFFFFFF0ull);
    ALLOC(e->dTermLinks, c.maxTerminals * sizeof(uint2));
    ALLOC(e->dNodeGrad, c.nodeCapacity * 6 * sizeof(float));
    ALLOC(e->dChildKey, c.nodeCapacity * sizeof(uint32_t));
    ALLOC(e->dPageNext, c.nodeCapacity * sizeof(uint32_t));
    ALLOC(e->dSlots, e->slotCap * sizeof(uint32_t));
    ALLOC(e->dBlockSums, kMaxAdjointBlocks * sizeof(unsigned long long));
  }
  // LBVH scratch for up to maxTerminals leaves.
  e->sortTempBytes = pga_lbvh_temp_bytes(c.maxTerminals);
  ALLOC(e->dSortTemp, e->sortTempBytes);
  ALLOC(e->dKeysA, c.maxTerminals * sizeof(unsigned long long));
  ALLOC(e->dLeafAabb, c.maxTerminals * 6 * sizeof(float));
  ALLOC(e->dLeafAabbSorted, c.maxTerminals * 6 * sizeof(float));
  ALLOC(e->dNodeOther, c.maxTerminals * sizeof(int32_t));
  ALLOC(e->dValsA, c.maxTerminals * sizeof(uint32_t));
  ALLOC(e->dValsB, c.maxTerminals * sizeof(uint32_t));
  ALLOC(e->dArrival, c.maxTerminals * sizeof(uint32_t));
#undef ALLOC
  err = cudaMemcpy(e->dRules, e->hRules.data(), e->hRules.size() * sizeof(DevRule), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(e->dParams, e->hParams.data(), e->hParams.size() * sizeof(DevParam), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(e->dSucc, e->hSucc.data(), e->hSucc.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (err == cudaSuccess)
    err = cudaMemcpy(e->dExpPool, e->hExpPool.data(), e->hExpPool.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaMemset(e->dState, 0, sizeof(DevState));
  if (err != cudaSuccess) return fail(cuda_status(err, "pga_engine_create upload"));

  // Shared memory: block scratch, plus the rule table when it is small.
  size_t tableBytes = e->hRules.size() * sizeof(DevRule) + e->hParams.size() * sizeof(DevParam) +
                      e->hSucc.size() * sizeof(int32_t);
  e->tableInSmem = tableBytes <= 48 * 1024;
  e->smemBytes = sizeof(Smem) + (e->tableInSmem ? ((tableBytes + 15) & ~size_t(15)) : 0);
  err = cudaGetDevice(&e->device);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&e->numSMs, cudaDevAttrMultiProcessorCount, e->device);
  if (err == cudaSuccess) err = set_kernel_smem(e->kernels, e->smemBytes);
  int perSM = 0;
  if (err == cudaSuccess) err = persistent_occupancy(e->kernels, &perSM, e->threads, e->smemBytes);
  if (err != cudaSuccess) return fail(cuda_status(err, "pga_engine_create occupancy"));
  if (c.blocksPerSM > 0 && (int)c.blocksPerSM < perSM) perSM = (int)c.blocksPerSM;
  if (perSM < 1) perSM = 1;
  {
    // The end-of-launch compaction keeps per-warp tables in the same dynamic
    // shared memory (the rule table is no longer read by then).
    const size_t need = compact_smem_bytes((uint32_t)(perSM * e->numSMs * (e->threads / 32)));
    if (need > e->smemBytes) {
      e->smemBytes = (need + 15) & ~size_t(15);
      err = set_kernel_smem(e->kernels, e->smemBytes);
      int again = 0;
      if (err == cudaSuccess) err = persistent_occupancy(e->kernels, &again, e->threads, e->smemBytes);
      if (err != cudaSuccess) return fail(cuda_status(err, "pga_engine_create occupancy"));
      perSM = std::max(1, std::min(perSM, again));  // fewer warps need fewer bytes
    }
  }
  e->persistentBlocks = perSM * e->numSMs;
  {
    // Paged output of the persistent engine: every warp may leave one partly
    // filled terminal page, so up to warps * kTermPage slots can lie past the
    // caller's capacity before compaction; they go to a tail buffer.
    const unsigned long long warps = (unsigned long long)e->persistentBlocks * (e->threads / 32);
    e->tailCap = warps * kTermPage;
    err = cudaMalloc((void**)&e->dTail, e->tailCap * sizeof(PgaTerminal));
    if (err == cudaSuccess && c.recordTape) err = cudaMalloc((void**)&e->dTailLinks, e->tailCap * sizeof(uint2));
    if (err == cudaSuccess) err = cudaMalloc((void**)&e->dScratch, (warps + 2) * sizeof(unsigned long long));
    if (err != cudaSuccess) return fail(cuda_status(err, "pga_engine_create tail"));
  }
  *out = e;
  return PGA_OK;
}

PgaStatus pga_engine_destroy(PgaEngine* e) {
  if (!e) return PGA_ERR_INVALID_ARGUMENT;
  cudaDeviceSynchronize();
  free_engine(e);
  return PGA_OK;
}

}  // extern "C"

// One persistent launch over axioms [first, end) of dAxioms (path hashes are
// seeded from the absolute axiom index, so a batch derived in ranges gives the
// same terminals as one launch).
// Axiom grouping (PGA_FLAG_GROUP_AXIOMS): a counting sort of the axiom indices
// by root entry -- count, one-block exclusive scan, scatter -- with one atomic
// per warp and entry (a batch may hold tens of thousands of axioms of one
// entry).  Entries out of range share the last bucket; the seed reports them.
__device__ __forceinline__ uint32_t group_bucket(const PgaAxiom* ax, uint32_t i, uint32_t numEntries) {
  const uint32_t e = __ldg(&ax[i].entry);
  return e < numEntries ? e : numEntries;
}

__global__ void k_group_count(const PgaAxiom* ax, uint32_t n, uint32_t numEntries, uint32_t* count) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t e = i < n ? group_bucket(ax, i, numEntries) : 0xFFFFFFFFu;
  const unsigned same = __match_any_sync(0xFFFFFFFFu, e);
  if (i < n && (threadIdx.x & 31u) == (uint32_t)(__ffs(same) - 1)) atomicAdd(count + e, (uint32_t)__popc(same));
}

__global__ void k_group_scan(uint32_t* count, uint32_t buckets) {
  __shared__ uint32_t warpSum[32];
  __shared__ uint32_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t t0 = 0; t0 < buckets; t0 += blockDim.x) {
    const uint32_t k = t0 + threadIdx.x;
    const uint32_t v = k < buckets ? count[k] : 0u;
    uint32_t x = v;
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, d);
      if (lane >= (unsigned)d) x += y;
    }
    if (lane == 31) warpSum[warp] = x;
    __syncthreads();
    uint32_t before = carry, total = 0;
    for (uint32_t w = 0; w < (blockDim.x >> 5); w++) {
      before += w < warp ? warpSum[w] : 0u;
      total += warpSum[w];
    }
    if (k < buckets) count[k] = before + x - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += total;
    __syncthreads();
  }
}

__global__ void k_group_scatter(const PgaAxiom* ax, uint32_t n, uint32_t numEntries, uint32_t* offset,
                                uint32_t* order) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t e = i < n ? group_bucket(ax, i, numEntries) : 0xFFFFFFFFu;
  const unsigned same = __match_any_sync(0xFFFFFFFFu, e);
  const uint32_t leader = (uint32_t)(__ffs(same) - 1);
  uint32_t base = 0;
  if (i < n && (threadIdx.x & 31u) == leader) base = atomicAdd(offset + e, (uint32_t)__popc(same));
  base = __shfl_sync(0xFFFFFFFFu, base, leader);
  unsigned lt;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
  if (i < n) order[base + __popc(same & lt)] = i;
}

// The seed order of a pga_derive over n axioms: null (index order) unless the
// engine groups axioms; the order lives in the LBVH key scratch, idle during
// a derivation (up to 2 maxTerminals axioms; larger batches keep index order).
static PgaStatus group_axioms(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t n, cudaStream_t s,
                              const uint32_t** order) {
  *order = nullptr;
  if (!(e->cfg.flags & PGA_FLAG_GROUP_AXIOMS) || n < 2 || (uint64_t)n > 2 * e->cfg.maxTerminals) return PGA_OK;
  const uint32_t numEntries = (uint32_t)e->hRules.size();
  uint32_t* out = reinterpret_cast<uint32_t*>(e->dKeysA);
  PGA_CUDA_TRY(cudaMemsetAsync(e->dGroupCount, 0, (numEntries + 1) * sizeof(uint32_t), s));
  const unsigned blocks = (n + 255) / 256;
  k_group_count<<<blocks, 256, 0, s>>>(dAxioms, n, numEntries, e->dGroupCount);
  PGA_CUDA_TRY(cudaGetLastError());
  k_group_scan<<<1, 1024, 0, s>>>(e->dGroupCount, numEntries + 1);
  PGA_CUDA_TRY(cudaGetLastError());
  k_group_scatter<<<blocks, 256, 0, s>>>(dAxioms, n, numEntries, e->dGroupCount, out);
  PGA_CUDA_TRY(cudaGetLastError());
  *order = out;
  return PGA_OK;
}

static PgaStatus launch_persistent(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t first, uint32_t end,
                                   const float* dParamBlocks, PgaTerminal* dOut, uint64_t capacity, uint64_t* dCount,
                                   cudaStream_t s, const uint32_t* order = nullptr) {
  PGA_CUDA_TRY(cudaMemsetAsync(e->dState, 0, sizeof(DevState), s));
  DeriveArgs a = make_args(e, dAxioms, end, dParamBlocks, dOut, capacity, (unsigned long long*)dCount);
  a.axiomBase = first;
  a.axiomOrder = order;
  void* args[] = {&a};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)e->persistentBlocks);
  cfg.blockDim = dim3((unsigned)e->threads);
  cfg.dynamicSmemBytes = e->smemBytes;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const void* kernel = persistent_kernel(e);
  PGA_CUDA_TRY(cudaLaunchKernelExC(&cfg, kernel, args));
  e->lastAxioms = dAxioms;
  e->lastNumAxioms = end;
  e->lastBlocks = dParamBlocks;
  e->lastOut = dOut;
  e->lastCap = capacity;
  e->lastWasBatched = first == 0;
  return PGA_OK;
}

// Bounds of the colliders' centres (one block), for the Morton codes of their LBVH.
__global__ void k_collider_bounds(const PgaTerminal* rec, unsigned long long n, float* out) {
  __shared__ float sh[6][256];
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (unsigned long long i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = 0; k < 3; k++) {
      const float c = rec[i].m[k * 4 + 3];
      lo[k] = fminf(lo[k], c);
      hi[k] = fmaxf(hi[k], c);
    }
  for (int k = 0; k < 3; k++) {
    sh[k][threadIdx.x] = lo[k];
    sh[3 + k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (unsigned w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; k++) {
        sh[k][threadIdx.x] = fminf(sh[k][threadIdx.x], sh[k][threadIdx.x + w]);
        sh[3 + k][threadIdx.x] = fmaxf(sh[3 + k][threadIdx.x], sh[3 + k][threadIdx.x + w]);
      }
    __syncthreads();
  }
  if (threadIdx.x < 6) out[threadIdx.x] = sh[threadIdx.x][0];
}

// Multi-phase derivation (MultiPhaseEvaluator::execute, CPUEvaluator.h:330-352,
// with the GPU evaluator's BVH construction between phases): phase 0 from the
// axioms; every later phase from the shapes the previous launch deferred, with
// the colliders stored so far in an LBVH for IfCollides.  Each phase is one
// persistent launch appending to the output; the host reads the counts back
// between phases.
static PgaStatus derive_phases(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t numAxioms, const float* dBlocks,
                               PgaTerminal* dOut, uint64_t capacity, uint64_t* dCount, cudaStream_t s) {
  PGA_CUDA_TRY(cudaMemsetAsync(e->dPhaseCounters, 0, 4 * sizeof(unsigned long long), s));
  uint64_t total = 0, numDefer = 0;
  uint32_t visible = 0;
  e->phasesRun = 0;
  for (uint32_t phase = 0; phase < kMaxPhases; phase++) {
    PGA_CUDA_TRY(cudaMemsetAsync(e->dState, 0, sizeof(DevState), s));
    PGA_CUDA_TRY(cudaMemsetAsync(e->dPhaseCounters + 1, 0, 2 * sizeof(unsigned long long), s));
    const uint64_t off = std::min(total, capacity);
    DeriveArgs a = make_args(e, dAxioms, numAxioms, dBlocks, dOut ? dOut + off : nullptr, capacity - off,
                             e->dPhaseCounters + 2);
    a.phase = phase;
    if (phase > 0) {
      a.deferIn = e->dDefer[(phase + 1) & 1];
      a.deferRotIn = e->dDeferRot[(phase + 1) & 1];
      a.numDeferIn = numDefer;
    }
    a.deferOut = e->dDefer[phase & 1];
    a.deferRotOut = e->dDeferRot[phase & 1];
    a.numColliders = visible;
    void* args[] = {&a};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)e->persistentBlocks);
    cfg.blockDim = dim3((unsigned)e->threads);
    cfg.dynamicSmemBytes = e->smemBytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PGA_CUDA_TRY(cudaLaunchKernelExC(&cfg, persistent_kernel(e), args));
    DevState snap;
    unsigned long long counters[2];
    PGA_CUDA_TRY(cudaMemcpyAsync(&snap, e->dState, sizeof snap, cudaMemcpyDeviceToHost, s));
    PGA_CUDA_TRY(cudaMemcpyAsync(counters, e->dPhaseCounters, sizeof counters, cudaMemcpyDeviceToHost, s));
    PGA_CUDA_TRY(cudaStreamSynchronize(s));
    e->phasesRun = phase + 1;
    total += snap.termCount;
    numDefer = counters[1];
    if (snap.status != 0 || numDefer == 0) break;
    // The colliders stored so far, for the next phase's IfCollides.
    visible = (uint32_t)std::min<unsigned long long>(counters[0], e->colCap);
    if (visible == 1) {
      PGA_CUDA_TRY(cudaMemsetAsync(e->dColLeaf, 0, sizeof(uint32_t), s));
    } else if (visible >= 2) {
      float* dB = reinterpret_cast<float*>(e->dColAabbs);  // scratch until the LBVH writes it
      k_collider_bounds<<<1, 256, 0, s>>>(e->dColRec, visible, dB);
      PGA_CUDA_TRY(cudaGetLastError());
      float hb[6];
      PGA_CUDA_TRY(cudaMemcpyAsync(hb, dB, sizeof hb, cudaMemcpyDeviceToHost, s));
      PGA_CUDA_TRY(cudaStreamSynchronize(s));
      PgaBounds b;
      for (int k = 0; k < 3; k++) {
        b.min[k] = hb[k] - 1.0f;
        b.max[k] = hb[3 + k] + 1.0f;
      }
      PgaLbvh out = {e->dColNodes, e->dColParents, e->dColAabbs, e->dColLeaf, e->dColKeys};
      const PgaStatus st = pga_lbvh_build(e, e->dColRec, visible, &b, &out, s);
      if (st != PGA_OK) return st;
    }
  }
  e->phaseTerminals = total;
  if (dCount) {
    e->phaseTerminalsHost = total;
    PGA_CUDA_TRY(cudaMemcpyAsync(dCount, &e->phaseTerminalsHost, sizeof(uint64_t), cudaMemcpyHostToDevice, s));
    PGA_CUDA_TRY(cudaStreamSynchronize(s));
  }
  e->lastAxioms = dAxioms;
  e->lastNumAxioms = numAxioms;
  e->lastBlocks = dBlocks;
  e->lastOut = dOut;
  e->lastCap = capacity;
  e->lastWasBatched = true;
  return PGA_OK;
}

extern "C" {

PgaStatus pga_derive(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t numAxioms, const float* dParamBlocks,
                     PgaTerminal* dOut, uint64_t capacity, uint64_t* dCount, void* stream) {
  if (!e || (!dAxioms && numAxioms) || (!dOut && capacity)) {
    set_error("pga_derive: null engine or buffers");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (e->phased) return derive_phases(e, dAxioms, numAxioms, dParamBlocks, dOut, capacity, dCount, (cudaStream_t)stream);
  const uint32_t* order = nullptr;
  const PgaStatus st = group_axioms(e, dAxioms, numAxioms, (cudaStream_t)stream, &order);
  if (st != PGA_OK) return st;
  return launch_persistent(e, dAxioms, 0, numAxioms, dParamBlocks, dOut, capacity, dCount, (cudaStream_t)stream, order);
}

// Grows an engine-owned device buffer (kept until the engine is destroyed).
static cudaError_t ensure_buffer(void** p, size_t* have, size_t need) {
  if (*have >= need && *p) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  cudaError_t err = cudaMalloc(p, need);
  if (err == cudaSuccess) *have = need;
  return err;
}

PgaStatus pga_derive_to_host(PgaEngine* e, const PgaAxiom* hAxioms, uint32_t numAxioms, const float* dParamBlocks,
                             PgaTerminal* hOut, uint64_t capacity, uint64_t* hCount, void* stream) {
  if (!e || (!hAxioms && numAxioms) || (!hOut && capacity) || !hCount) {
    set_error("pga_derive_to_host: null engine, buffers or count");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (e->phased) {
    set_error("pga_derive_to_host: a multi-phase table (phases, Collider, IfCollides) needs pga_derive");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  *hCount = 0;
  PGA_CUDA_TRY(ensure_buffer((void**)&e->dStageAxioms, &e->stageAxiomBytes, std::max<size_t>(numAxioms, 1) * sizeof(PgaAxiom)));
  PGA_CUDA_TRY(ensure_buffer((void**)&e->dStageOut, &e->stageOutBytes, std::max<uint64_t>(capacity, 1) * sizeof(PgaTerminal)));
  PGA_CUDA_TRY(ensure_buffer((void**)&e->dStageCount, &e->stageCountBytes, sizeof(uint64_t)));
  if (!e->copyStream) PGA_CUDA_TRY(cudaStreamCreateWithFlags(&e->copyStream, cudaStreamNonBlocking));
  if (!e->evDerived) PGA_CUDA_TRY(cudaEventCreateWithFlags(&e->evDerived, cudaEventDisableTiming));
  if (numAxioms == 0) return PGA_OK;
  PGA_CUDA_TRY(cudaMemcpyAsync(e->dStageAxioms, hAxioms, (size_t)numAxioms * sizeof(PgaAxiom), cudaMemcpyHostToDevice, s));
  // A small first range gets the copy engine going early; the rest follows in
  // three equal ranges, each derived while the previous one is copied out.
  uint32_t bounds[5];
  uint32_t nr = 0;
  bounds[nr++] = 0;
  if (numAxioms >= 64) {
    const uint32_t first = std::max<uint32_t>(numAxioms / 16, 1);
    bounds[nr++] = first;
    for (uint32_t k = 1; k <= 3; k++) bounds[nr++] = first + (uint32_t)((uint64_t)(numAxioms - first) * k / 3);
  } else {
    bounds[nr++] = numAxioms;
  }
  uint64_t offset = 0;
  PgaStatus status = PGA_OK;
  for (uint32_t r = 0; r + 1 < nr && status == PGA_OK; r++) {
    if (bounds[r + 1] == bounds[r]) continue;
    PgaStatus st = launch_persistent(e, e->dStageAxioms, bounds[r], bounds[r + 1], dParamBlocks, e->dStageOut + offset,
                                     capacity - offset, e->dStageCount, s);
    if (st != PGA_OK) {
      status = st;
      break;
    }
    PgaDeriveReport rep;
    st = pga_engine_sync_report(e, s, &rep);  // waits for this range; OUTPUT_OVERFLOW past the capacity left
    const uint64_t n = std::min<uint64_t>(rep.terminals, capacity - offset);
    if (n) {
      PGA_CUDA_TRY(cudaEventRecord(e->evDerived, s));
      PGA_CUDA_TRY(cudaStreamWaitEvent(e->copyStream, e->evDerived, 0));
      PGA_CUDA_TRY(cudaMemcpyAsync(hOut + offset, e->dStageOut + offset, n * sizeof(PgaTerminal), cudaMemcpyDeviceToHost,
                                   e->copyStream));
    }
    if (st != PGA_OK) {
      *hCount = offset + rep.terminals;
      status = st;
      break;
    }
    offset += n;
    *hCount = offset;
  }
  PGA_CUDA_TRY(cudaStreamSynchronize(e->copyStream));
  e->lastWasBatched = false;  // the staging ranges leave no tape for pga_adjoint
  return status;
}

}  // extern "C"

// Bookkeeping of pga_derive_per_axiom between two launches.  The launch that
// just finished left its records at stage[0, st->termCount) and its status in
// *st.  Append the records at out[*countIn, ...) (what fits below cap), write
// *countOut = *countIn + termCount (the two counters alternate, so no block
// reads the word another block writes), keep the first nonzero status in
// book[2] (status << 32 | detail) and add the launch's queued items to book[3].
__global__ void k_append_axiom(const DevState* st, const PgaTerminal* stage, unsigned long long stageCap,
                               PgaTerminal* out, unsigned long long cap, const unsigned long long* countIn,
                               unsigned long long* countOut, unsigned long long* book) {
  const unsigned long long base = *countIn;
  const unsigned long long n = ((const volatile DevState*)st)->termCount;
  const unsigned long long m = min(n, stageCap);
  const unsigned long long fit = base < cap ? min(m, cap - base) : 0ull;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < fit;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const uint4* from = reinterpret_cast<const uint4*>(stage + i);
    uint4* to = reinterpret_cast<uint4*>(out + base + i);
    uint4 r[4];
#pragma unroll
    for (int q = 0; q < 4; q++) r[q] = __ldcs(from + q);
#pragma unroll
    for (int q = 0; q < 4; q++) __stcs(to + q, r[q]);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *countOut = base + n;
    int status = ((const volatile DevState*)st)->status, detail = ((const volatile DevState*)st)->detail;
    if (status == 0 && n > stageCap) status = PGA_ERR_OUTPUT_OVERFLOW;
    if (status != 0 && book[2] == 0) book[2] = ((unsigned long long)(uint32_t)status << 32) | (uint32_t)detail;
    book[3] += ((const volatile DevState*)st)->nodeNext;
  }
}

// The end of pga_derive_per_axiom: the whole sequence's count, first status
// and items go into the engine state (for pga_engine_sync_report) and *dCount.
__global__ void k_finish_per_axiom(DevState* st, const unsigned long long* count, const unsigned long long* book,
                                   unsigned long long* dCount) {
  st->termCount = *count;
  st->nodeNext = book[3];
  if (book[2] != 0) {
    st->status = (int32_t)(book[2] >> 32);
    st->detail = (int32_t)(uint32_t)book[2];
  }
  if (dCount) *dCount = *count;
}

extern "C" {

PgaStatus pga_derive_per_axiom(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t numAxioms, const float* dParamBlocks,
                               PgaTerminal* dOut, uint64_t capacity, uint64_t* dCount, void* stream) {
  if (!e || (!dAxioms && numAxioms) || (!dOut && capacity)) {
    set_error("pga_derive_per_axiom: null engine or buffers");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (e->phased) {
    set_error("pga_derive_per_axiom: a multi-phase table (phases, Collider, IfCollides) needs pga_derive");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PGA_CUDA_TRY(ensure_buffer((void**)&e->dStageOut, &e->stageOutBytes, std::max<uint64_t>(capacity, 1) * sizeof(PgaTerminal)));
  PGA_CUDA_TRY(ensure_buffer((void**)&e->dStageCount, &e->stageCountBytes, 4 * sizeof(uint64_t)));
  unsigned long long* book = reinterpret_cast<unsigned long long*>(e->dStageCount);
  PGA_CUDA_TRY(cudaMemsetAsync(book, 0, 4 * sizeof(uint64_t), s));
  const uint64_t stageCap = e->stageOutBytes / sizeof(PgaTerminal);
  for (uint32_t ax = 0; ax < numAxioms; ax++) {
    const PgaStatus st = launch_persistent(e, dAxioms, ax, ax + 1, dParamBlocks, e->dStageOut, stageCap, nullptr, s);
    if (st != PGA_OK) return st;
    k_append_axiom<<<64, 256, 0, s>>>(e->dState, e->dStageOut, stageCap, dOut, capacity, book + (ax & 1),
                                      book + ((ax + 1) & 1), book);
    PGA_CUDA_TRY(cudaGetLastError());
  }
  if (numAxioms == 0) PGA_CUDA_TRY(cudaMemsetAsync(e->dState, 0, sizeof(DevState), s));
  k_finish_per_axiom<<<1, 1, 0, s>>>(e->dState, book + (numAxioms & 1), book, (unsigned long long*)dCount);
  PGA_CUDA_TRY(cudaGetLastError());
  e->lastCap = capacity;
  e->lastWasBatched = false;  // no tape for pga_adjoint
  return PGA_OK;
}

PgaStatus pga_derive_plain(PgaEngine* e, const PgaAxiom* dAxioms, uint32_t numAxioms, const float* dParamBlocks,
                           PgaTerminal* dOut, uint64_t capacity, uint64_t* dCount, void* stream) {
  if (!e || (!dAxioms && numAxioms) || (!dOut && capacity)) {
    set_error("pga_derive_plain: null engine or buffers");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (e->phased) {
    set_error("pga_derive_plain: a multi-phase table (phases, Collider, IfCollides) needs pga_derive");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  PGA_CUDA_TRY(cudaMemsetAsync(e->dState, 0, sizeof(DevState), s));
  DeriveArgs a = make_args(e, dAxioms, numAxioms, dParamBlocks, dOut, capacity, (unsigned long long*)dCount);
  a.termLinks = nullptr;
  const unsigned threads = (unsigned)e->threads;
  for (uint32_t ax = 0; ax < numAxioms; ax++) {
    // One grammar (axiom) at a time: reset the queue, seed, expand level by level.
    PGA_CUDA_TRY(cudaMemsetAsync(&e->dState->nodeNext, 0, sizeof(unsigned long long), s));
    {
      uint32_t first = ax, count = 1;
      void* args[] = {&a, &first, &count};
      PGA_CUDA_TRY(cudaLaunchKernel(e->kernels.seed, dim3(1), dim3(threads), args, e->smemBytes, s));
    }
    unsigned long long lo = 0, hi = 0;
    int32_t status = 0;
    for (uint32_t level = 0;; level++) {
      DevState snap;
      PGA_CUDA_TRY(cudaMemcpyAsync(&snap, e->dState, sizeof(DevState), cudaMemcpyDeviceToHost, s));
      PGA_CUDA_TRY(cudaStreamSynchronize(s));
      status = snap.status;
      hi = std::min<unsigned long long>(snap.nodeNext, e->cfg.nodeCapacity);
      if (status != 0 || hi == lo) break;
      if (level >= e->cfg.maxLevels) {
        set_error("pga_derive_plain: maxLevels exceeded");
        return PGA_ERR_DEPTH;
      }
      unsigned long long n = hi - lo;
      unsigned long long blocks = (n + threads - 1) / threads;
      {
        void* args[] = {&a, &lo, &hi};
        PGA_CUDA_TRY(cudaLaunchKernel(e->kernels.expand, dim3((unsigned)blocks), dim3(threads), args, e->smemBytes, s));
      }
      lo = hi;
    }
    if (status != 0) break;
  }
  e->lastCap = capacity;
  if (dCount) {
    k_write_count<<<1, 1, 0, s>>>(e->dState, (unsigned long long*)dCount);
    PGA_CUDA_TRY(cudaGetLastError());
  }
  PGA_CUDA_TRY(cudaStreamSynchronize(s));
  e->lastWasBatched = false;
  return PGA_OK;
}

PgaStatus pga_engine_sync_report(PgaEngine* e, void* stream, PgaDeriveReport* report) {
  if (!e || !report) return PGA_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  DevState snap;
  PGA_CUDA_TRY(cudaMemcpyAsync(&snap, e->dState, sizeof(DevState), cudaMemcpyDeviceToHost, s));
  PGA_CUDA_TRY(cudaStreamSynchronize(s));
  memset(report, 0, sizeof *report);
  if (e->phased) snap.termCount = e->phaseTerminals;  // over all phases
  // Terminals past the caller's capacity were dropped (never wrapped around):
  // that is an output overflow, reported with the full count.
  if (snap.status == 0 && snap.termCount > e->lastCap) snap.status = PGA_ERR_OUTPUT_OVERFLOW;
  report->status = snap.status;
  report->detail = snap.detail;
  report->terminals = snap.termCount;
  report->nodes = snap.nodeNext;
  report->levels = snap.levels;
  report->maxLevelNodes = snap.maxLevelNodes;
  return (PgaStatus)snap.status;
}

PgaStatus pga_engine_levels(PgaEngine* e, void* stream, uint64_t* starts, uint64_t* nanos, uint32_t capacity,
                            uint32_t* numLevels) {
  if (!e || !numLevels) return PGA_ERR_INVALID_ARGUMENT;
  cudaStream_t s = (cudaStream_t)stream;
  DevState snap;
  PGA_CUDA_TRY(cudaMemcpyAsync(&snap, e->dState, sizeof(DevState), cudaMemcpyDeviceToHost, s));
  PGA_CUDA_TRY(cudaStreamSynchronize(s));
  uint32_t n = std::min<uint32_t>(snap.levels + 1, e->cfg.maxLevels + 1);
  *numLevels = n;
  uint32_t k = std::min(n, capacity);
  if (k && starts) PGA_CUDA_TRY(cudaMemcpy(starts, e->dLevelStart, k * sizeof(uint64_t), cudaMemcpyDeviceToHost));
  if (nanos && capacity) {
    nanos[0] = snap.clockStart;
    const uint32_t kc = std::min(n, capacity - 1);
    if (kc) PGA_CUDA_TRY(cudaMemcpy(nanos + 1, e->dLevelClock, kc * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (n + 1 < capacity) nanos[n + 1] = snap.clockEnd;
  }
  return PGA_OK;
}

}  // extern "C"

#include "adjoint.cuh"
