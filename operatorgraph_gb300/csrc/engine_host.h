// Host-side engine object shared by the translation units of libpga_gb300.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "engine.cuh"

struct PgaEngine {
  // Lowered rule table (device).
  pga::DevRule* dRules = nullptr;
  pga::DevParam* dParams = nullptr;
  int32_t* dSucc = nullptr;
  float* dExpPool = nullptr;
  uint32_t numEntries = 0;
  std::vector<pga::DevRule> hRules;
  std::vector<pga::DevParam> hParams;
  std::vector<int32_t> hSucc;
  std::vector<float> hExpPool;

  PgaEngineConfig cfg{};
  int device = 0;
  int numSMs = 0;
  int persistentBlocks = 0;
  int threads = 256;
  bool useSeeds = false;
  bool tableInSmem = false;
  size_t smemBytes = 0;

  // Work storage (allocated once in pga_engine_create).
  pga::DevState* dState = nullptr;
  pga::Node* dNodes = nullptr;
  float4* dNodeRot = nullptr;  // general frames: 2 float4 of rotation entries per work item
  // Multi-phase derivation (successor edges into later phases, Collider, IfCollides).
  bool phased = false;
  pga::Node* dDefer[2] = {nullptr, nullptr};   // shapes deferred to the next phase (input / output)
  float4* dDeferRot[2] = {nullptr, nullptr};
  PgaTerminal* dColRec = nullptr;              // colliders as records (LBVH input)
  float4* dColShape = nullptr;                 // colliders as oriented boxes (5 float4 each)
  int32_t* dColNodes = nullptr;                // the colliders' LBVH
  uint32_t* dColParents = nullptr;
  float* dColAabbs = nullptr;
  uint32_t* dColLeaf = nullptr;
  uint64_t* dColKeys = nullptr;
  unsigned long long* dPhaseCounters = nullptr;  // [0] colliders, [1] deferred, [2] terminals of a launch
  uint64_t colCap = 0;
  uint64_t phaseTerminals = 0;                 // terminals of the last multi-phase derivation
  uint64_t phaseTerminalsHost = 0;             // its copy for the device count
  uint32_t phasesRun = 0;
  uint2* dTermLinks = nullptr;
  unsigned long long* dLevelStart = nullptr;
  unsigned long long* dLevelClock = nullptr;
  unsigned long long* dScratchCount = nullptr;
  // Paged output: tail slots past the caller's capacity and compaction scratch.
  PgaTerminal* dTail = nullptr;
  uint2* dTailLinks = nullptr;
  unsigned long long tailCap = 0;
  unsigned long long* dScratch = nullptr;

  // LBVH scratch.
  void* dSortTemp = nullptr;
  size_t sortTempBytes = 0;
  unsigned long long* dKeysA = nullptr;
  uint32_t* dValsA = nullptr;
  uint32_t* dValsB = nullptr;
  uint32_t* dArrival = nullptr;
  float* dLeafAabb = nullptr;        // LBVH leaf boxes in terminal order
  float* dLeafAabbSorted = nullptr;  // the same in sorted (leaf) order
  int32_t* dNodeOther = nullptr;     // LBVH internal node i: the other end of its leaf range (one end is i)

  // Adjoint scratch: per work item the gradient of (translation, size), its
  // child key and the next page of the same child; the child slots (slotCap
  // of them); per block of the reverse launch its chunk's child count.
  float* dNodeGrad = nullptr;
  uint32_t* dChildKey = nullptr;
  uint32_t* dPageNext = nullptr;
  uint32_t* dSlots = nullptr;
  unsigned long long* dBlockSums = nullptr;
  unsigned long long slotCap = 0;

  // PGA_FLAG_GROUP_AXIOMS: per root entry (and one bucket for entries out of
  // range) its axiom count, then its next free place in the seed order.
  uint32_t* dGroupCount = nullptr;

  // Last pga_derive, for pga_adjoint.
  const PgaAxiom* lastAxioms = nullptr;
  uint32_t lastNumAxioms = 0;
  const float* lastBlocks = nullptr;
  PgaTerminal* lastOut = nullptr;
  unsigned long long lastCap = 0;
  bool leafKernel = false;  // launch the instantiation that expands leaf children in place
  bool affineKernel = false;  // the table has Translate / Scale / RandomRule / Rotate rules
  bool generalFrames = false;  // the table has Rotate rules: general-frame kernels (derive_gen.cu)
  pga::FrameKernels kernels{};  // the kernels of the engine's frame build
  bool lastWasBatched = false;
  int adjointBlocks = 0;  // grid of the cooperative adjoint launch (set on first use)
  // pga_derive_to_host staging (allocated on first use, grown as needed)
  PgaAxiom* dStageAxioms = nullptr;
  PgaTerminal* dStageOut = nullptr;
  uint64_t* dStageCount = nullptr;
  size_t stageAxiomBytes = 0, stageOutBytes = 0, stageCountBytes = 0;
  cudaStream_t copyStream = nullptr;
  cudaEvent_t evDerived = nullptr;
};

namespace pga {
void set_error(const std::string& msg);
PgaStatus cuda_status(cudaError_t e, const char* what);
DeriveArgs make_args(PgaEngine* e, const PgaAxiom* axioms, uint32_t numAxioms, const float* blocks,
                     PgaTerminal* out, unsigned long long cap, unsigned long long* count);
}  // namespace pga

#define PGA_CUDA_TRY(call)                                     \
  do {                                                         \
    cudaError_t _e = (call);                                   \
    if (_e != cudaSuccess) return pga::cuda_status(_e, #call); \
  } while (0)
