/*
 * pga_gb300.h -- C ABI of the GB300 derivation engine for PGA shape grammars.
 *
 * Plain C: pointers, sizes and POD structs only; streams are passed as
 * `void*` holding a cudaStream_t (0 = the legacy default stream).
 *
 * The data formats follow the reference's dispatch-table path so that a grammar
 * written for it runs unchanged:
 *   - PgaParameter / PgaSuccessor / PgaEntry  ~ PGA::DispatchTableEntry
 *     (include/pga/core/DispatchTableEntry.h:8-36), minus the instrumentation
 *     fields numEdgeIndices/edgeIndices/subGraphIndex, which the engine has no use for.
 *   - PgaProc ~ one Proc<ShapeT, OperatorT, NumThreadsT> of a procedure list
 *     (include/pga/core/Proc.cuh:19-27); an entry's operatorCode indexes the
 *     procedure list exactly as in the reference (CPUEvaluator.h:230-239,
 *     GPUEvaluator.cuh:194-211).
 *   - PgaTerminal ~ the instanced-mesh record written by
 *     GenerationFunction<GenFuncFilter, 1>::perShape
 *     (include/pga/rendering/GenerationFunctions.cuh:158-188): the model matrix
 *     model4 * scale(size) (row-major 3x4 here; the 4th row is always 0 0 0 1)
 *     plus the custom attribute, extended with the emitting rule and a
 *     derivation-path hash.
 */
#ifndef PGA_GB300_H
#define PGA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Limits of one dispatch-table entry (include/pga/core/GlobalConstants.h:9-14). */
#define PGA_MAX_NUM_PARAMETERS 17
#define PGA_MAX_NUM_PARAMETER_VALUES 16
#define PGA_MAX_NUM_SUCCESSORS 20
#define PGA_MAX_EXP_LEVELS 4

/* Parameter types: 0..5 are PGA::ParameterType (include/pga/core/ParameterType.h).
 * PGA_PT_BLOCK is an addition: value[0] is a slot in the axiom's parameter block
 * (per-axiom continuous parameters, the ones pga_adjoint differentiates). */
typedef enum PgaParameterType {
  PGA_PT_SCALAR = 0,
  PGA_PT_RAND = 1,
  PGA_PT_SHAPE_ATTR = 2,
  PGA_PT_EXP = 3,
  PGA_PT_VEC2 = 4,
  PGA_PT_VEC4 = 5,
  PGA_PT_BLOCK = 16
} PgaParameterType;

typedef struct PgaParameter {
  int32_t type;                                  /* PgaParameterType */
  float value[PGA_MAX_NUM_PARAMETER_VALUES];
} PgaParameter;                                  /* 68 B */

typedef struct PgaSuccessor {
  int32_t entryIndex;
  int32_t phaseIndex;                            /* single-phase engine: ignored */
} PgaSuccessor;

typedef struct PgaEntry {
  int32_t operatorCode;                          /* index into the procedure list */
  uint32_t numParameters;
  uint32_t numSuccessors;
  uint32_t reserved;
  PgaParameter parameters[PGA_MAX_NUM_PARAMETERS];
  PgaSuccessor successors[PGA_MAX_NUM_SUCCESSORS];
} PgaEntry;                                      /* 1332 B */

/* Operator kinds of the hot path (include/pga/core/{Subdivide,Repeat,
 * ComponentSplit,Extrude,If,Generate,Discard,Translate,Scale,RandomRule}.cuh). */
typedef enum PgaOperator {
  PGA_OP_SUBDIVIDE = 0,        /* Subdivide<DynParams>: axis = p0, factors = p1.., successor j for factor j+1 */
  PGA_OP_SUBDIVIDE_STATIC = 1, /* Subdivide<DynParam<0>, Pair<DynParam<k+1>, DCall<k>>...>: numChildren pairs, zero factors skipped */
  PGA_OP_REPEAT = 2,           /* Repeat<false, DynParam<0> axis, DynParam<1> extent, DynParam<2> mode, DCall<0>> */
  PGA_OP_COMPONENT_SPLIT = 3,  /* ComponentSplit<false, DCall<0> top, DCall<1> bottom, DCall<2> sides> (Box only) */
  PGA_OP_EXTRUDE = 4,          /* Extrude<DynParam<0> axis (unused), DynParam<1> extent, DCall<0>> (Quad -> Box) */
  PGA_OP_IF_SIZE_LESS = 5,     /* IfSizeLess<DynParam<0> axis, DynParam<1> size, DCall<0> true, DCall<1> false> */
  PGA_OP_GENERATE = 6,         /* Generate<false, 1, DynParam<0> terminal index>: instanced terminal */
  PGA_OP_DISCARD = 7,          /* Discard */
  PGA_OP_TRANSLATE = 8,        /* Translate<DynParam<0..2> x y z, DCall<0>>: model * translate(x, y, z), in place */
  PGA_OP_SCALE = 9,            /* Scale<DynParam<0..2>, DCall<0>>: per axis, v < 0 scales the size by -v, v > 0 sets it */
  PGA_OP_RANDOM_RULE = 10,     /* RandomRule<DynParams>: p0 chance (fractional part), p1.. weights, successor per weight */
  PGA_OP_ROTATE = 11,          /* Rotate<DynParam<0..2> degrees about x y z, DCall<0>>: model * rotateXYZ, in place;
                                  the angles must be scalars (the rotation is built once, at engine creation) */
  PGA_OP_REPLICATE = 12,       /* Replicate<DynParams>: the shape, unchanged, once per successor */
  PGA_OP_RANDOM_RULE_STATIC = 13 /* RandomRule<Chance, Pair<weight, successor>...> (the static form): p0 chance,
                                    p1.. weights; a zero weight is never picked and the last pair is taken when
                                    no other is (RandomRule.cuh:33-99) */,
  PGA_OP_IF = 14,              /* If<DynParam<0> condition, DCall<0> true, DCall<1> false>: nonzero is true */
  PGA_OP_SWAP_SIZE = 15,       /* SwapSize<DynParam<0..2> axes, DCall<0>>: size = (size[a0], size[a1], size[a2]) */
  PGA_OP_GENERATE_MESH = 16,   /* Generate<false, 0, DynParam<0> mesh index>: a triangle-mesh terminal; its record
                                  is written like an instanced one and pga_generate_meshes expands it */
  PGA_OP_COLLIDER = 17,        /* Collider<DynParam<0> tag, DCall<0>>: a tag > 0 stores the shape for IfCollides */
  PGA_OP_IF_COLLIDES = 18      /* IfCollides<DynParam<0> tag, DCall<0> true, DCall<1> false>: does a shape stored
                                  with the tag in an earlier phase overlap this one */
} PgaOperator;

typedef enum PgaShape { PGA_SHAPE_BOX = 0, PGA_SHAPE_QUAD = 1 } PgaShape;

/* One procedure of the procedure list: Proc<ShapeT, OperatorT, NumThreadsT>. */
typedef struct PgaProc {
  uint32_t op;           /* PgaOperator */
  uint32_t shape;        /* PgaShape the procedure expects */
  uint32_t numChildren;  /* PGA_OP_SUBDIVIDE_STATIC: number of Pair<> arguments; otherwise 0 */
  uint32_t numThreads;   /* NumThreadsT; accepted and ignored (one thread per shape) */
} PgaProc;

typedef struct PgaRuleTable {
  const PgaProc* procs;
  uint32_t numProcs;
  const PgaEntry* entries;
  uint32_t numEntries;
} PgaRuleTable;

/* One axiom. Rotation is the identity, as for the reference's axiom generators
 * (Grid.cuh:140-144, 199-204 set position, size, seed and custom attribute). */
typedef struct PgaAxiom {
  float position[3];
  float seed;
  float size[3];
  float custom;
  uint32_t entry;        /* root dispatch-table entry */
  uint32_t shape;        /* PgaShape; must match the root procedure's shape */
  uint32_t block;        /* parameter block used by PGA_PT_BLOCK parameters */
  uint32_t flags;        /* reserved, 0 */
} PgaAxiom;              /* 48 B */

/* One instanced terminal, 64 B, written with four 16-byte stores. */
typedef struct PgaTerminal {
  float m[12];           /* row-major 3x4 of model4 * scale(size) */
  uint32_t rule;         /* bits 0..23 entry of the Generate rule, bits 24..30 terminal (mesh) index, bit 31 = 1 for a Quad */
  float custom;          /* custom attribute (attr1 of the instanced generation function) */
  uint64_t path;         /* derivation-path hash */
} PgaTerminal;

/* PgaEngineConfig.flags.  By default a child whose rule is a Subdivide with
 * shape-independent factors and only constant-index Generate or Discard
 * successors is expanded by the thread that created it (its terminals written
 * at once) instead of being queued as a work item; engines with recordTape = 1
 * never do this.  PGA_FLAG_NO_INLINE turns it off. */
#define PGA_FLAG_NO_INLINE 1u
/* pga_derive seeds the axioms grouped by root entry (a counting sort on the
 * device before the launch) instead of in index order, so that warps expand
 * shapes of one grammar together, level after level.  Results are the same
 * records (each axiom keeps its index, hence its path hashes and parameter
 * block); only their order in the output changes.  For batches that mix
 * grammars; pga_derive_to_host and multi-phase tables (phases, Collider,
 * IfCollides) keep index order.  No reference counterpart. */
#define PGA_FLAG_GROUP_AXIOMS 2u
/* pga_derive hands out the last quarter of each wide level's work items (a
 * level of at least four rounds of warp chunks; at least two rounds are left)
 * from a shared per-level counter, one chunk per warp at a time, instead of in
 * the fixed grid-stride order, so that warps whose items had more children do
 * not hold the level's end.  A derivation that expands leaf children in place
 * (the default without recordTape, for tables with leaf rules) keeps the
 * fixed order.  The records are the same; their order in the output changes
 * from run to run.  (pga_adjoint hands out its wide levels this way with or
 * without the flag.)  No reference counterpart (the reference's queues are
 * dynamic throughout). */
#define PGA_FLAG_DYNAMIC_CHUNKS 4u

typedef struct PgaEngineConfig {
  uint64_t nodeCapacity;     /* non-terminal shapes held per derivation (queue storage) */
  uint64_t maxTerminals;     /* sizes the LBVH / adjoint scratch */
  uint32_t blockStride;      /* floats per parameter block (PGA_PT_BLOCK) */
  uint32_t threadsPerBlock;  /* 0 = default */
  uint32_t blocksPerSM;      /* 0 = occupancy maximum */
  uint32_t recordTape;       /* 1 = keep the derivation tape so pga_adjoint can run */
  uint32_t spinLimit;        /* iterations before a bounded wait gives up (0 = default) */
  uint32_t maxLevels;        /* derivation depth limit (0 = default 4096) */
  uint32_t flags;            /* PGA_FLAG_* */
  uint32_t subItem;          /* children per queued work item, 1..64 (0 = default 8) */
  uint32_t itemsPerLane;     /* work items per lane in one warp chunk (0 = default 1) */
  uint32_t narrowSubItem;    /* children per work item queued while the level being expanded has fewer
                                items than the grid has threads, 1..64 (0 = default) */
} PgaEngineConfig;


typedef enum PgaStatus {
  PGA_OK = 0,
  PGA_ERR_QUEUE_OVERFLOW = 1,   /* nodeCapacity too small */
  PGA_ERR_OUTPUT_OVERFLOW = 2,  /* terminal capacity too small (the count keeps counting) */
  PGA_ERR_TIMEOUT = 3,          /* a bounded wait ran out */
  PGA_ERR_BAD_OPCODE = 4,       /* operatorCode / entry index out of range, or shape mismatch */
  PGA_ERR_BAD_PARAM = 5,        /* an operator argument the reference rejects (e.g. Repeat extent <= 0) */
  PGA_ERR_CUDA = 6,             /* a CUDA runtime call failed */
  PGA_ERR_INVALID_ARGUMENT = 7, /* bad host-side argument */
  PGA_ERR_NO_TAPE = 8,          /* pga_adjoint without a recorded tape */
  PGA_ERR_DEPTH = 9,            /* maxLevels exceeded (likely a recursive grammar) */
  PGA_ERR_INTERNAL = 10         /* a bounds check of a checked build failed (detail = check site) */
} PgaStatus;

/* Result of the last derivation, read back by pga_engine_sync_report. */
typedef struct PgaDeriveReport {
  int32_t status;            /* PgaStatus raised on the device (first error wins) */
  int32_t detail;            /* entry index or level where it was raised */
  uint64_t terminals;        /* terminals emitted (may exceed capacity on overflow) */
  uint64_t nodes;            /* non-terminal shapes queued */
  uint32_t levels;           /* derivation levels run */
  uint32_t reserved;
  uint64_t maxLevelNodes;    /* largest level */
} PgaDeriveReport;

typedef struct PgaBounds { float min[3]; float max[3]; } PgaBounds;

/* LBVH over n terminals; every pointer is caller-owned device memory. */
typedef struct PgaLbvh {
  int32_t* nodes;            /* (n-1) x {parent, left, right}; child >= 0: leaf, < 0: -internal index (RadixTree.h:7-13) */
  uint32_t* leafParents;     /* n */
  float* aabbs;              /* (n-1) x {min xyz, max xyz} of internal nodes */
  uint32_t* leafTerminal;    /* n: terminal index of leaf i (sorted order) */
  uint64_t* keys;            /* n: sorted keys, morton30 << 34 | path >> 30 */
} PgaLbvh;

typedef struct PgaEngine PgaEngine;

/* Library version string. */
const char* pga_version(void);

/* Message of the last host-side failure in this thread. */
const char* pga_last_error(void);

/* The generic procedure list used by the reference's interpreter-style grammars
 * (src/interpreter/PGAFacade.cu, src/test_runner/MengerSponge.cuh:28-33),
 * every argument a DynParam and every successor a DCall. Operator codes:
 *   0 Box  Subdivide<DynParams>          1 Quad Subdivide<DynParams>
 *   2 Box  Subdivide, 3 static pairs     3 Quad Subdivide, 3 static pairs
 *   4 Box  Repeat                        5 Quad Repeat
 *   6 Box  ComponentSplit                7 Quad Extrude
 *   8 Box  IfSizeLess                    9 Quad IfSizeLess
 *  10 Box  Generate (instanced)         11 Quad Generate (instanced)
 *  12 Box  Discard                      13 Quad Discard
 *  14 Box  Translate                    15 Quad Translate
 *  16 Box  Scale                        17 Quad Scale
 *  18 Box  RandomRule<DynParams>        19 Quad RandomRule<DynParams>
 *  20 Box  Rotate                       21 Quad Rotate
 *  22 Box  Replicate<DynParams>         23 Quad Replicate<DynParams>
 *  24 Box  RandomRule, 2 static pairs   25 Quad RandomRule, 2 static pairs
 *  26 Box  RandomRule, 3 static pairs   27 Quad RandomRule, 3 static pairs
 *  28 Box  RandomRule, 4 static pairs   29 Quad RandomRule, 4 static pairs
 *  30 Box  If                           31 Quad If
 *  32 Box  SwapSize                     33 Quad SwapSize
 *  34 Box  Generate (triangle mesh)     35 Quad Generate (triangle mesh)
 *  36 Box  Collider                     37 Quad Collider
 *  38 Box  IfCollides                   39 Quad IfCollides */
const PgaProc* pga_default_procs(uint32_t* numProcs);

/* Replaces SinglePhaseEvaluator::initialize(DispatchTableEntry*, n)
 * (include/pga/core/GPUEvaluator.cuh:475-506, CPUEvaluator.h:444-451):
 * validates and lowers the table to the device rule table and allocates all
 * work storage. No later call allocates device memory, except the staging
 * buffers of pga_derive_to_host on its first use. */
PgaStatus pga_engine_create(const PgaRuleTable* table, const PgaEngineConfig* config, PgaEngine** engine);

/* Replaces SinglePhaseEvaluator::release() (GPUEvaluator.cuh:528-536). */
PgaStatus pga_engine_destroy(PgaEngine* engine);

/* Replaces SinglePhaseEvaluator::execute(numAxioms) (GPUEvaluator.cuh:508-521)
 * for the batched persistent engine: derives every axiom in one persistent
 * launch. dAxioms, dParamBlocks (may be NULL), dOut and dCount are device
 * pointers; *dCount receives the number of terminals. Asynchronous on
 * `stream`; capturable in a CUDA graph. */
PgaStatus pga_derive(PgaEngine* engine, const PgaAxiom* dAxioms, uint32_t numAxioms,
                     const float* dParamBlocks, PgaTerminal* dOut, uint64_t capacity,
                     uint64_t* dCount, void* stream);

/* SinglePhaseEvaluator::execute (GPUEvaluator.cuh:508-521) for callers whose
 * axioms and terminal buffer live in host memory (pinned memory is fastest):
 * copies the axioms in, derives them in four axiom ranges (a small first one,
 * then three equal ones) and copies each range's terminals out on a second
 * stream while the next range derives, so most of the derivation hides behind
 * the device-to-host copy.  Terminals are the same records as pga_derive's
 * (path hashes use absolute axiom indices), range after range.  dParamBlocks
 * stays a device pointer.  Returns when hOut holds *hCount terminals;
 * PGA_ERR_OUTPUT_OVERFLOW when they do not fit in capacity.  Its staging
 * buffers are allocated on first use and kept by the engine; it leaves no
 * tape for pga_adjoint. */
PgaStatus pga_derive_to_host(PgaEngine* engine, const PgaAxiom* hAxioms, uint32_t numAxioms,
                             const float* dParamBlocks, PgaTerminal* hOut, uint64_t capacity, uint64_t* hCount,
                             void* stream);

/* The plain GPU form: one axiom (grammar) per launch sequence, one kernel
 * launch per derivation level, the host reading the level size back each time.
 * Same outputs as pga_derive; synchronous. */
PgaStatus pga_derive_plain(PgaEngine* engine, const PgaAxiom* dAxioms, uint32_t numAxioms,
                           const float* dParamBlocks, PgaTerminal* dOut, uint64_t capacity,
                           uint64_t* dCount, void* stream);

/* SinglePhaseEvaluator::execute (GPUEvaluator.cuh:508-521) called once per
 * grammar, as a caller without batching would: one persistent launch per
 * axiom (the same kernel and schedule as pga_derive, each launch deriving one
 * axiom), the launches enqueued back to back on `stream` with no host
 * read-back, so the sequence can also be captured in a CUDA graph.  Each
 * launch derives into an engine staging buffer and a small copy kernel
 * appends its records at the running count, which lives on the device.  Same
 * records as pga_derive, in axiom order; *dCount gets the total.  The staging
 * buffer (capacity records) is allocated on first use and kept by the engine;
 * make the first call before any capture.  The first failing axiom's status
 * is reported by pga_engine_sync_report.  No tape for pga_adjoint. */
PgaStatus pga_derive_per_axiom(PgaEngine* engine, const PgaAxiom* dAxioms, uint32_t numAxioms,
                               const float* dParamBlocks, PgaTerminal* dOut, uint64_t capacity,
                               uint64_t* dCount, void* stream);

/* Synchronises `stream` and reports the device status of the last derivation:
 * PGA_ERR_OUTPUT_OVERFLOW when it produced more terminals than the capacity it
 * was given (report->terminals holds the full count; records past the
 * capacity were dropped, never wrapped around). */
PgaStatus pga_engine_sync_report(PgaEngine* engine, void* stream, PgaDeriveReport* report);

/* Per-level profile of the last pga_derive: starts[l] = first node of level l
 * (starts[l+1] its end) for up to `capacity` levels; device clock (ns)
 * nanos[0] = launch start, nanos[l + 1] = when level l's range was fixed (after
 * the axioms were seeded for l = 0), nanos[numLevels + 1] = launch end (after
 * the output compaction), as far as `capacity` entries reach; *numLevels
 * receives the level count.  Synchronises `stream`.  Counterpart of the
 * reference's per-subgraph clock instrumentation
 * (include/pga/core/Instrumentation.cuh:44-74). */
PgaStatus pga_engine_levels(PgaEngine* engine, void* stream, uint64_t* starts, uint64_t* nanos,
                            uint32_t capacity, uint32_t* numLevels);

/* Replaces ContextSensitivity::GPU::BVHConstructor::construct(min, max)
 * (include/pga/core/GPUBVHConstructor.cuh:265-331), applied to terminal boxes:
 * 30-bit Morton codes of the terminal centres in `bounds`, radix sort,
 * Karras topology and bottom-up AABB refit. `bounds` is a host pointer.
 * 2 <= n <= maxTerminals and n < 2^30. */
PgaStatus pga_lbvh_build(PgaEngine* engine, const PgaTerminal* dTerminals, uint64_t n,
                         const PgaBounds* bounds, const PgaLbvh* out, void* stream);

/* pga_lbvh_build (same construct(), GPUBVHConstructor.cuh:265-331) over the
 * first min(*dCount, capacity) terminals, with the count read on the device:
 * dCount is a device pointer, typically the one pga_derive wrote, so a
 * derivation, its LBVH and its adjoint can be captured in one CUDA graph with
 * no host read-back between them.  `capacity` (2 <= capacity <= maxTerminals,
 * below 2^30) sizes the launches and the radix sort, which orders `capacity`
 * keys: out->keys[count, capacity) holds padding (all ones) after the real
 * keys.  The tree and leaf arrays are those of pga_lbvh_build for `count`
 * leaves, bit for bit; a count below 2 builds no tree. */
PgaStatus pga_lbvh_build_counted(PgaEngine* engine, const PgaTerminal* dTerminals, const uint64_t* dCount,
                                 uint64_t capacity, const PgaBounds* bounds, const PgaLbvh* out, void* stream);

/* Same LBVH as pga_lbvh_build, for callers that cannot allocate device memory
 * (their budget is fixed up front, or the allocator belongs to a host
 * application): it needs no engine and calls no allocator.  Its scratch is a
 * fixed device array inside this library (6 MiB, held by every GPU that loads
 * the library until the process exits), so n is limited to
 * PGA_LBVH_STATIC_MAX_LEAVES; larger n (and n = 1) is rejected with
 * PGA_ERR_INVALID_ARGUMENT.  The first call on a device loads the library's
 * module there (which commits the array) and looks the array's device address
 * up: make it at start-up, before the device budget is handed out and before
 * any stream capture -- a call with n = 0 (pointers may be null) does only
 * that.  The address is cached for the life of the process, which assumes the
 * device's primary context is never reset.  Calls share the array and race
 * when they overlap on the GPU: serialise them on one stream.  No counterpart
 * in the reference. */
#define PGA_LBVH_STATIC_MAX_LEAVES 65536u
PgaStatus pga_lbvh_build_static(const PgaTerminal* dTerminals, uint64_t n, const PgaBounds* bounds,
                                const PgaLbvh* out, void* stream);

/* Adjoint of the last pga_derive (recordTape = 1): dGradTerminals holds
 * dL/dm (12 floats per terminal, same order as that derivation's output).
 * Accumulates dL/dDynParam into dGradParams (numBlocks x blockStride; may be NULL)
 * and dL/d(axiom size) into dGradAxiomSizes (3 per axiom; may be NULL).
 * Both outputs are overwritten, not added to.  One cooperative launch on
 * `stream`, asynchronous; if the last derivation failed or overflowed, the
 * gradients are zero and pga_engine_sync_report gives the status.  Engines
 * created with maxTerminals >= 2^23 launch a variant with more resident
 * blocks per SM (faster on large tapes, slower on small ones); the gradients
 * agree to FP32 accumulation order.  No reference counterpart. */
PgaStatus pga_adjoint(PgaEngine* engine, const float* dGradTerminals, float* dGradParams,
                      uint32_t numBlocks, float* dGradAxiomSizes, void* stream);

/* pga_adjoint with dL/dm of terminal t at dGradTerminals[t * gradStride + 0..11]
 * (gradStride >= 12 floats): a gradient kept inside a larger per-terminal
 * record -- for L = |m|^2 / 2, the terminal records themselves, stride 16.
 * pga_adjoint is this call with stride 12.  No reference counterpart. */
PgaStatus pga_adjoint_strided(PgaEngine* engine, const float* dGradTerminals, uint32_t gradStride,
                              float* dGradParams, uint32_t numBlocks, float* dGradAxiomSizes, void* stream);

/* One vertex of a generated triangle mesh: the layout of
 * PGA::Rendering::TriangleMeshData::VertexAttributes (16-byte aligned
 * position, normal and uv; include/pga/rendering/TriangleMeshData.h:10-18). */
typedef struct PgaVertex {
  float position[4];
  float normal[3];
  float uv[2];
  float pad[3];
} PgaVertex;

/* A triangle mesh being filled: the layout of PGA::Rendering::TriangleMeshData
 * (TriangleMeshData.h:19-27).  numVertices / numIndices are advanced
 * atomically by pga_generate_meshes and keep counting past the maxima. */
typedef struct PgaTriangleMesh {
  uint32_t numVertices, numIndices;
  uint32_t maxNumVertices, maxNumIndices;
  PgaVertex* vertices; /* device, maxNumVertices */
  uint32_t* indices;   /* device, maxNumIndices */
} PgaTriangleMesh;

/* Triangle-mesh generation, GenerationFunction<GenFuncFilter, 0> over
 * ShapeGenerator<Box> / <Quad> (include/pga/rendering/GenerationFunctions.cuh:41-153,
 * include/pga/core/ShapeGenerator.cuh:377-512, 671-708): for every record of
 * dTerminals whose rule is a triangle-mesh Generate (PGA_OP_GENERATE_MESH) of
 * this engine's table, appends to mesh dMeshes[mesh index] its vertices (24
 * for a Box: 6 faces x 4, 4 for a Quad) with the reference's positions,
 * normals and uvs (counter-clockwise), and its indices (two triangles per
 * face, absolute vertex numbers).  dMeshes is a DEVICE array of numMeshes
 * meshes (the reference's Device::TriangleMeshes).  Space is taken with one
 * atomic per mesh per warp, so the order of terminals in a mesh is not fixed
 * (the reference's atomics give no order either); a terminal's vertices and
 * indices are contiguous.  A mesh index >= numMeshes is PGA_ERR_BAD_PARAM; a
 * terminal that does not fit is not written (PGA_ERR_OUTPUT_OVERFLOW, the
 * counters keep counting; the reference wraps around instead).  Statuses
 * through pga_engine_sync_report.  One launch on `stream`, asynchronous. */
PgaStatus pga_generate_meshes(PgaEngine* engine, const PgaTerminal* dTerminals, uint64_t numTerminals,
                              PgaTriangleMesh* dMeshes, uint32_t numMeshes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PGA_GB300_H */
