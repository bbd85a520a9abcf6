// Test infrastructure (a checker), never part of the product.
//
// Harness around the reference's OWN host-side derivation path:
// PGA::CPU::SinglePhaseEvaluator (include/pga/core/CPUEvaluator.h:393-459)
// running the reference's __host__ __device__ operator templates on the CPU.
// It is compiled by oracle/make_ref.py against a patched shadow copy of the
// reference headers (oracle/_ref/shadow, git-ignored).
//
// Input  (argv[1]): a grammar batch, format written by
//                   operatorgraph_gb300/grammar.py::write_batch_file
// Output (argv[2]): terminal records, 64 B each (same layout as PgaTerminal in
//                   include/pga_gb300.h).  The path hash is the one oracle/make_ref.py
//                   instruments the reference's child-creation call sites with.
// argv[3] (optional): number of timed repetitions of execute().
// Options after the positional arguments:
//   --axiom-base B   axiom k of the batch is axiom B + k for its root path hash
//                    (a shard of a larger batch hashes like the whole batch)
//   --entry-mod E    child entry indices are hashed modulo E (a batch that gives
//                    each axiom its own copy of an E-entry table hashes like the
//                    one shared table)
//   --no-output      keep the terminals in memory but write no terminal file
//                    (timing runs: only execute() is timed either way)
//
// ref_harness --collide <pairs.bin> <out.bin> runs the reference's collision
// predicate PGA::ContextSensitivity::Collision::check (Collision.cuh) on shape
// pairs instead: per pair two uint32 kinds (0 box, 1 quad), then for A and B a
// row-major 3x4 model and a size (15 floats each); out: one byte per pair.
// When the grammar has triangle-mesh terminals (Generate<false, 0, ...>), their
// meshes go to argv[2] + ".mesh": "PGAM", mesh count, then per mesh the vertex
// and index counts, the vertices (48 B each, TriangleMeshData::VertexAttributes
// layout) and the indices, in the order the reference wrote them.
//
// The procedure list is the generic "interpreter style" list: one procedure per
// (operator, shape) with every argument a DynParam and every successor a DCall,
// as in src/interpreter/PGAFacade.cu and src/test_runner/MengerSponge.cuh:28-33.
// Its indices are the operator codes that the grammar batch uses and that
// pga_default_procs() in the product exposes.
#define PGA_CORE_EXPORT 0
#include <cuda_runtime_api.h>
#include <pga/core/CPUEvaluator.h>
#include <pga/core/ComponentSplit.cuh>
#include <pga/core/Discard.cuh>
#include <pga/core/DispatchTable.h>
#include <pga/core/Extrude.cuh>
#include <pga/core/Generate.cuh>
#include <pga/core/If.cuh>
#include <pga/core/Proc.cuh>
#include <pga/core/RandomRule.cuh>
#include <pga/core/Repeat.cuh>
#include <pga/core/Replicate.cuh>
#include <pga/core/Rotate.cuh>
#include <pga/core/Scale.cuh>
#include <pga/core/SwapSize.cuh>
#include <pga/core/ShapeGenerator.cuh>
#include <pga/core/Subdivide.cuh>
#include <pga/core/TStdLib.h>
#include <pga/core/Translate.cuh>
#include <pga/core/Collision.cuh>
#include <pga/rendering/ShapeMeshAttributes.cuh>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace PGA;
using namespace PGA::Operators;
using namespace PGA::Shapes;
using namespace PGA::Parameters;

struct HarnessFilter;

struct HarnessTerminal {
  float m[12];
  uint32_t rule;
  float custom;
  uint64_t path;
};
static_assert(sizeof(HarnessTerminal) == 64, "terminal record must be 64 B");

static std::vector<HarnessTerminal> g_terminals;

template <typename ShapeT> struct IsQuadShape { static const uint32_t value = 0; };
template <> struct IsQuadShape<Quad> { static const uint32_t value = 1; };

namespace PGA {
// Instanced terminal emission, mirroring GenerationFunction<GenFuncFilter, 1>::perShape
// (include/pga/rendering/GenerationFunctions.cuh:158-188): model4 * scale(size)
// (kept row-major here, not transposed) plus the custom attribute (attr1).
template <> struct GenerationFunction<HarnessFilter, 1> {
  template <typename ShapeT, typename... ArgsT>
  static void perShape(ShapeT& shape, unsigned int terminalIndex, float attr1, ArgsT...) {
    math::float4x4 M = shape.getModel4() * math::float4x4::scale(shape.getSize());
    HarnessTerminal t;
    t.m[0] = M._11; t.m[1] = M._12; t.m[2] = M._13; t.m[3] = M._14;
    t.m[4] = M._21; t.m[5] = M._22; t.m[6] = M._23; t.m[7] = M._24;
    t.m[8] = M._31; t.m[9] = M._32; t.m[10] = M._33; t.m[11] = M._34;
    // The shape handed to perShape is the base sub-object of the Symbol that
    // Generate dispatched (CPUEvaluator.h:268-276), so its entry index is
    // reachable through the derived type.
    int entry = static_cast<Symbol<ShapeT>&>(shape).entryIndex;
    t.rule = (uint32_t(entry) & 0xFFFFFFu) | ((terminalIndex & 0x7Fu) << 24) | (IsQuadShape<ShapeT>::value << 31);
    t.custom = attr1;
    t.path = static_cast<Symbol<ShapeT>&>(shape).pathHash;
    g_terminals.push_back(t);
  }
  template <typename ShapeT, typename... ArgsT> static unsigned int allocateVertices(ShapeT&, unsigned int, ArgsT...) { return 0; }
  template <typename... ArgsT> static void perVertex(unsigned int, const math::float4&, const math::float3&, const math::float2&, unsigned int, ArgsT...) {}
  template <typename ShapeT, typename... ArgsT> static unsigned int allocateIndices(ShapeT&, unsigned int, ArgsT...) { return 0; }
  template <typename... ArgsT> static void perTriangle(unsigned int, unsigned int, unsigned int, unsigned int, unsigned int, ArgsT...) {}
};

// Triangle meshes, mirroring GenerationFunction<GenFuncFilter, 0>
// (GenerationFunctions.cuh:41-153) on the host side: vertex and index space
// taken in order, the vertex attributes and triangles the reference's
// ShapeGenerator computes stored as given.  perShape also records the
// terminal, so that the derivation itself is compared for these rules too.
struct HarnessMesh {
  std::vector<float> vertices;  // 12 floats per vertex
  std::vector<uint32_t> indices;
};
static std::vector<HarnessMesh> g_meshes;

template <> struct GenerationFunction<HarnessFilter, 0> {
  static HarnessMesh& mesh(unsigned int terminalIndex) {
    if (terminalIndex >= g_meshes.size()) g_meshes.resize(terminalIndex + 1);
    return g_meshes[terminalIndex];
  }
  template <typename ShapeT, typename... ArgsT>
  static void perShape(ShapeT& shape, unsigned int terminalIndex, float attr1, ArgsT... args) {
    GenerationFunction<HarnessFilter, 1>::perShape(shape, terminalIndex, attr1, args...);
  }
  template <typename ShapeT, typename... ArgsT>
  static unsigned int allocateVertices(ShapeT& shape, unsigned int terminalIndex, ArgsT...) {
    HarnessMesh& m = mesh(terminalIndex);
    const unsigned int i = (unsigned int)(m.vertices.size() / 12);
    m.vertices.resize(m.vertices.size() + 12 * Rendering::ShapeMeshAttributes<ShapeT>::getNumVertices(shape), 0.0f);
    return i;
  }
  template <typename... ArgsT>
  static void perVertex(unsigned int vertexIndex, const math::float4& vertex, const math::float3& normal,
                        const math::float2& uv, unsigned int terminalIndex, ArgsT...) {
    float* v = &mesh(terminalIndex).vertices[(size_t)vertexIndex * 12];
    v[0] = vertex.x; v[1] = vertex.y; v[2] = vertex.z; v[3] = vertex.w;
    v[4] = normal.x; v[5] = normal.y; v[6] = normal.z;
    v[7] = uv.x; v[8] = uv.y;
  }
  template <typename ShapeT, typename... ArgsT>
  static unsigned int allocateIndices(ShapeT& shape, unsigned int terminalIndex, ArgsT...) {
    HarnessMesh& m = mesh(terminalIndex);
    const unsigned int i = (unsigned int)m.indices.size();
    m.indices.resize(m.indices.size() + Rendering::ShapeMeshAttributes<ShapeT>::getNumIndices(shape), 0u);
    return i;
  }
  template <typename... ArgsT>
  static void perTriangle(unsigned int index, unsigned int v0, unsigned int v1, unsigned int v2,
                          unsigned int terminalIndex, ArgsT...) {
    uint32_t* d = &mesh(terminalIndex).indices[index];
    d[0] = v0; d[1] = v1; d[2] = v2;
  }
};
}  // namespace PGA

// Operator codes 0..35 (see pga_default_procs() in include/pga_gb300.h).
struct HarnessProcs : T::List<
  /* 0 */ Proc<Box, Subdivide<DynParams>, 1>,
  /* 1 */ Proc<Quad, Subdivide<DynParams>, 1>,
  /* 2 */ Proc<Box, Subdivide<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>, T::Pair<DynParam<3>, DCall<2>>>, 1>,
  /* 3 */ Proc<Quad, Subdivide<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>, T::Pair<DynParam<3>, DCall<2>>>, 1>,
  /* 4 */ Proc<Box, Repeat<false, DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 5 */ Proc<Quad, Repeat<false, DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 6 */ Proc<Box, ComponentSplit<false, DCall<0>, DCall<1>, DCall<2>>, 1>,
  /* 7 */ Proc<Quad, Extrude<DynParam<0>, DynParam<1>, DCall<0>>, 1>,
  /* 8 */ Proc<Box, IfSizeLess<DynParam<0>, DynParam<1>, DCall<0>, DCall<1>>, 1>,
  /* 9 */ Proc<Quad, IfSizeLess<DynParam<0>, DynParam<1>, DCall<0>, DCall<1>>, 1>,
  /* 10 */ Proc<Box, Generate<false, 1, DynParam<0>>, 1>,
  /* 11 */ Proc<Quad, Generate<false, 1, DynParam<0>>, 1>,
  /* 12 */ Proc<Box, Discard, 1>,
  /* 13 */ Proc<Quad, Discard, 1>,
  /* 14 */ Proc<Box, Translate<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 15 */ Proc<Quad, Translate<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 16 */ Proc<Box, Scale<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 17 */ Proc<Quad, Scale<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 18 */ Proc<Box, RandomRule<DynParams>, 1>,
  /* 19 */ Proc<Quad, RandomRule<DynParams>, 1>,
  /* 20 */ Proc<Box, Rotate<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 21 */ Proc<Quad, Rotate<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 22 */ Proc<Box, Replicate<DynParams>, 1>,
  /* 23 */ Proc<Quad, Replicate<DynParams>, 1>,
  /* 24 */ Proc<Box, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>>, 1>,
  /* 25 */ Proc<Quad, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>>, 1>,
  /* 26 */ Proc<Box, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                T::Pair<DynParam<3>, DCall<2>>>, 1>,
  /* 27 */ Proc<Quad, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                 T::Pair<DynParam<3>, DCall<2>>>, 1>,
  /* 28 */ Proc<Box, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                T::Pair<DynParam<3>, DCall<2>>, T::Pair<DynParam<4>, DCall<3>>>, 1>,
  /* 29 */ Proc<Quad, RandomRule<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                 T::Pair<DynParam<3>, DCall<2>>, T::Pair<DynParam<4>, DCall<3>>>, 1>,
  /* 30 */ Proc<Box, If<DynParam<0>, DCall<0>, DCall<1>>, 1>,
  /* 31 */ Proc<Quad, If<DynParam<0>, DCall<0>, DCall<1>>, 1>,
  /* 32 */ Proc<Box, SwapSize<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 33 */ Proc<Quad, SwapSize<DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
  /* 34 */ Proc<Box, Generate<false, 0, DynParam<0>>, 1>,
  /* 35 */ Proc<Quad, Generate<false, 0, DynParam<0>>, 1>
> {};

#pragma pack(push, 1)
struct FileHeader { char magic[4]; uint32_t version, nEntries, nAxioms; };
struct FileParam { int32_t type; float value[16]; };
struct FileSucc { int32_t entry, phase; };
struct FileEntry { int32_t opcode; uint32_t nParams, nSucc, pad; FileParam params[17]; FileSucc succ[20]; };
struct FileAxiom { float position[3]; float seed; float size[3]; float custom; uint32_t entry, shape, block, flags; };
#pragma pack(pop)
static_assert(sizeof(FileEntry) == 1332, "entry size");
static_assert(sizeof(FileAxiom) == 48, "axiom size");

static std::vector<FileAxiom> g_axioms;
static unsigned long long g_axiomBase = 0;

struct HarnessAxioms {
  static unsigned int getNumAxioms() { return (unsigned int)g_axioms.size(); }
  template <typename SymbolManagerT, typename QueueT>
  static void generateAxiom(int id, QueueT* queue) {
    const FileAxiom& a = g_axioms[id];
    PathHash::currentAxiom() = g_axiomBase + (unsigned long long)id;
    if (a.shape == 1) {
      Quad q;
      q.setSize(math::float3(a.size[0], a.size[1], a.size[2]));
      q.setPosition(math::float3(a.position[0], a.position[1], a.position[2]));
      q.setSeed(a.seed);
      q.setCustomAttribute(a.custom);
      SymbolManagerT::dispatchAxiom(q, (int)a.entry, queue);
    } else {
      Box b;
      b.setSize(math::float3(a.size[0], a.size[1], a.size[2]));
      b.setPosition(math::float3(a.position[0], a.position[1], a.position[2]));
      b.setSeed(a.seed);
      b.setCustomAttribute(a.custom);
      SymbolManagerT::dispatchAxiom(b, (int)a.entry, queue);
    }
  }
};

template <typename ShapeT>
static ShapeT make_shape(const float* m, const float* size) {
  ShapeT s;
  s.setModel(math::float3x4(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], m[9], m[10], m[11]));
  s.setSize(math::float3(size[0], size[1], size[2]));
  return s;
}

static int collide_main(const char* in, const char* outPath) {
  FILE* f = fopen(in, "rb");
  if (!f) { perror("open pairs"); return 2; }
  std::vector<uint8_t> results;
  struct Pair { uint32_t ka, kb; float ma[12], sa[3], mb[12], sb[3]; } p;
  static_assert(sizeof(Pair) == 128, "pair record");
  while (fread(&p, sizeof p, 1, f) == 1) {
    bool hit;
    using ContextSensitivity::Collision;
    if (p.ka == 0 && p.kb == 0) hit = Collision::check(make_shape<Box>(p.ma, p.sa), make_shape<Box>(p.mb, p.sb));
    else if (p.ka == 0) hit = Collision::check(make_shape<Box>(p.ma, p.sa), make_shape<Quad>(p.mb, p.sb));
    else if (p.kb == 0) hit = Collision::check(make_shape<Quad>(p.ma, p.sa), make_shape<Box>(p.mb, p.sb));
    else hit = Collision::check(make_shape<Quad>(p.ma, p.sa), make_shape<Quad>(p.mb, p.sb));
    results.push_back(hit ? 1 : 0);
  }
  fclose(f);
  FILE* o = fopen(outPath, "wb");
  if (!o) { perror("open output"); return 2; }
  fwrite(results.data(), 1, results.size(), o);
  fclose(o);
  printf("{\"pairs\": %zu}\n", results.size());
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 4 && strcmp(argv[1], "--collide") == 0) return collide_main(argv[2], argv[3]);
  std::vector<const char*> pos;
  bool writeOutput = true;
  for (int i = 1; i < argc; i++) {
    if (strcmp(argv[i], "--axiom-base") == 0 && i + 1 < argc) g_axiomBase = strtoull(argv[++i], nullptr, 10);
    else if (strcmp(argv[i], "--entry-mod") == 0 && i + 1 < argc) PathHash::entryModulus() = (unsigned)atoi(argv[++i]);
    else if (strcmp(argv[i], "--no-output") == 0) writeOutput = false;
    else pos.push_back(argv[i]);
  }
  if (pos.size() < 2) {
    fprintf(stderr, "usage: ref_harness <batch.bin> <terminals.bin> [repeats] [--axiom-base B] [--entry-mod E] [--no-output]\n");
    return 2;
  }
  int repeats = pos.size() > 2 ? atoi(pos[2]) : 1;
  FILE* f = fopen(pos[0], "rb");
  if (!f) { perror("open input"); return 2; }
  FileHeader h;
  if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, "PGAB", 4) != 0) { fprintf(stderr, "bad header\n"); return 2; }
  std::vector<FileEntry> entries(h.nEntries);
  g_axioms.resize(h.nAxioms);
  if (fread(entries.data(), sizeof(FileEntry), h.nEntries, f) != h.nEntries ||
      fread(g_axioms.data(), sizeof(FileAxiom), h.nAxioms, f) != h.nAxioms) {
    fprintf(stderr, "truncated input\n");
    return 2;
  }
  fclose(f);

  // Build the reference's own DispatchTableEntry array (DispatchTableEntry.h:8-36).
  std::vector<DispatchTableEntry> table(h.nEntries);
  for (uint32_t i = 0; i < h.nEntries; i++) {
    DispatchTableEntry& e = table[i];
    memset(&e, 0, sizeof e);
    e.operatorCode = entries[i].opcode;
    e.numParameters = entries[i].nParams;
    for (uint32_t p = 0; p < 17; p++) {
      e.parameters[p].type = (ParameterType)entries[i].params[p].type;
      for (int v = 0; v < 16; v++) e.parameters[p].value[v] = entries[i].params[p].value[v];
    }
    e.numSuccessors = entries[i].nSucc;
    for (uint32_t s = 0; s < 20; s++) {
      e.successors[s].entryIndex = s < entries[i].nSucc ? entries[i].succ[s].entry : -1;
      e.successors[s].phaseIndex = s < entries[i].nSucc ? entries[i].succ[s].phase : -1;
    }
    e.numEdgeIndices = 0;
    for (int s = 0; s < 20; s++) e.edgeIndices[s] = -1;
    e.subGraphIndex = -1;
  }

  std::vector<double> times;
  int rc = 0;
  for (int r = 0; r < repeats; r++) {
    g_terminals.clear();
    g_terminals.reserve(1 << 20);
    g_meshes.clear();
    CPU::SinglePhaseEvaluator<HarnessProcs, HarnessAxioms, HarnessFilter> ev;
    ev.initialize(table.data(), table.size());
    try {
      auto t0 = std::chrono::steady_clock::now();
      ev.execute();
      auto t1 = std::chrono::steady_clock::now();
      times.push_back(std::chrono::duration<double>(t1 - t0).count());
    } catch (const std::exception& ex) {
      fprintf(stderr, "reference threw: %s\n", ex.what());
      rc = 3;
    }
    ev.release();
    if (rc) break;
  }
  uint64_t n = g_terminals.size();
  if (writeOutput) {
    FILE* o = fopen(pos[1], "wb");
    if (!o) { perror("open output"); return 2; }
    fwrite("PGAT", 1, 4, o);
    uint32_t zero = 0;
    fwrite(&zero, 4, 1, o);
    fwrite(&n, 8, 1, o);
    fwrite(g_terminals.data(), sizeof(HarnessTerminal), n, o);
    fclose(o);
  }
  if (writeOutput && !g_meshes.empty()) {
    std::string mp = std::string(pos[1]) + ".mesh";
    FILE* mf = fopen(mp.c_str(), "wb");
    if (!mf) { perror("open mesh output"); return 2; }
    fwrite("PGAM", 1, 4, mf);
    uint32_t nm = (uint32_t)g_meshes.size();
    fwrite(&nm, 4, 1, mf);
    for (const HarnessMesh& m : g_meshes) {
      uint32_t nv = (uint32_t)(m.vertices.size() / 12), ni = (uint32_t)m.indices.size();
      fwrite(&nv, 4, 1, mf);
      fwrite(&ni, 4, 1, mf);
      fwrite(m.vertices.data(), sizeof(float), m.vertices.size(), mf);
      fwrite(m.indices.data(), sizeof(uint32_t), m.indices.size(), mf);
    }
    fclose(mf);
  }
  std::string all;  // in run order
  for (size_t k = 0; k < times.size(); k++) {
    char buf[32];
    snprintf(buf, sizeof buf, "%s%.9g", k ? ", " : "", times[k]);
    all += buf;
  }
  std::sort(times.begin(), times.end());
  double med = times.empty() ? 0.0 : times[times.size() / 2];
  printf("{\"terminals\": %llu, \"seconds\": %.9g, \"repeats\": %d, \"status\": %d, \"all_seconds\": [%s]}\n",
         (unsigned long long)n, med, (int)times.size(), rc, all.c_str());
  return rc;
}
