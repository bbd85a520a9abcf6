// PGA::GB300::Evaluator (pga/engine.hpp) used the way the reference's test
// runner uses SinglePhaseEvaluator: initialize with the Menger procedure list
// and dispatch table, execute one axiom, read the terminals back.  Writes the
// terminal records to argv[1] for the Python test to compare with the oracle.
#include <pga/engine.hpp>

#include <cuda_runtime_api.h>

#include <cstdio>
#include <vector>

using namespace PGA;
using namespace PGA::Operators;
using namespace PGA::Parameters;
using namespace PGA::Shapes;

struct ProcedureList
    : T::List<Proc<Box, Subdivide<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                  T::Pair<DynParam<3>, DCall<2>>>, 1>,
              Proc<Box, Discard, 1>,
              Proc<Box, IfSizeLess<DynParam<0>, DynParam<1>, DCall<0>, DCall<1>>, 1>,
              Proc<Box, Generate<false, 1, DynParam<0>>, 1>> {};

#define CHECK_CUDA(x)                                                         \
  do {                                                                        \
    cudaError_t e_ = (x);                                                     \
    if (e_ != cudaSuccess) {                                                  \
      std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));           \
      return 1;                                                               \
    }                                                                         \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  using P = DispatchTable::Parameter;
  const P rel{PT_SCALAR, {-1}};
  const DispatchTable table{
      {2, {P{PT_SCALAR, {0}}, P{PT_SCALAR, {0.05}}}, {{1, 0}, {2, 0}}},
      {3, {P{PT_SCALAR, {0}}}, {}},
      {0, {P{PT_SCALAR, {0}}, rel, rel, rel}, {{3, 0}, {7, 0}, {3, 0}}},
      {0, {P{PT_SCALAR, {1}}, rel, rel, rel}, {{4, 0}, {5, 0}, {4, 0}}},
      {0, {P{PT_SCALAR, {2}}, rel, rel, rel}, {{0, 0}, {0, 0}, {0, 0}}},
      {0, {P{PT_SCALAR, {2}}, rel, rel, rel}, {{0, 0}, {6, 0}, {0, 0}}},
      {1, {}, {}},
      {0, {P{PT_SCALAR, {1}}, rel, rel, rel}, {{5, 0}, {8, 0}, {5, 0}}},
      {1, {}, {}},
  };
  PgaEngineConfig cfg = {};
  cfg.nodeCapacity = 1 << 16;
  cfg.maxTerminals = 1 << 16;
  GB300::Evaluator<ProcedureList> evaluator;
  PgaAxiom axiom = {};
  axiom.size[0] = axiom.size[1] = axiom.size[2] = 1.0f;
  axiom.seed = 0.5f;
  axiom.custom = 0.5f;
  axiom.entry = 0;
  axiom.shape = PGA_SHAPE_BOX;
  const uint64_t cap = 10000;
  PgaAxiom* dAxiom = nullptr;
  PgaTerminal* dOut = nullptr;
  uint64_t* dCount = nullptr;
  CHECK_CUDA(cudaMalloc((void**)&dAxiom, sizeof axiom));
  CHECK_CUDA(cudaMalloc((void**)&dOut, cap * sizeof(PgaTerminal)));
  CHECK_CUDA(cudaMalloc((void**)&dCount, sizeof(uint64_t)));
  CHECK_CUDA(cudaMemcpy(dAxiom, &axiom, sizeof axiom, cudaMemcpyHostToDevice));
  uint64_t n = 0;
  try {
    evaluator.initialize(table, &cfg);
    n = evaluator.execute(dAxiom, 1, dOut, cap, dCount);
    // a second call on the same evaluator (the engine is reusable)
    n = evaluator.execute(dAxiom, 1, dOut, cap, dCount);
  } catch (const GB300::Error& e) {
    std::fprintf(stderr, "evaluator error %d: %s\n", (int)e.status, e.what());
    return 3;
  }
  std::vector<PgaTerminal> out(n);
  uint64_t count = 0;
  CHECK_CUDA(cudaMemcpy(out.data(), dOut, n * sizeof(PgaTerminal), cudaMemcpyDeviceToHost));
  CHECK_CUDA(cudaMemcpy(&count, dCount, sizeof count, cudaMemcpyDeviceToHost));
  evaluator.release();
  // an error path: a capacity too small is reported, not wrapped around
  GB300::Evaluator<ProcedureList> small;
  int overflowStatus = 0;
  try {
    small.initialize(table, &cfg);
    small.execute(dAxiom, 1, dOut, 100, dCount);
  } catch (const GB300::Error& e) {
    overflowStatus = (int)e.status;
  }
  small.release();
  cudaFree(dAxiom);
  cudaFree(dOut);
  cudaFree(dCount);
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  fwrite(out.data(), sizeof(PgaTerminal), n, f);
  std::fclose(f);
  std::printf("%llu %llu %d\n", (unsigned long long)n, (unsigned long long)count, overflowStatus);
  return 0;
}
