/*
 * pga/engine.hpp -- C++ evaluator over the GB300 engine's C ABI.
 *
 * PGA::GB300::Evaluator<ProcedureListT> has the three calls of the reference's
 * SinglePhaseEvaluator (initialize / execute / release, include/pga/core/
 * GPUEvaluator.cuh:475-536 and CPUEvaluator.h:393-459): initialize lowers the
 * dispatch table written for ProcedureListT (pga/core.hpp) and creates the
 * engine, execute derives a batch of axioms into a caller-owned device buffer
 * and returns the terminal count, release frees the engine.  Errors throw
 * PGA::GB300::Error carrying the PgaStatus, where the reference throws
 * PGA::CUDA::Exception or traps on the device.
 *
 * Device memory stays the caller's: axioms, parameter blocks, the terminal
 * buffer and the count are device pointers.  Streams are cudaStream_t values
 * passed as void*.
 */
#ifndef PGA_GB300_ENGINE_HPP
#define PGA_GB300_ENGINE_HPP

#include <pga/core.hpp>

#include <cstdint>
#include <stdexcept>
#include <string>

namespace PGA {
namespace GB300 {

class Error : public std::runtime_error {
 public:
  Error(PgaStatus s, const std::string& what) : std::runtime_error(what), status(s) {}
  PgaStatus status;
};

inline void check(PgaStatus s, const char* call) {
  if (s != PGA_OK) {
    const char* msg = pga_last_error();
    throw Error(s, std::string(call) + ": " + (msg && *msg ? msg : "status " + std::to_string((int)s)));
  }
}

template <typename ProcedureListT>
class Evaluator {
 public:
  Evaluator() = default;
  Evaluator(const Evaluator&) = delete;
  Evaluator& operator=(const Evaluator&) = delete;
  ~Evaluator() { release(); }

  /* Lowers the table and creates the engine; `config` may be null (defaults). */
  void initialize(const DispatchTable& table, const PgaEngineConfig* config = nullptr) {
    table_ = lower<ProcedureListT>(table);
    create(config);
  }
  void initialize(const PgaEntry* entries, size_t numEntries, const PgaEngineConfig* config = nullptr) {
    table_ = lower<ProcedureListT>(entries, numEntries);
    create(config);
  }

  /* Derives numAxioms axioms into dOut (capacity records) and returns the
   * number of terminals; *dCount receives it on the device as well.  Blocks
   * on `stream` to read the device status. */
  uint64_t execute(const PgaAxiom* dAxioms, uint32_t numAxioms, PgaTerminal* dOut, uint64_t capacity,
                   uint64_t* dCount, void* stream = nullptr, const float* dParamBlocks = nullptr) {
    if (!engine_) throw Error(PGA_ERR_INVALID_ARGUMENT, "Evaluator::execute before initialize");
    check(pga_derive(engine_, dAxioms, numAxioms, dParamBlocks, dOut, capacity, dCount, stream), "pga_derive");
    PgaDeriveReport r;
    const PgaStatus s = pga_engine_sync_report(engine_, stream, &r);
    if (s != PGA_OK) check(s, "pga_derive (device)");
    return r.terminals;
  }

  void release() {
    if (engine_) pga_engine_destroy(engine_);
    engine_ = nullptr;
  }

  PgaEngine* handle() const { return engine_; }
  const LoweredTable& table() const { return table_; }

 private:
  void create(const PgaEngineConfig* config) {
    release();
    const PgaRuleTable view = table_.view();
    check(pga_engine_create(&view, config, &engine_), "pga_engine_create");
  }

  LoweredTable table_;
  PgaEngine* engine_ = nullptr;
};

}  // namespace GB300
}  // namespace PGA

#endif  // PGA_GB300_ENGINE_HPP
