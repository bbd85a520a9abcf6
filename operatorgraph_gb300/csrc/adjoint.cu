// Adjoint of the derivation (placeholder until the reverse sweep lands).
#include "engine_host.h"

extern "C" PgaStatus pga_adjoint(PgaEngine* e, const float* dGradTerminals, float* dGradParams, uint32_t numBlocks,
                                 float* dGradAxiomSizes, void* stream) {
  (void)dGradTerminals; (void)dGradParams; (void)numBlocks; (void)dGradAxiomSizes; (void)stream;
  if (!e) return PGA_ERR_INVALID_ARGUMENT;
  pga::set_error("pga_adjoint: not available in this build");
  return PGA_ERR_NO_TAPE;
}
