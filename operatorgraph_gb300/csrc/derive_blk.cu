// The derivation and adjoint kernels of the frame-code build with block
// parameters (PGA_PT_BLOCK) read inline (PGA_INLINE_BLOCKS): engines whose
// table has block parameters and no Rotate launch these (pga::permb) instead
// of derive.cu's, whose kernels keep the register allocation of tables
// without block parameters.
#define PGA_INLINE_BLOCKS 1
#include "derive_kernels.cuh"
#define PGA_ADJOINT_DEVICE_ONLY 1
#include "adjoint.cuh"

namespace pga {
FrameKernels block_frame_kernels() {
  FrameKernels k = frame_kernels();
  k.adjoint = adjoint_kernel();
  k.adjointWide = adjoint_kernel_wide();
  return k;
}
}  // namespace pga
