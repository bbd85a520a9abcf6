// The derivation and adjoint kernels built with general rotation frames
// (PGA_GENERAL_FRAMES): engines whose table has Rotate rules launch these
// (pga::gen) instead of the frame-code kernels of derive.cu.
#define PGA_GENERAL_FRAMES 1
#include "derive_kernels.cuh"
#define PGA_ADJOINT_DEVICE_ONLY 1
#include "adjoint.cuh"

namespace pga {
FrameKernels general_frame_kernels() {
  FrameKernels k = frame_kernels();
  k.adjoint = adjoint_kernel();
  k.adjointWide = adjoint_kernel_wide();
  return k;
}
}  // namespace pga
