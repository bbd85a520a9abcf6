// The derivation kernels built with general rotation frames (PGA_GENERAL_FRAMES):
// engines whose table has Rotate rules launch these (pga::gen) instead of the
// frame-code kernels of derive.cu.
#define PGA_GENERAL_FRAMES 1
#include "derive_kernels.cuh"

namespace pga {
FrameKernels general_frame_kernels() { return frame_kernels(); }
}  // namespace pga
