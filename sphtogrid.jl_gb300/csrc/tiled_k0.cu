// tiled_k0.cu -- K3/K4 of the tiled deposition for kernel shape 0
// (cubic).  Compiled with --fmad=false (see tiled_fp32.cu).
#include "tiled_kernels.cuh"

namespace sphg {
SPHG_TILED_SHAPE(0)
}  // namespace sphg
