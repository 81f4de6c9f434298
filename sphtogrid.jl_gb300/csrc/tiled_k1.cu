// tiled_k1.cu -- K3/K4 of the tiled deposition for kernel shape 1
// (quintic).  Compiled with --fmad=false (see tiled_fp32.cu).
#include "tiled_kernels.cuh"

namespace sphg {
SPHG_TILED_SHAPE(1)
}  // namespace sphg
