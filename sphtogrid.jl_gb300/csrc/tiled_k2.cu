// tiled_k2.cu -- K3/K4 of the tiled deposition for kernel shape 2
// (Wendland C4).  Compiled with --fmad=false (see tiled_fp32.cu).
#include "tiled_kernels.cuh"

namespace sphg {
SPHG_TILED_SHAPE(2)
}  // namespace sphg
