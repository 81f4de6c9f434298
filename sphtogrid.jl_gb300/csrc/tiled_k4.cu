// tiled_k4.cu -- K3/K4 of the tiled deposition for kernel shape 4
// (Wendland C8).  Compiled with --fmad=false (see tiled_fp32.cu).
#include "tiled_kernels.cuh"

namespace sphg {
SPHG_TILED_SHAPE(4)
}  // namespace sphg
