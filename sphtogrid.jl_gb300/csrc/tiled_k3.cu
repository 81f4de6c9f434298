// tiled_k3.cu -- K3/K4 of the tiled deposition for kernel shape 3
// (Wendland C6).  Compiled with --fmad=false (see tiled_fp32.cu).
#include "tiled_kernels.cuh"

namespace sphg {
SPHG_TILED_SHAPE(3)
}  // namespace sphg
