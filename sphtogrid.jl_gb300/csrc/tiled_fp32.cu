// tiled_fp32.cu -- K1/K2 and the host launcher of the FP32-compensated tiled
// deposition (see tiled.cuh for the pipeline; K3/K4 are in tiled_kernels.cuh).  Compiled with --fmad=false so
// that the FP64 arithmetic shared with the plain path rounds exactly as the
// reference; the FP32 hot loops use explicit fmaf.
#include <cuda_runtime.h>

#include <climits>

#include "internal.h"
#include "tiled_kernels.cuh"

namespace sphg {
using namespace tiled_detail;

namespace {

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }


template <int DIMS>
__global__ void __launch_bounds__(256) k_prep_count(TiledArgs A) {
  __shared__ PrepShared sh;
  prep_count<DIMS>(A, (int64_t)blockIdx.x * blockDim.x, (int64_t)gridDim.x * blockDim.x, sh);
}

__global__ void __launch_bounds__(1024) k_scan_tiles(TiledArgs A) {
  __shared__ long long part[1024];
  scan_tiles(A, part);
}

}  // namespace

void tiled_geometry(int dims, int64_t P, int tdim[3], int ntile[3], int64_t* n_tiles) {
  if (dims == 2) {
    tdim[0] = 16; tdim[1] = 16; tdim[2] = 1;
  } else {
    tdim[0] = kTile3X; tdim[1] = kTile3Y; tdim[2] = kTile3Z;
  }
  for (int d = 0; d < 3; ++d) ntile[d] = (d < dims) ? (int)((P + tdim[d] - 1) / tdim[d]) : 1;
  *n_tiles = (int64_t)ntile[0] * ntile[1] * ntile[2];
}

// Launches K1..K4 on `s`.  With `ev` (4 events) the phases prep+scan,
// norm+fill and deposit are bracketed for timing.  Returns the number of
// kernels launched through `n_launch`.
cudaError_t launch_tiled_fp32(int kernel, const TiledArgs& A, int num_sms, cudaStream_t s,
                              cudaEvent_t* ev, int* n_launch) {
  const int dims = A.mp.dims;
  int grid = ceil_div(A.pt.n, 256);
  if (grid > num_sms * 8) grid = num_sms * 8;
  if (grid < 1) grid = 1;
  if (ev) cudaEventRecord(ev[0], s);
  if (dims == 2) k_prep_count<2><<<grid, 256, 0, s>>>(A);
  else k_prep_count<3><<<grid, 256, 0, s>>>(A);
  k_scan_tiles<<<1, 1024, 0, s>>>(A);
  if (ev) cudaEventRecord(ev[1], s);
  int grid_rec = ceil_div(A.pt.n, 8);
  if (grid_rec > num_sms * 16) grid_rec = num_sms * 16;
  if (grid_rec < 1) grid_rec = 1;
  switch (kernel) {
    case 0: launch_norm_deposit_0(A, grid_rec, s, ev); break;
    case 1: launch_norm_deposit_1(A, grid_rec, s, ev); break;
    case 2: launch_norm_deposit_2(A, grid_rec, s, ev); break;
    case 3: launch_norm_deposit_3(A, grid_rec, s, ev); break;
    default: launch_norm_deposit_4(A, grid_rec, s, ev); break;
  }
  if (ev) cudaEventRecord(ev[3], s);
  if (n_launch) *n_launch = 6;
  return cudaGetLastError();
}

}  // namespace sphg
