// probe.cu -- shared-memory accumulation microbenchmark: the on-chip ceiling
// of the tile deposit.  Every deposit adds one value per channel into a
// shared-memory tile accumulator, so the rate of that accumulation step alone
// (without the weight computation) bounds the deposit rate from above:
// ceiling = rate / (Nq + 1) channel additions per deposit.
//
// Kinds: 0 FP32 atomic add whose old value is used (the first half of the
// compensated add); 1 FP32 atomic add without return; 2 int64 atomic add
// (deterministic mode, as 64-bit atomics); 3 the compensated add with two
// FP32 atomics (atomic add with return, TwoSum, error term added to a second
// accumulator, the FP32C deposit's); 4 the same compensated add of an
// adjacent (hi, lo) pair by one 64-bit compare-and-swap (not used by the
// deposit); 5 the deterministic deposit's int64 fixed-point add as two native
// 32-bit atomics with a carry.  Lanes of a warp address distinct banks, as the cells of one
// deposit iteration do, so the figure is the conflict-free ceiling.
#include <cuda_runtime.h>

#include "internal.h"
#include "tiled.cuh"

namespace sphg {
namespace {

constexpr int kProbeCells = 4096;  // one 16 x 16 x 16 tile channel
constexpr int kProbeIters = 4096;

template <int KIND>
__global__ void __launch_bounds__(256, 4) k_probe_smem(float* sink) {
  __shared__ __align__(16) unsigned char raw[kProbeCells * 8];
  float* hi = (float*)raw;
  float* lo = hi + kProbeCells;
  unsigned long long* fx = (unsigned long long*)raw;
  for (int v = threadIdx.x; v < kProbeCells * 2; v += blockDim.x) hi[v] = 0.0f;
  __syncthreads();
  float v = 1.0e-3f * (float)(threadIdx.x + 1);
  float used = 0.0f;
  const int base = threadIdx.x;
#pragma unroll 4
  for (int i = 0; i < kProbeIters; ++i) {
    const int idx = (base + i * 257) & (kProbeCells - 1);
    if (KIND == 0) {
      used += atomicAdd(&hi[idx], v);
    } else if (KIND == 1) {
      atomicAdd(&hi[idx], v);
    } else if (KIND == 2) {
      atomicAdd(&fx[idx], (unsigned long long)(i + threadIdx.x));
    } else if (KIND == 3) {
      acc_twosum(&hi[idx], &lo[idx], v);
    } else if (KIND == 4) {
      acc_pair(reinterpret_cast<float2*>(raw) + idx, v);
    } else {  // int64 fixed point as two native 32-bit words with a carry
      unsigned* w = reinterpret_cast<unsigned*>(raw);
      const unsigned long long x = (unsigned long long)(long long)(v * 1.0e9f);
      const unsigned xl = (unsigned)x;
      const unsigned old = atomicAdd(&w[idx], xl);
      const unsigned xh = (unsigned)(x >> 32) + (old + xl < old ? 1u : 0u);
      if (xh != 0u) atomicAdd(&w[kProbeCells + idx], xh);
    }
    v = v * 1.0001f;
  }
  __syncthreads();
  if (threadIdx.x == 0) sink[blockIdx.x] = used + hi[blockIdx.x & (kProbeCells - 1)];
}

template <int KIND>
void launch_probe(int grid, float* sink, cudaStream_t s) {
  k_probe_smem<KIND><<<grid, 256, 0, s>>>(sink);
}

}  // namespace

cudaError_t probe_smem_rate(int kind, int num_sms, cudaStream_t s, double* ops_per_s) {
  const int grid = num_sms * 4;
  float* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&sink, grid * sizeof(float));
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best = 0.0f;
  for (int rep = 0; e == cudaSuccess && rep < 4; ++rep) {  // first launch is a warm-up
    cudaEventRecord(e0, s);
    switch (kind) {
      case 0: launch_probe<0>(grid, sink, s); break;
      case 1: launch_probe<1>(grid, sink, s); break;
      case 2: launch_probe<2>(grid, sink, s); break;
      case 3: launch_probe<3>(grid, sink, s); break;
      case 4: launch_probe<4>(grid, sink, s); break;
      default: launch_probe<5>(grid, sink, s); break;
    }
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess && rep > 0 && (best == 0.0f || ms < best)) best = ms;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) *ops_per_s = (double)grid * 256.0 * kProbeIters / (best * 1e-3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (sink) cudaFree(sink);
  return e;
}

}  // namespace sphg
