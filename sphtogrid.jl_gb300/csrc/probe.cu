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
// 32-bit atomics with a carry (its tiles of more than 2047 pairs); 6 the same
// fixed point as three 21-bit chunks, three 32-bit reductions without
// return (its tiles of at most 2047 pairs).  Lanes of a warp address
// distinct banks, as the cells of one deposit iteration do, so the figure is
// the conflict-free ceiling.
#include <cuda_runtime.h>

#include "internal.h"
#include "tiled.cuh"
#include "tiled_kernels.cuh"

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
    } else if (KIND == 6) {  // three 21-bit chunks (planes of kProbeCells / 2 cells)
      int* w = reinterpret_cast<int*>(raw);
      const int j = idx & (kProbeCells / 2 - 1);
      int x0, x1, x2;
      tiled_detail::fixed_chunks(v * 1.0e9f, x0, x1, x2);
      atomicAdd(&w[j], x0);
      atomicAdd(&w[kProbeCells / 2 + j], x1);
      atomicAdd(&w[kProbeCells + j], x2);
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

// The deposit's bounded staging wait on a barrier that no bulk copy
// completes (no copy is issued): the wait gives up after `polls` polls and
// the kernel records that, as the deposit records a timeout.
__global__ void __launch_bounds__(32) k_probe_wait(int polls, int* timed_out) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    tiled_detail::mbar_init(&bar, 1);
    tiled_detail::fence_proxy_async_smem();
    tiled_detail::fence_mbar_init();
  }
  __syncwarp();
  const bool done = tiled_detail::mbar_wait_warp(&bar, 0u, polls);
  if (threadIdx.x == 0) *timed_out = done ? 0 : 1;
}

// The deterministic mode's three-chunk rounding of each v, recombined, next
// to the 64-bit conversion it must equal.
__global__ void __launch_bounds__(256) k_probe_chunks(const float* v, long long* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int x0, x1, x2;
  tiled_detail::fixed_chunks(v[i], x0, x1, x2);
  out[2 * i] = (long long)x2 * (1LL << 42) + (long long)x1 * (1LL << 21) + x0;
  out[2 * i + 1] = __float2ll_rn(v[i]);
}

}  // namespace

cudaError_t probe_fixed_chunks(int n, const float* v, long long* x, cudaStream_t s) {
  float* dv = nullptr;
  long long* dx = nullptr;
  cudaError_t e = cudaMalloc(&dv, (size_t)n * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&dx, 2 * (size_t)n * sizeof(long long));
  if (e == cudaSuccess) e = cudaMemcpyAsync(dv, v, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    k_probe_chunks<<<(n + 255) / 256, 256, 0, s>>>(dv, dx, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, dx, 2 * (size_t)n * sizeof(long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (dv) cudaFree(dv);
  if (dx) cudaFree(dx);
  return e;
}

cudaError_t probe_wait_timeout(int polls, cudaStream_t s, int* timed_out) {
  int* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int));
  if (e == cudaSuccess) {
    k_probe_wait<<<1, 32, 0, s>>>(polls, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(timed_out, d, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFree(d);
  return e;
}

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
      case 5: launch_probe<5>(grid, sink, s); break;
      default: launch_probe<6>(grid, sink, s); break;
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
