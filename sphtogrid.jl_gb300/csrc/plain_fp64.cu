// plain_fp64.cu -- the plain FP64 deposition (one warp per particle, FP64
// arithmetic and FP64 global atomics) and the image reduction kernels.
//
// This translation unit is compiled with --fmad=false: every per-pixel weight
// is then computed with the operation order and rounding of the reference
// (src/cic_interpolation/cic_2D.jl:11-244, cic_3D.jl:13-208), and the only
// difference to a serial FP64 run is the order of the atomic sums.
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace sphg {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Footprint cell f = (ia nj + jb) nk + kc of a lane-strided walk: the lane's
// first cell is decomposed once, then each step of 32 cells advances
// (ia, jb, kc) in that mixed radix with adds and compares -- no 64-bit
// integer division per cell (the same cells, in the same order).
struct CellWalk {
  int64_t ia, jb, kc;
  int64_t da, db, dc, nj, nk;
  __device__ __forceinline__ CellWalk(int lane, int64_t nj_, int64_t nk_) : nj(nj_), nk(nk_) {
    const int64_t njk = nj * nk;
    ia = lane / njk;
    const int64_t r = lane - ia * njk;
    jb = r / nk;
    kc = r - jb * nk;
    da = 32 / njk;
    const int64_t r32 = 32 - da * njk;
    db = r32 / nk;
    dc = r32 - db * nk;
  }
  __device__ __forceinline__ void step() {
    kc += dc;
    const bool wk = kc >= nk;
    kc = wk ? kc - nk : kc;
    jb += db + (wk ? 1 : 0);
    const bool wj = jb >= nj;
    jb = wj ? jb - nj : jb;
    ia += da + (wj ? 1 : 0);
  }
};

// One warp deposits one particle: pass 1 sums kernel x area weights over the
// footprint (calculate_weights), pass 2 recomputes them and adds the
// renormalised weight to the image (update_image!).
template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) k_plain_fp64(DevParticles pt, DevMapParams mp,
                                                     double* __restrict__ accq, double* __restrict__ accw,
                                                     int64_t PD, DevStatus* __restrict__ st) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double L = mp.L;
  const int64_t P = mp.P;
  const int nq = pt.nq;
  unsigned long long c_mapped = 0, c_dep = 0;
  double c_gm = 0.0, c_pm = 0.0;
  unsigned flags = 0;

  for (int64_t p = wid; p < pt.n; p += nw) {
    PrepFP64 q;
    const int state = prep_particle_fp64<DIMS>(pt, mp, p, lane == 0, &q);
    if (state == kPrepNonFinite) flags |= kFlagNonFinite;
    if (state != kPrepMapped) continue;
    const int64_t iMin = q.lo[0], jMin = q.lo[1], kMin = q.lo[2];
    const int64_t ni = q.hi[0] - iMin + 1, nj = q.hi[1] - jMin + 1, nk = q.hi[2] - kMin + 1;
    const int64_t njk = nj * nk;
    const int64_t F = ni * njk;

    // pass 1: calculate_weights (cic_2D.jl:11-72 / cic_3D.jl:13-78)
    double s_w = 0.0, s_a = 0.0;
    long long n_d = 0, n_t = 0;
    CellWalk w1(lane, nj, nk);
    for (int64_t f = lane; f < F; f += 32, w1.step()) {
      const int64_t ia = w1.ia, jb = w1.jb, kc = w1.kc;
      double u, a;
      cell_fp64<DIMS>(q, iMin + ia, jMin + jb, kMin + kc, &u, &a);
      s_a += a;
      n_t += 1;
      if (u <= 1.0) {
        s_w += kshape<KERN, double>(u) * q.knorm * a;
        n_d += 1;
      }
    }
    s_w = warp_sum(s_w);
    s_a = warp_sum(s_a);
    n_d = warp_sum(n_d);
    n_t = warp_sum(n_t);
    const bool fallback = (s_w == 0.0);
    double wpp;
    if (fallback) {  // no pixel centre inside the kernel: spread by area
      n_d = n_t;
      wpp = s_a != 0.0 ? (double)n_d / s_a : 1.0;
    } else {
      wpp = (double)n_d / s_w;
    }
    const double norm = DIMS == 2 ? q.area / (double)n_d * wpp * q.wgt * q.col
                                  : q.vol / (double)n_d * wpp * q.wgt * L;

    // pass 2: deposit (cic_2D.jl:193-222, cic_3D.jl:172-188)
    double gm = 0.0;
    CellWalk w2(lane, nj, nk);
    for (int64_t f = lane; f < F; f += 32, w2.step()) {
      const int64_t i = iMin + w2.ia, j = jMin + w2.jb, k = kMin + w2.kc;
      double u, a;
      cell_fp64<DIMS>(q, i, j, k, &u, &a);
      const double wk = fallback ? 1.0 : (u <= 1.0 ? kshape<KERN, double>(u) * q.knorm : 0.0);
      const double pw = wk * a * norm;
      const int64_t idx = DIMS == 2 ? i * P + j : (i * P + j) * P + k;
      if (pw != 0.0) {
        atomicAdd(accw + idx, pw);
        if (q.scalar_zero) {
          atomicAdd(accq + idx, 0.0 * pw);
        } else {
          for (int c = 0; c < nq; ++c)
            atomicAdd(accq + idx + c * PD, ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + c * pt.qsk) * pw);
        }
      }
      if (DIMS == 3) gm += q.rho_in * wk * a / (L * L * L);
    }
    c_gm += gm;
    if (lane == 0) {
      c_mapped += 1;
      c_dep += (unsigned long long)F;
      c_pm += q.m_in;
    }
  }
  // fold the per-thread statistics: one atomic per warp
  c_gm = warp_sum(c_gm);
  c_pm = warp_sum(c_pm);
  c_mapped = (unsigned long long)warp_sum((long long)c_mapped);
  c_dep = (unsigned long long)warp_sum((long long)c_dep);
  flags = __reduce_or_sync(0xffffffffu, flags);
  if (lane == 0) {
    if (c_mapped) {
      atomicAdd(&st->n_mapped, c_mapped);
      atomicAdd(&st->deposits, c_dep);
      atomicAdd(&st->particle_mass, c_pm);
      if (DIMS == 3) atomicAdd(&st->grid_mass, c_gm);
    }
    if (flags) atomicOr(&st->flags, flags);
  }
}

// reduce_image_2D (reduce_image.jl:8-31): raw row ix*P+iy -> out[ix, iy, q]
// (column-major), dividing by the weight where it is positive.  32x32 tiles
// through shared memory keep both the read and the write coalesced.
__global__ void __launch_bounds__(256) k_reduce_2d(const double* __restrict__ acc, int64_t P, int nq,
                                                    int reduce, double* __restrict__ out) {
  __shared__ double tq[32][33];
  const int64_t PD = P * P;
  const int64_t ix0 = (int64_t)blockIdx.y * 32, iy0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // (32, 8)
  for (int q = 0; q < nq; ++q) {
    for (int r = ty; r < 32; r += 8) {
      const int64_t ix = ix0 + r, iy = iy0 + tx;
      double v = 0.0;
      if (ix < P && iy < P) {
        const int64_t k = ix * P + iy;
        v = acc[k + q * PD];
        const double W = acc[k + (int64_t)nq * PD];
        if (reduce && W > 0.0) v /= W;
      }
      tq[r][tx] = v;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int64_t iy = iy0 + r, ix = ix0 + tx;
      if (ix < P && iy < P) out[ix + P * iy + PD * q] = tq[tx][r];
    }
    __syncthreads();
  }
}

// reduce_image_3D (reduce_image.jl:39-55): the raw row ix*P^2+iy*P+iz already
// is the column-major index of out[iz, iy, ix]; divide only where Q > 0.
__global__ void __launch_bounds__(256) k_reduce_3d(const double* __restrict__ q, const double* __restrict__ w,
                                                    int64_t PD, int w_is_one, double* __restrict__ out) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < PD;
       m += (int64_t)gridDim.x * blockDim.x) {
    double v = q[m];
    if (v > 0.0) v /= (w_is_one ? 1.0 : w[m]);
    out[m] = v;
  }
}

// distributed_cic_map's summation of sub-file maps (distributed_mapping/cic.jl:
// 55-78): finite entries of `part` are added into `sum`, NaN and Inf skipped.
__global__ void __launch_bounds__(256) k_accumulate_finite(const double* __restrict__ part,
                                                            double* __restrict__ sum, int64_t len) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < len;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double v = part[e];
    if (isfinite(v)) sum[e] += v;
  }
}

// Per-particle state and integer pixel ranges (sphg_footprints): the
// centring, filter, quantity skip and pix_index_min_max of the FP32 method's
// first pass (prep_particle_lite, which hands particles it cannot decide in
// FP32 to prep_particle_fp64, the plain method's preparation).
template <int DIMS>
__global__ void __launch_bounds__(256) k_footprints(DevParticles pt, DevMapParams mp, long long* rng,
                                                    signed char* state, DevStatus* st) {
  unsigned flags = 0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < pt.n; p += (int64_t)gridDim.x * blockDim.x) {
    PrepLite q;
    const int s = prep_particle_lite<DIMS>(pt, mp, p, false, &q);
    signed char code = 0;
    long long r[6] = {0, 0, 0, 0, 0, 0};
    if (s == kPrepMapped) {
      code = 2;
      for (int d = 0; d < DIMS; ++d) {
        r[2 * d] = q.lo[d];
        r[2 * d + 1] = q.hi[d];
      }
    } else if (s == kPrepZeroQ) {
      code = 1;
    } else if (s == kPrepNonFinite) {
      code = 3;
      flags |= kFlagNonFinite;
    }
    state[p] = code;
    for (int k = 0; k < 6; ++k) rng[6 * p + k] = r[k];
  }
  if (flags) atomicOr(&st->flags, flags);
}

template <int DIMS>
void launch_plain_dims(int kernel, const DevParticles& pt, const DevMapParams& mp, double* accq,
                       double* accw, int64_t PD, DevStatus* st, int grid, cudaStream_t s) {
  switch (kernel) {
    case 0: k_plain_fp64<DIMS, 0><<<grid, 256, 0, s>>>(pt, mp, accq, accw, PD, st); break;
    case 1: k_plain_fp64<DIMS, 1><<<grid, 256, 0, s>>>(pt, mp, accq, accw, PD, st); break;
    case 2: k_plain_fp64<DIMS, 2><<<grid, 256, 0, s>>>(pt, mp, accq, accw, PD, st); break;
    case 3: k_plain_fp64<DIMS, 3><<<grid, 256, 0, s>>>(pt, mp, accq, accw, PD, st); break;
    default: k_plain_fp64<DIMS, 4><<<grid, 256, 0, s>>>(pt, mp, accq, accw, PD, st); break;
  }
}

}  // namespace

cudaError_t probe_kernel_image(cudaFuncAttributes* fa) {
  return cudaFuncGetAttributes(fa, k_reduce_3d);
}

void launch_plain_fp64(int kernel, const DevParticles& pt, const DevMapParams& mp, double* accq,
                       double* accw, int64_t PD, DevStatus* st, int num_sms, cudaStream_t s) {
  if (pt.n <= 0) return;
  const int64_t warps_needed = pt.n;
  int64_t grid = (warps_needed + 7) / 8;
  const int64_t cap = (int64_t)num_sms * 8 * 4;
  if (grid > cap) grid = cap;
  if (mp.dims == 2) launch_plain_dims<2>(kernel, pt, mp, accq, accw, PD, st, (int)grid, s);
  else launch_plain_dims<3>(kernel, pt, mp, accq, accw, PD, st, (int)grid, s);
}

void launch_accumulate(const double* part, double* sum, int64_t len, int num_sms, cudaStream_t s) {
  int64_t grid = (len + 255) / 256;
  if (grid > (int64_t)num_sms * 16) grid = (int64_t)num_sms * 16;
  if (grid < 1) grid = 1;
  k_accumulate_finite<<<(int)grid, 256, 0, s>>>(part, sum, len);
}

void launch_reduce_2d(const double* acc, int64_t P, int nq, int reduce, double* out, cudaStream_t s) {
  dim3 grid((unsigned)((P + 31) / 32), (unsigned)((P + 31) / 32));
  k_reduce_2d<<<grid, dim3(32, 8), 0, s>>>(acc, P, nq, reduce, out);
}

void launch_reduce_3d(const double* q, const double* w, int64_t PD, int w_is_one, double* out,
                      int num_sms, cudaStream_t s) {
  int64_t grid = (PD + 255) / 256;
  const int64_t cap = (int64_t)num_sms * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  k_reduce_3d<<<(int)grid, 256, 0, s>>>(q, w, PD, w_is_one, out);
}

void launch_footprints(const DevParticles& pt, const DevMapParams& mp, long long* rng, signed char* state,
                       DevStatus* st, int num_sms, cudaStream_t s) {
  int grid = (int)((pt.n + 255) / 256);
  if (grid > num_sms * 8) grid = num_sms * 8;
  if (grid < 1) grid = 1;
  if (mp.dims == 2) k_footprints<2><<<grid, 256, 0, s>>>(pt, mp, rng, state, st);
  else k_footprints<3><<<grid, 256, 0, s>>>(pt, mp, rng, state, st);
}

}  // namespace sphg
