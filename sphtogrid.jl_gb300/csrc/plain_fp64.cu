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

// Julia min/max on finite floats.
__device__ __forceinline__ double jmin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double jmax(double a, double b) { return b > a ? b : a; }

// Per-pixel geometry of one footprint cell: pixel-centre offsets and overlap.
__device__ __forceinline__ void cell_axis(double x, double h, int64_t i, double* dist, double* ov) {
  *dist = x - (double)i - 0.5;                                   // get_x_dx, cic_shared.jl:70-76
  *ov = jmin(x + h, (double)(i + 1)) - jmax(x - h, (double)i);   // get_dxyz, cic_shared.jl:60-62
}

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
    // center_particles (filter_shift.jl:6-32) and filter (filter_shift.jl:40-58)
    double c[3];
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int64_t o = p * pt.sp + d * pt.sc;
      double v = ld_elem(pt.pos_dtype, pt.pos, o);
      if (mp.center_mode != 0) {
        v = round_to(pt.pos_dtype, v - mp.cen[d]);
        if (mp.periodic && fabs(v) > mp.boxsize / 2)
          v = round_to(pt.pos_dtype, v > 0 ? v - mp.boxsize / 2 : v + mp.boxsize / 2);
        if (mp.center_mode == 1 && lane == 0) st_elem(pt.pos_dtype, pt.pos, o, v);
      }
      c[d] = v;
      if (mp.filter && !(mp.lo[d] <= v && v <= mp.hi[d])) in = false;
    }
    if (!in) continue;
    // skip particles without a quantity (cic_2D.jl:154-168, cic_3D.jl:140-144)
    bool allzero = true;
    for (int k = 0; k < nq; ++k)
      if (ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + k * pt.qsk) != 0.0) allzero = false;
    if (allzero && !mp.calc_mean) continue;
    const bool scalar_zero = (nq > 1) && allzero;

    const double m_in = ld_elem(pt.attr_dtype, pt.mass, p);
    const double rho_in = ld_elem(pt.attr_dtype, pt.rho, p);
    const double wgt = ld_elem(pt.attr_dtype, pt.w, p);
    const double hsml = ld_elem(pt.attr_dtype, pt.hsml, p) * L;
    const double h_inv = 1.0 / hsml;
    double area = 0.0, col = 0.0, vol = 0.0;
    if (DIMS == 2) {  // get_quantities_2D, cic_2D.jl:80-91
      area = (2.0 * hsml) * (2.0 * hsml);
      const double rho = rho_in * (1.0 / (L * L * L));
      col = m_in / rho / area;
    } else {  // get_quantities_3D, cic_3D.jl:87-97
      const double rho = rho_in / (L * L * L);
      vol = m_in / rho;
    }
    const double hd = mp.kernel_dim == 2 ? h_inv * h_inv : h_inv * h_inv * h_inv;
    const double knorm = mp.sigma * hd;  // SPHKernels normalisation x h_inv^D
    // get_xyz (cic_shared.jl:85-99) and pix_index_min_max (cic_shared.jl:46-52)
    double x = c[0] * L, y = c[1] * L, z = c[2] * L;
    x += 0.5 * (double)P;
    y += 0.5 * (double)P;
    z += 0.5 * (double)P;
    int64_t a0, a1, b0, b1, e0 = 0, e1 = 0;
    if (!floor_int(x - hsml, &a0) || !floor_int(x + hsml, &a1) || !floor_int(y - hsml, &b0) ||
        !floor_int(y + hsml, &b1) ||
        (DIMS == 3 && (!floor_int(z - hsml, &e0) || !floor_int(z + hsml, &e1)))) {
      flags |= kFlagNonFinite;
      continue;
    }
    const int64_t iMin = a0 > 0 ? a0 : 0, iMax = a1 < P - 1 ? a1 : P - 1;
    const int64_t jMin = b0 > 0 ? b0 : 0, jMax = b1 < P - 1 ? b1 : P - 1;
    const int64_t kMin = DIMS == 3 ? (e0 > 0 ? e0 : 0) : 0;
    const int64_t kMax = DIMS == 3 ? (e1 < P - 1 ? e1 : P - 1) : 0;
    const int64_t ni = iMax >= iMin ? iMax - iMin + 1 : 0;
    const int64_t nj = jMax >= jMin ? jMax - jMin + 1 : 0;
    const int64_t nk = kMax >= kMin ? kMax - kMin + 1 : 0;
    const int64_t njk = nj * nk;
    const int64_t F = ni * njk;

    // pass 1: calculate_weights (cic_2D.jl:11-72 / cic_3D.jl:13-78)
    double s_w = 0.0, s_a = 0.0;
    long long n_d = 0, n_t = 0;
    for (int64_t f = lane; f < F; f += 32) {
      const int64_t ia = f / njk, r = f - ia * njk;
      const int64_t jb = r / nk, kc = r - jb * nk;
      double xd, dx, yd, dy, zd = 0.0, dz = 1.0;
      cell_axis(x, hsml, iMin + ia, &xd, &dx);
      cell_axis(y, hsml, jMin + jb, &yd, &dy);
      double u, a;
      if (DIMS == 2) {
        u = sqrt(xd * xd + yd * yd) * h_inv;
        a = dx * dy;
      } else {
        cell_axis(z, hsml, kMin + kc, &zd, &dz);
        a = dx * dy * dz;
        u = sqrt(xd * xd + yd * yd + zd * zd) * h_inv;
      }
      s_a += a;
      n_t += 1;
      if (u <= 1.0) {
        s_w += kshape<KERN, double>(u) * knorm * a;
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
    const double norm = DIMS == 2 ? area / (double)n_d * wpp * wgt * col
                                  : vol / (double)n_d * wpp * wgt * L;

    // pass 2: deposit (cic_2D.jl:193-222, cic_3D.jl:172-188)
    double gm = 0.0;
    for (int64_t f = lane; f < F; f += 32) {
      const int64_t ia = f / njk, r = f - ia * njk;
      const int64_t jb = r / nk, kc = r - jb * nk;
      const int64_t i = iMin + ia, j = jMin + jb, k = kMin + kc;
      double xd, dx, yd, dy, zd = 0.0, dz = 1.0;
      cell_axis(x, hsml, i, &xd, &dx);
      cell_axis(y, hsml, j, &yd, &dy);
      double u, a;
      if (DIMS == 2) {
        u = sqrt(xd * xd + yd * yd) * h_inv;
        a = dx * dy;
      } else {
        cell_axis(z, hsml, k, &zd, &dz);
        a = dx * dy * dz;
        u = sqrt(xd * xd + yd * yd + zd * zd) * h_inv;
      }
      const double wk = fallback ? 1.0 : (u <= 1.0 ? kshape<KERN, double>(u) * knorm : 0.0);
      const double pw = wk * a * norm;
      const int64_t idx = DIMS == 2 ? i * P + j : (i * P + j) * P + k;
      if (pw != 0.0) {
        atomicAdd(accw + idx, pw);
        if (scalar_zero) {
          atomicAdd(accq + idx, 0.0 * pw);
        } else {
          for (int q = 0; q < nq; ++q)
            atomicAdd(accq + idx + q * PD, ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + q * pt.qsk) * pw);
        }
      }
      if (DIMS == 3) gm += rho_in * wk * a / (L * L * L);
    }
    c_gm += gm;
    if (lane == 0) {
      c_mapped += 1;
      c_dep += (unsigned long long)F;
      c_pm += m_in;
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

}  // namespace sphg
