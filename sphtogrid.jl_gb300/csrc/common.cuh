// common.cuh -- device-side definitions shared by the deposition kernels.
//
// Kernel shapes are those of SPHKernels.jl (called by SPHtoGrid.jl at
// src/cic_interpolation/cic_shared.jl:24): cubic and quintic B-splines and the
// Wendland C4/C6/C8 functions, all with compact support u = r/h in [0, 1].
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sphg {

constexpr int kMaxQ = 16;  // quantities per map (Bin_Quant rows)

constexpr double kPi = 3.14159265358979323846;

// Normalisation sigma_D of each kernel for support radius h.
__host__ __device__ inline double kernel_sigma(int kernel, int kdim) {
  switch (kernel) {
    case 0: return kdim == 2 ? 40.0 / (7.0 * kPi) : 8.0 / kPi;
    case 1: return kdim == 2 ? 15309.0 / (478.0 * kPi) : 2187.0 / (40.0 * kPi);
    case 2: return kdim == 2 ? 9.0 / kPi : 495.0 / (32.0 * kPi);
    case 3: return kdim == 2 ? 78.0 / (7.0 * kPi) : 1365.0 / (64.0 * kPi);
    default: return kdim == 2 ? 40.0 / (3.0 * kPi) : 1785.0 / (64.0 * kPi);
  }
}

// Un-normalised kernel shape; callers only evaluate it for u <= 1.  The
// expression order is the one of the oracle, so in FP64 without FMA
// contraction both give the same bits.
template <int KERN, typename T>
__device__ __forceinline__ T kshape(T u) {
  const T one = T(1);
  if (KERN == 0) {  // cubic
    if (u < T(0.5)) return one + T(6) * (u - one) * (u * u);
    if (u < one) { T t = one - u; return T(2) * (t * t * t); }
    return T(0);
  } else if (KERN == 1) {  // quintic
    T a = one - u, b = T(2) / T(3) - u, c = one / T(3) - u;
    T a5 = a * a * a * a * a, b5 = b * b * b * b * b, c5 = c * c * c * c * c;
    if (u < one / T(3)) return a5 - T(6) * b5 + T(15) * c5;
    if (u < T(2) / T(3)) return a5 - T(6) * b5;
    if (u < one) return a5;
    return T(0);
  } else if (KERN == 2) {  // Wendland C4
    if (u < one) { T t = one - u; T t2 = t * t; return t2 * t2 * t2 * (one + T(6) * u + T(35) / T(3) * (u * u)); }
    return T(0);
  } else if (KERN == 3) {  // Wendland C6
    if (u < one) {
      T t = one - u; T t2 = t * t; t2 = t2 * t2;
      return t2 * t2 * (one + T(8) * u + T(25) * (u * u) + T(32) * (u * u * u));
    }
    return T(0);
  } else {  // Wendland C8
    if (u < one) {
      T t = one - u; T t2 = t * t; T t4 = t2 * t2; T t8 = t4 * t4; T u2 = u * u;
      return t8 * t2 * (one + T(10) * u + T(42) * u2 + T(90) * (u2 * u) + T(429) / T(5) * (u2 * u2));
    }
    return T(0);
  }
}

// Particle arrays as passed through the C ABI (element strides).
struct DevParticles {
  int64_t n;
  int pos_dtype, attr_dtype;
  void* pos;
  int64_t sp, sc;
  const void *hsml, *mass, *rho, *w, *q;
  int nq;
  int64_t qsp, qsk;
};

// Mapping parameters the kernels need (derived on the host).
struct DevMapParams {
  double cen[3];          // centring shift (the caller's param.center)
  double lo[3], hi[3];    // inclusive filter box of the centred parameters
  double boxsize;
  int periodic;
  int center_mode;        // SPHG_CENTER_*
  int filter;
  int calc_mean;
  int kernel_dim;
  int dims;
  double L;               // len2pix
  int64_t P;              // Npixels
  double sigma;           // kernel normalisation
};

// Device-side status and statistics of one map call.
struct DevStatus {
  unsigned int flags;
  unsigned int pad;
  unsigned long long n_mapped;
  unsigned long long deposits;
  double grid_mass;
  double particle_mass;
};

enum : unsigned { kFlagNonFinite = 1u, kFlagTimeout = 2u, kFlagOverflow = 4u };

__device__ __forceinline__ double ld_elem(int dtype, const void* p, int64_t i) {
  return dtype == 0 ? (double)__ldg((const float*)p + i) : __ldg((const double*)p + i);
}

// Value of `v` after being stored into an array of `dtype` (Julia's convert
// rounds to nearest).
__device__ __forceinline__ double round_to(int dtype, double v) {
  return dtype == 0 ? (double)__double2float_rn(v) : v;
}

__device__ __forceinline__ void st_elem(int dtype, void* p, int64_t i, double v) {
  if (dtype == 0) ((float*)p)[i] = __double2float_rn(v);
  else ((double*)p)[i] = v;
}

// floor(Integer, v) with the reference's InexactError for non-finite values.
__device__ __forceinline__ bool floor_int(double v, int64_t* out) {
  if (!(fabs(v) < 9.2e18)) return false;
  *out = (int64_t)floor(v);
  return true;
}

}  // namespace sphg
