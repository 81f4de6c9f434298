// common.cuh -- device-side definitions shared by the deposition kernels.
//
// Kernel shapes are those of SPHKernels.jl (called by SPHtoGrid.jl at
// src/cic_interpolation/cic_shared.jl:24): cubic and quintic B-splines and the
// Wendland C4/C6/C8 functions, all with compact support u = r/h in [0, 1].
#pragma once

#include <cmath>
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
  // map_it's projection (cic_interpolation.jl:330-345), read through on the
  // fly: 0 none; 1 axis permutation (coordinate d is input component
  // perm[d], exact, input precision); 2 FP64 3x3 matrix (row-major; the
  // rotated positions are Float64, as Julia promotes them)
  int xform = 0;
  int perm[3] = {0, 1, 2};
  double rot[9] = {};
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
  // Single-precision constants of prep_particle_lite, set on the host by
  // set_lite_params; lite = 0 leaves every particle to prep_particle_fp64.
  float lo_f[3] = {0.0f, 0.0f, 0.0f};  // lo rounded up to a float
  float hi_f[3] = {0.0f, 0.0f, 0.0f};  // hi rounded down to a float
  float L_hi = 0.0f, L_lo = 0.0f;      // L = L_hi + L_lo to about 2^-48 of L
  int lite = 0;
  float cen_f[3] = {0.0f, 0.0f, 0.0f};  // cen as floats, used when cen_f_exact
  int cen_f_exact = 0;                  // every cen[d] is a float
  float fac_m[3] = {0.0f, 0.0f, 0.0f};  // L, L^3 and sigma as fac_m 2^fac_e,
  int fac_e[3] = {0, 0, 0};             // fac_m in [0.5, 1]
  int fac_ok = 0;                       // the three are finite and positive
};

// Fills the constants of prep_particle_lite from the FP64 parameters.  A
// float v satisfies lo_f <= v <= hi_f exactly when (double)v satisfies the
// reference's lo <= v <= hi (NaN bounds fail both).
inline void set_lite_params(DevMapParams& mp) {
  for (int d = 0; d < 3; ++d) {
    float lo = (float)mp.lo[d], hi = (float)mp.hi[d];
    if ((double)lo < mp.lo[d]) lo = std::nextafter(lo, INFINITY);
    if ((double)hi > mp.hi[d]) hi = std::nextafter(hi, -INFINITY);
    mp.lo_f[d] = lo;
    mp.hi_f[d] = hi;
  }
  mp.L_hi = (float)mp.L;
  mp.L_lo = (float)(mp.L - (double)mp.L_hi);
  mp.lite = std::isfinite(mp.L_hi) && std::isfinite(mp.L_lo) && mp.L_hi != 0.0f && mp.P > 0 && mp.P < (1 << 22);
  mp.cen_f_exact = 1;
  for (int d = 0; d < 3; ++d) {
    mp.cen_f[d] = (float)mp.cen[d];
    if (!((double)mp.cen_f[d] == mp.cen[d])) mp.cen_f_exact = 0;
  }
  const double fac[3] = {mp.L, mp.L * mp.L * mp.L, mp.sigma};
  mp.fac_ok = 1;
  for (int i = 0; i < 3; ++i) {
    if (!(std::isfinite(fac[i]) && fac[i] > 0.0)) {
      mp.fac_ok = 0;
      continue;
    }
    int e = 0;
    mp.fac_m[i] = (float)std::frexp(fac[i], &e);
    mp.fac_e[i] = e;
  }
}

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

// 1/x to FP32 accuracy (relative error below 2^-22) over the whole FP64
// range, without an FP64 division: the mantissa's reciprocal in FP32, the
// exponent negated by bit arithmetic.  Zero, subnormal and non-finite x take
// the FP64 division.
__device__ __forceinline__ double rcp_approx(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0 || ex >= 0x7fe || ex <= 1) return 1.0 / x;
  const double m = __longlong_as_double((b & 0x800fffffffffffffLL) | (1023LL << 52));  // +-[1, 2)
  const double r = (double)__frcp_rn((float)m);                                        // +-(0.5, 1]
  return r * __longlong_as_double((long long)(2046 - ex) << 52);                       // * 2^(1023 - ex)
}

// Julia min/max on finite floats.
__device__ __forceinline__ double jmin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double jmax(double a, double b) { return b > a ? b : a; }

// One particle after centring, filtering and unit conversion, in the
// reference's FP64 arithmetic (translation units that include this header are
// compiled without FMA contraction).
struct PrepFP64 {
  double x, y, z;           // pixel coordinates (get_xyz, cic_shared.jl:85-99)
  double hsml, h_inv, knorm;
  double area, col, vol;    // 2D: (2h)^2 and m/rho_pix/area; 3D: m/rho_pix
  double m_in, rho_in, wgt;
  int64_t lo[3], hi[3];     // pix_index_min_max per axis (hi = lo - 1 when empty)
  bool scalar_zero;
};

// kPrepSkip: filtered out; kPrepZeroQ: every quantity zero without calc_mean.
enum { kPrepSkip = 0, kPrepMapped = 1, kPrepNonFinite = 2, kPrepZeroQ = 3 };

// center_particles / filter (filter_shift.jl:6-58), the quantity skip
// (cic_2D.jl:154-168), get_quantities_2D/3D (cic_2D.jl:80-91,
// cic_3D.jl:87-97), get_xyz and pix_index_min_max (cic_shared.jl:46-99).
// `store_pos` writes the centred position back (SPHG_CENTER_INPLACE).
// FACTORS = false skips the per-particle factors (h_inv, area, col, vol,
// knorm: FP64 divisions) for callers that derive their own; the centring,
// filter and pixel ranges are the same either way.
template <int DIMS, bool FACTORS = true>
__device__ __forceinline__ int prep_particle_fp64(const DevParticles& pt, const DevMapParams& mp, int64_t p,
                                                  bool store_pos, PrepFP64* o) {
  double c[3];
  bool in = true;
  double xr[3] = {0.0, 0.0, 0.0};
  if (pt.xform == 2) {  // (R0 x0 + R1 x1) + R2 x2 per row, in FP64
    const double x0 = ld_elem(pt.pos_dtype, pt.pos, p * pt.sp);
    const double x1 = ld_elem(pt.pos_dtype, pt.pos, p * pt.sp + pt.sc);
    const double x2 = ld_elem(pt.pos_dtype, pt.pos, p * pt.sp + 2 * pt.sc);
#pragma unroll
    for (int d = 0; d < 3; ++d) xr[d] = (pt.rot[3 * d] * x0 + pt.rot[3 * d + 1] * x1) + pt.rot[3 * d + 2] * x2;
  }
  const int vdt = pt.xform == 2 ? 1 : pt.pos_dtype;  // precision the centring rounds to
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int64_t off = p * pt.sp + (pt.xform == 1 ? pt.perm[d] : d) * pt.sc;
    double v = pt.xform == 2 ? xr[d] : ld_elem(pt.pos_dtype, pt.pos, off);
    if (mp.center_mode != 0) {
      v = round_to(vdt, v - mp.cen[d]);
      if (mp.periodic && fabs(v) > mp.boxsize / 2)
        v = round_to(vdt, v > 0 ? v - mp.boxsize / 2 : v + mp.boxsize / 2);
      if (mp.center_mode == 1 && store_pos && pt.xform == 0) st_elem(pt.pos_dtype, pt.pos, off, v);
    }
    c[d] = v;
    if (mp.filter && !(mp.lo[d] <= v && v <= mp.hi[d])) in = false;
  }
  if (!in) return kPrepSkip;
  bool allzero = true;
  for (int k = 0; k < pt.nq; ++k)
    if (ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + k * pt.qsk) != 0.0) allzero = false;
  if (allzero && !mp.calc_mean) return kPrepZeroQ;
  o->scalar_zero = (pt.nq > 1) && allzero;
  const double L = mp.L;
  const int64_t P = mp.P;
  o->m_in = ld_elem(pt.attr_dtype, pt.mass, p);
  o->rho_in = ld_elem(pt.attr_dtype, pt.rho, p);
  o->wgt = ld_elem(pt.attr_dtype, pt.w, p);
  const double hsml = ld_elem(pt.attr_dtype, pt.hsml, p) * L;
  o->hsml = hsml;
  o->h_inv = o->knorm = 0.0;
  o->area = o->col = o->vol = 0.0;
  if (FACTORS) {
    o->h_inv = 1.0 / hsml;
    if (DIMS == 2) {
      o->area = (2.0 * hsml) * (2.0 * hsml);
      const double rho = o->rho_in * (1.0 / (L * L * L));
      o->col = o->m_in / rho / o->area;
    } else {
      const double rho = o->rho_in / (L * L * L);
      o->vol = o->m_in / rho;
    }
    const double hd = mp.kernel_dim == 2 ? o->h_inv * o->h_inv : o->h_inv * o->h_inv * o->h_inv;
    o->knorm = mp.sigma * hd;
  }
  double x = c[0] * L, y = c[1] * L, z = c[2] * L;
  x += 0.5 * (double)P;
  y += 0.5 * (double)P;
  z += 0.5 * (double)P;
  o->x = x;
  o->y = y;
  o->z = z;
  const double xs[3] = {x, y, z};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (d >= DIMS) {
      o->lo[d] = 0;
      o->hi[d] = 0;
      continue;
    }
    int64_t a, b;
    if (!floor_int(xs[d] - hsml, &a) || !floor_int(xs[d] + hsml, &b)) return kPrepNonFinite;
    o->lo[d] = a > 0 ? a : 0;
    o->hi[d] = b < P - 1 ? b : P - 1;
    if (o->hi[d] < o->lo[d]) o->hi[d] = o->lo[d] - 1;
  }
  return kPrepMapped;
}

// One particle as the FP32 method's first pass needs it.
struct PrepLite {
  int64_t lo[3], hi[3];     // pix_index_min_max per axis, as PrepFP64
  float g[4];               // x - lo[0], y - lo[1], z - lo[2] and hsml, pixel units
  double m_in, rho_in, wgt, hsml;  // set when !f32
  float m32, rho32, w32;    // set when f32 (Float32 inputs, FP32 preparation)
  bool f32;
  bool scalar_zero;

  __device__ double mass() const { return f32 ? (double)m32 : m_in; }
  __device__ double rho() const { return f32 ? (double)rho32 : rho_in; }
  __device__ double weight() const { return f32 ? (double)w32 : wgt; }
  __device__ double h() const { return f32 ? (double)g[3] : hsml; }
};

// Error-free a + b == s + e (Knuth's TwoSum; no FMA contraction here).
__device__ __forceinline__ void prep_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// floor(xh + xl + hh + hl) from two unevaluated float sums (the pixel
// coordinate and +-hsml in pixels); false when the sum lies within `delta`
// of an integer.  s1 - floor(s1) is exact for |s1| < 2^23, so the only
// roundings are those of the small terms and of the final sum (at most
// 2^-23 absolute, as r < 2).
__device__ __forceinline__ bool floor_lite(float xh, float xl, float hh, float hl, float delta, int64_t* out) {
  float s1, e1;
  prep_two_sum(xh, hh, s1, e1);
  const float a = floorf(s1);
  const float r = (s1 - a) + ((e1 + xl) + hl);
  const float k = floorf(r);
  const float fr = r - k;
  if (!(fr >= delta && fr <= 1.0f - delta)) return false;
  *out = (int)(a + k);  // |a + k| < 2^23: a 32-bit conversion (64-bit ones take the FP64 pipe)
  return true;
}

// prep_particle_lite's FP64 path: prep_particle_fp64, results as PrepLite
// (out of line: it is the rare path, and inlined it costs the common one
// registers).
template <int DIMS>
__device__ __noinline__ int prep_lite_fp64(const DevParticles& pt, const DevMapParams& mp, int64_t p,
                                           bool store_pos, PrepLite* o) {
  o->f32 = false;
  PrepFP64 q;
  const int state = prep_particle_fp64<DIMS, false>(pt, mp, p, store_pos, &q);
  if (state == kPrepMapped) {
    const double xs[3] = {q.x, q.y, q.z};
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o->lo[d] = q.lo[d];
      o->hi[d] = q.hi[d];
      o->g[d] = d < DIMS ? __double2float_rn(xs[d] - (double)q.lo[d]) : 0.0f;
    }
    o->g[3] = __double2float_rn(q.hsml);
    o->m_in = q.m_in;
    o->rho_in = q.rho_in;
    o->wgt = q.wgt;
    o->hsml = q.hsml;
    o->scalar_zero = q.scalar_zero;
  }
  return state;
}

// The centring, filter, quantity skip and pixel ranges of prep_particle_fp64
// for FP32 inputs, in FP32 arithmetic (FP64 only to centre on a point that
// is not a float, and for periodic wrapping): the same state, the same
// centred positions and the same integer ranges, bit for bit.
//  - The filter compares the centred float against the box rounded inwards
//    to floats (set_lite_params), which is exact.
//  - pix_index_min_max takes floor(x -+ h) with x = c L + P/2 and h = hsml L
//    (cic_shared.jl:46-52, 85-99).  Here x and h L are unevaluated sums of
//    two floats (L = L_hi + L_lo; products split exactly by FMA), accurate
//    to about 2^-44 of M = |c L| + P/2 + |h L|; the reference's four FP64
//    roundings move its value by under 2^-50 M.  When the two-float value
//    is farther than delta = 2^-21 + 2^-36 M from every integer, the floor
//    of the reference's FP64 value is the floor of the two-float one.
//  - Otherwise (a value that close to an integer, M >= 2^22, non-finite
//    values, FP64 or rotated inputs) the particle is prepared by
//    prep_particle_fp64 from its untouched inputs.
//  - The centring is the reference's FP64 subtraction rounded to Float32;
//    when the centre is a float it is one FP32 subtraction, which is the
//    same: the difference of two floats is exact in FP64 unless their
//    exponents differ by more than 29, and then it is within half an FP32
//    ulp of the larger, far from an FP32 rounding boundary, so rounding it
//    to FP64 first does not change its FP32 rounding.
// The particle's inputs are all read first, so the loads overlap.  The
// record's FP32 offsets x - lo and hsml are rounded from the two-float
// sums (within an FP32 rounding of the FP64-derived values).
template <int DIMS>
__device__ __forceinline__ int prep_particle_lite(const DevParticles& pt, const DevMapParams& mp, int64_t p,
                                                  bool store_pos, PrepLite* o) {
  bool fp64 = !mp.lite || pt.pos_dtype != 0 || pt.attr_dtype != 0 || pt.xform == 2;
  int state = kPrepMapped;
  o->f32 = false;
  if (!fp64) {
    float c[3];
    int64_t off[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      off[d] = p * pt.sp + (pt.xform == 1 ? pt.perm[d] : d) * pt.sc;
      c[d] = __ldg((const float*)pt.pos + off[d]);
    }
    const float hin = __ldg((const float*)pt.hsml + p);
    const float q0 = pt.nq > 0 ? __ldg((const float*)pt.q + p * pt.qsp) : 0.0f;
    o->m32 = __ldg((const float*)pt.mass + p);
    o->rho32 = __ldg((const float*)pt.rho + p);
    o->w32 = __ldg((const float*)pt.w + p);
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float v = c[d];
      if (mp.center_mode != 0) {
        v = mp.cen_f_exact ? v - mp.cen_f[d] : __double2float_rn((double)v - mp.cen[d]);
        if (mp.periodic && fabs((double)v) > mp.boxsize / 2) {
          const double vd = v;
          v = __double2float_rn(vd > 0 ? vd - mp.boxsize / 2 : vd + mp.boxsize / 2);
        }
      }
      c[d] = v;
      if (mp.filter && !(mp.lo_f[d] <= v && v <= mp.hi_f[d])) in = false;
    }
    if (!in) {
      state = kPrepSkip;
    } else {
      bool allzero = q0 == 0.0f;
      for (int k = 1; k < pt.nq; ++k)
        if (__ldg((const float*)pt.q + p * pt.qsp + k * pt.qsk) != 0.0f) allzero = false;
      if (allzero && !mp.calc_mean) {
        state = kPrepZeroQ;
      } else {
        o->scalar_zero = (pt.nq > 1) && allzero;
        const float halfP = 0.5f * (float)mp.P;
        const float hh = hin * mp.L_hi;
        const float hl = fmaf(hin, mp.L_hi, -hh) + hin * mp.L_lo;
        o->g[3] = hh + hl;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          if (d >= DIMS) {
            o->lo[d] = 0;
            o->hi[d] = 0;
            o->g[d] = 0.0f;
            continue;
          }
          const float ph = c[d] * mp.L_hi;
          const float pe = fmaf(c[d], mp.L_hi, -ph);
          float xh, e0;
          prep_two_sum(ph, halfP, xh, e0);
          const float xl = (e0 + pe) + c[d] * mp.L_lo;
          const float M = (fabsf(ph) + halfP) + fabsf(hh) + 1.0f;
          int64_t a, b;
          if (!(M < 0x1p22f)) {
            fp64 = true;
            break;
          }
          const float delta = 0x1p-21f + M * 0x1p-36f;
          if (!floor_lite(xh, xl, -hh, -hl, delta, &a) || !floor_lite(xh, xl, hh, hl, delta, &b)) {
            fp64 = true;
            break;
          }
          const int64_t P = mp.P;
          o->lo[d] = a > 0 ? a : 0;
          o->hi[d] = b < P - 1 ? b : P - 1;
          if (o->hi[d] < o->lo[d]) o->hi[d] = o->lo[d] - 1;
          float g1, g2;
          prep_two_sum(xh, -(float)(int)o->lo[d], g1, g2);
          o->g[d] = g1 + (g2 + xl);
        }
        if (!fp64) o->f32 = true;  // m_in, rho_in, wgt and hsml left to the caller (m32, rho32, w32, g[3])
      }
    }
    if (!fp64) {
      if (mp.center_mode == 1 && store_pos && pt.xform == 0)
#pragma unroll
        for (int d = 0; d < 3; ++d) ((float*)pt.pos)[off[d]] = c[d];
      return state;
    }
  }
  PrepLite slow;  // only this path's copy leaves registers
  state = prep_lite_fp64<DIMS>(pt, mp, p, store_pos, &slow);
  *o = slow;
  return state;
}

// Offset of a pixel centre and the overlap of [x - h, x + h] with pixel i
// (get_x_dx / get_dxyz, cic_shared.jl:60-76).
__device__ __forceinline__ void cell_axis_fp64(double x, double h, int64_t i, double* dist, double* ov) {
  *dist = x - (double)i - 0.5;
  *ov = jmin(x + h, (double)(i + 1)) - jmax(x - h, (double)i);
}

// Distance u (in units of h) and area/volume overlap of one footprint cell
// (calculate_weights, cic_2D.jl:25-47, cic_3D.jl:28-53).
template <int DIMS>
__device__ __forceinline__ void cell_fp64(const PrepFP64& q, int64_t i, int64_t j, int64_t k, double* u, double* a) {
  double xd, dx, yd, dy;
  cell_axis_fp64(q.x, q.hsml, i, &xd, &dx);
  cell_axis_fp64(q.y, q.hsml, j, &yd, &dy);
  if (DIMS == 2) {
    *u = sqrt(xd * xd + yd * yd) * q.h_inv;
    *a = dx * dy;
  } else {
    double zd, dz;
    cell_axis_fp64(q.z, q.hsml, k, &zd, &dz);
    *a = dx * dy * dz;
    *u = sqrt(xd * xd + yd * yd + zd * zd) * q.h_inv;
  }
}

}  // namespace sphg
