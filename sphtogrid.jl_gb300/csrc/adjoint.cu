// adjoint.cu -- hand-written adjoint of the deposition (no counterpart in the
// reference).  Forward, per mapped particle p and footprint pixel x:
//
//   pw(p, x) = K_p g(p, x) / S_p,   S_p = sum_x g(p, x),
//   g = s(u) A   (A = overlap area/volume, s = kernel shape, u = |d|/h),
//   g = A        in the fallback branch (no pixel centre inside the kernel),
//   K_p = w m L^3 / rho (2D; times L in 3D)   -- the closed form of
//   cic_2D.jl:187-199 and cic_3D.jl:168-179,
//   W(x) = sum_p pw,  Q_k(x) = sum_p q_k pw,  out = Q / W (reduce_image.jl).
//
// Backward: k_adj_reduce turns dL/d(out) into dL/dQ_k and dL/dW per pixel;
// k_adj_particles (one warp per particle) recomputes the footprint weights --
// nothing of the forward's particle-pixel list is stored -- and gathers
//   gamma(x) = dL/dW + sum_k q_k dL/dQ_k,   Gamma = sum_x f gamma  (f = g/S),
//   dL/dK = Gamma,  dL/dq_k = sum_x pw dL/dQ_k,
//   dL/dtheta = (K/S) sum_x (gamma - Gamma) dg/dtheta   for theta = x, y, z, h,
// including the derivative of the renormalisation S.
//
// Two precisions: FP64 throughout, or (FP32C) the per-cell weights and
// derivatives in FP32 with compensated (TwoSum) sums per lane and warp, the
// per-particle finish in FP64.  The FP32 path redoes in FP64 the particles
// the forward would (every pixel centre near the kernel edge, or a tiny
// renormalisation sum), footprints of 2^20 cells or more and maps of more
// than kAdjQ32 quantities.
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"
#include "tiled.cuh"

namespace sphg {

namespace {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float wsumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// prep_particle_fp64 by lane 0, broadcast: the warp's lanes share one
// particle, and FP64 is a small fraction of FP32 throughput on this GPU.
// Every lane gets the state, the pixel coordinates, hsml, 1/hsml, the
// kernel normalisation, the pixel ranges and scalar_zero; the factors
// (area, col, vol, m, rho, w) stay on lane 0, which finishes the particle.
template <int DIMS>
__device__ __forceinline__ int prep_adj(const DevParticles& pt, const DevMapParams& mp, int64_t p, int lane,
                                        PrepFP64* q) {
  const unsigned full = 0xffffffffu;
  PrepFP64 v;
  v.x = v.y = v.z = v.hsml = v.h_inv = v.knorm = v.area = v.col = v.vol = v.m_in = v.rho_in = v.wgt = 0.0;
  for (int d = 0; d < 3; ++d) v.lo[d] = v.hi[d] = 0;
  v.scalar_zero = false;
  int state = kPrepSkip;
  if (lane == 0) state = prep_particle_fp64<DIMS>(pt, mp, p, false, &v);
  *q = v;
  state = __shfl_sync(full, state, 0);
  q->x = __shfl_sync(full, v.x, 0);
  q->y = __shfl_sync(full, v.y, 0);
  q->z = __shfl_sync(full, v.z, 0);
  q->hsml = __shfl_sync(full, v.hsml, 0);
  q->h_inv = __shfl_sync(full, v.h_inv, 0);
  q->knorm = __shfl_sync(full, v.knorm, 0);
  for (int d = 0; d < 3; ++d) {
    q->lo[d] = __shfl_sync(full, (long long)v.lo[d], 0);
    q->hi[d] = __shfl_sync(full, (long long)v.hi[d], 0);
  }
  q->scalar_zero = __shfl_sync(full, v.scalar_zero ? 1 : 0, 0) != 0;
  return state;
}

// Derivative of the un-normalised kernel shape, u < 1.
template <int KERN>
__device__ __forceinline__ double kshape_du(double u) {
  if (u >= 1.0) return 0.0;
  if (KERN == 0) {
    if (u < 0.5) return -12.0 * u + 18.0 * u * u;
    const double t = 1.0 - u;
    return -6.0 * t * t;
  } else if (KERN == 1) {
    const double a = 1.0 - u, b = 2.0 / 3.0 - u, c = 1.0 / 3.0 - u;
    const double a4 = a * a * a * a, b4 = b * b * b * b, c4 = c * c * c * c;
    if (u < 1.0 / 3.0) return -5.0 * a4 + 30.0 * b4 - 75.0 * c4;
    if (u < 2.0 / 3.0) return -5.0 * a4 + 30.0 * b4;
    return -5.0 * a4;
  } else if (KERN == 2) {
    const double t = 1.0 - u, t2 = t * t, t5 = t2 * t2 * t;
    const double p = 1.0 + 6.0 * u + 35.0 / 3.0 * u * u;
    return -6.0 * t5 * p + t5 * t * (6.0 + 70.0 / 3.0 * u);
  } else if (KERN == 3) {
    const double t = 1.0 - u, t2 = t * t, t4 = t2 * t2, t7 = t4 * t2 * t;
    const double p = 1.0 + 8.0 * u + 25.0 * u * u + 32.0 * u * u * u;
    return -8.0 * t7 * p + t7 * t * (8.0 + 50.0 * u + 96.0 * u * u);
  } else {
    const double t = 1.0 - u, t2 = t * t, t4 = t2 * t2, t9 = t4 * t4 * t;
    const double u2 = u * u;
    const double p = 1.0 + 10.0 * u + 42.0 * u2 + 90.0 * u2 * u + 429.0 / 5.0 * u2 * u2;
    return -10.0 * t9 * p + t9 * t * (10.0 + 84.0 * u + 270.0 * u2 + 1716.0 / 5.0 * u2 * u);
  }
}

// FP32 derivative of the un-normalised kernel shape, u < 1 (kshape_du in
// FP32, the same polynomials).
template <int KERN>
__device__ __forceinline__ float kshape_du_f(float u) {
  if (u >= 1.0f) return 0.0f;
  if (KERN == 0) {
    if (u < 0.5f) return u * fmaf(18.0f, u, -12.0f);
    const float t = 1.0f - u;
    return -6.0f * t * t;
  } else if (KERN == 1) {
    const float a = 1.0f - u, b = (2.0f / 3.0f) - u, c = (1.0f / 3.0f) - u;
    const float a2 = a * a, b2 = b * b, c2 = c * c;
    const float a4 = a2 * a2, b4 = b2 * b2, c4 = c2 * c2;
    if (u < 1.0f / 3.0f) return fmaf(-75.0f, c4, fmaf(30.0f, b4, -5.0f * a4));
    if (u < 2.0f / 3.0f) return fmaf(30.0f, b4, -5.0f * a4);
    return -5.0f * a4;
  } else if (KERN == 2) {
    const float t = 1.0f - u, t2 = t * t, t5 = t2 * t2 * t;
    const float p = fmaf(u, fmaf(35.0f / 3.0f, u, 6.0f), 1.0f);
    return t5 * fmaf(t, fmaf(70.0f / 3.0f, u, 6.0f), -6.0f * p);
  } else if (KERN == 3) {
    const float t = 1.0f - u, t2 = t * t, t4 = t2 * t2, t7 = t4 * t2 * t;
    const float p = fmaf(u, fmaf(u, fmaf(32.0f, u, 25.0f), 8.0f), 1.0f);
    return t7 * fmaf(t, fmaf(u, fmaf(96.0f, u, 50.0f), 8.0f), -8.0f * p);
  } else {
    const float t = 1.0f - u, t2 = t * t, t4 = t2 * t2, t9 = t4 * t4 * t;
    const float p = fmaf(u, fmaf(u, fmaf(u, fmaf(429.0f / 5.0f, u, 90.0f), 42.0f), 10.0f), 1.0f);
    return t9 * fmaf(t, fmaf(u, fmaf(u, fmaf(1716.0f / 5.0f, u, 270.0f), 84.0f), 10.0f), -10.0f * p);
  }
}

// dL/d(out) -> dL/dQ_k, dL/dW in raw row order (row = i*P + j or i*P^2 + j*P + k);
// g32 (FP32 path): the same [nq][PD] then [PD] as FP32 (hi, lo) pairs, the
// nq + 1 planes of hi = float(v) and then the nq + 1 planes of
// lo = float(v - hi), so hi + lo carries v to about 48 bits.
__global__ void __launch_bounds__(256) k_adj_reduce(const double* __restrict__ raw, const double* __restrict__ g,
                                                     int dims, int64_t P, int nq, int mode, int reduce,
                                                     double* __restrict__ gq, double* __restrict__ gw,
                                                     float* __restrict__ g32) {
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < PD;
       row += (int64_t)gridDim.x * blockDim.x) {
    const double W = raw[row + (int64_t)nq * PD];
    double dw = 0.0;
    if (dims == 3) {
      const double Q = raw[row];
      const double G = g[row];  // out[z, y, x] is column-major row i*P^2 + j*P + k
      if (mode == 1) {          // raw accumulator requested
        gq[row] = G;
        dw = g[row + PD];
      } else if (Q > 0.0 && reduce) {
        gq[row] = G / W;
        dw = -G * Q / (W * W);
      } else {
        gq[row] = G;
      }
    } else if (mode == 1) {
      for (int c = 0; c < nq; ++c) gq[row + c * PD] = g[row + c * PD];
      dw = g[row + (int64_t)nq * PD];
    } else {
      const int64_t i = row / P, j = row - (row / P) * P;
      const bool div = reduce && W > 0.0;
      for (int c = 0; c < nq; ++c) {
        const double G = g[i + P * j + PD * c];
        const double Q = raw[row + c * PD];
        gq[row + c * PD] = div ? G / W : G;
        if (div) dw -= G * Q / (W * W);
      }
    }
    gw[row] = dw;
    if (g32) {
      const int64_t LO = (int64_t)(nq + 1) * PD;
      for (int c = 0; c <= nq; ++c) {
        const double v = c < nq ? gq[row + c * PD] : dw;
        const float hv = (float)v;
        g32[row + c * PD] = hv;
        g32[LO + row + c * PD] = (float)(v - (double)hv);
      }
    }
  }
}

// FP32 path: a particle whose FP32 result misses the relative test of its
// own values waits for the second pass with its error estimates in output
// units (pos x, y, z and hsml; the absolute error of dL/dK; q_0..q_3).
struct AdjPending {
  long long p;
  float e[9];
  float pad;
};
// Scales of the second pass's test: the largest |value| of each output kind
// over all particles (float bits, atomic max): pos, hsml, mass, rho, w, q.
constexpr int kAdjScales = 6;

struct AdjArgs {
  DevParticles pt;
  DevMapParams mp;
  const double* gq;  // [nq][PD]
  const double* gw;  // [PD]
  const float* g32;  // FP32 path: gq then gw as FP32 (hi, lo) planes, or NULL (FP64 throughout)
  int64_t PD;
  double* d_pos;     // strides of pt.pos
  double *d_hsml, *d_mass, *d_rho, *d_w;
  double* d_q;       // strides of pt.q
  DevStatus* st;
  unsigned* scale;   // FP32 path: [kAdjScales], then the pending count
  unsigned* n_pend;
  AdjPending* pend;  // [n]
};

// Maps of at most this many quantities take the FP32 path.
constexpr int kAdjQ32 = 4;

// Below this u (within a few ulp of the forward's) the forward's u is < 1.
constexpr double kSureU = 0.9999999;

// A warp's per-axis terms of one footprint (shared memory): entry e < ni for
// column i = iMin + e, then nj entries for the rows, then nk (3D); formed
// once per footprint instead of once per cell, in the same FP64 operations.
constexpr int kAxisTab = 256;
struct AxisTab {
  double dist[kAxisTab], ov[kAxisTab];
  signed char dox[kAxisTab], doh[kAxisTab];
};

// One mapped particle in FP64 (the warp's lanes stride over its footprint):
// grad (x, y, z, h in pixel units), dL/dK and dL/dq_k.  u is the forward's
// to a few ulp (cell_fp64 forms sqrt(r^2) * (1/h)); a cell it moves across
// u = 1 has a weight and a derivative of order (1 - u)^2 or less, nil.  The
// forward's branch -- the fallback g = A where its renormalisation sum is
// zero -- is settled inside the pass that gathers the sums: a cell with
// u < kSureU at positive overlap has a positive term (every kernel shape is
// positive below u = 1, at least (2^-53)^10 there), and with no negative
// overlap in the footprint the sum is then positive.  Only a particle
// without such a cell (sub-pixel ones) runs the sum as a pass of its own,
// and the sums again on its branch.  tab: the warp's axis table, or NULL
// (terms formed per cell, as for footprints of more than kAxisTab axis
// entries).
template <int DIMS, int KERN>
__device__ void adj_particle_fp64(const AdjArgs& A, int64_t p, const PrepFP64& q, int lane, double grad[4],
                                  double& dK, double* dqk, AxisTab* tab) {
  const unsigned full = 0xffffffffu;
  const DevParticles& pt = A.pt;
  const double L = A.mp.L;
  const int64_t P = A.mp.P;
  const int nq = pt.nq;
  const int64_t iMin = q.lo[0], jMin = q.lo[1], kMin = q.lo[2];
  const int64_t ni = q.hi[0] - iMin + 1, nj = q.hi[1] - jMin + 1, nk = q.hi[2] - kMin + 1;
  const int64_t njk = nj * nk, F = ni * njk;
  const double xs[3] = {q.x, q.y, q.z};
  const double h = q.hsml, h_inv = q.h_inv;
  const int64_t ntab = ni + nj + (DIMS == 3 ? nk : 0);
  const bool use_tab = tab != nullptr && ntab <= kAxisTab;  // warp-uniform
  if (use_tab) {
    __syncwarp();  // the warp's previous footprint is read
    for (int e = lane; e < ntab; e += 32) {
      const int d = e < ni ? 0 : (e < ni + nj ? 1 : 2);
      const double x = d == 0 ? q.x : (d == 1 ? q.y : q.z);
      const int64_t c = d == 0 ? iMin + e : (d == 1 ? jMin + (e - ni) : kMin + (e - ni - nj));
      cell_axis_fp64(x, h, c, &tab->dist[e], &tab->ov[e]);
      const bool up = x + h < (double)(c + 1);
      const bool dn = x - h > (double)c;
      tab->dox[e] = (signed char)((up ? 1 : 0) - (dn ? 1 : 0));
      tab->doh[e] = (signed char)((up ? 1 : 0) + (dn ? 1 : 0));
    }
    __syncwarp();
  }
  double S, sgg, sgd[4], sd[4], sq[kMaxQ];
  bool fallback = false, decided = false;
  for (;;) {
    S = sgg = 0.0;
    for (int t = 0; t < 4; ++t) sgd[t] = sd[t] = 0.0;
    for (int k = 0; k < nq; ++k) sq[k] = 0.0;
    bool pos_term = false, neg_term = false;
    for (int64_t f = lane; f < F; f += 32) {
      const int64_t ia = f / njk, r = f - ia * njk, jb = r / nk, kc = r - jb * nk;
      const int64_t cell[3] = {iMin + ia, jMin + jb, kMin + kc};
      double dist[3] = {0, 0, 0}, ov[3] = {1, 1, 1}, dox[3] = {0, 0, 0}, doh[3] = {0, 0, 0};
      for (int d = 0; d < DIMS; ++d) {
        if (use_tab) {
          const int e = (int)(d == 0 ? ia : (d == 1 ? ni + jb : ni + nj + kc));
          dist[d] = tab->dist[e];
          ov[d] = tab->ov[e];
          dox[d] = (double)tab->dox[e];
          doh[d] = (double)tab->doh[e];
        } else {
          cell_axis_fp64(xs[d], h, cell[d], &dist[d], &ov[d]);
          const bool up = xs[d] + h < (double)(cell[d] + 1);  // min() takes x + h
          const bool dn = xs[d] - h > (double)cell[d];        // max() takes x - h
          dox[d] = (up ? 1.0 : 0.0) - (dn ? 1.0 : 0.0);
          doh[d] = (up ? 1.0 : 0.0) + (dn ? 1.0 : 0.0);
        }
      }
      const double A_ = ov[0] * ov[1] * ov[2];
      double dA[4];
      dA[3] = 0.0;
      for (int d = 0; d < 3; ++d) {
        double rest = 1.0;
        for (int e = 0; e < 3; ++e)
          if (e != d) rest *= ov[e];
        dA[d] = d < DIMS ? dox[d] * rest : 0.0;
        if (d < DIMS) dA[3] += doh[d] * rest;
      }
      double r2 = dist[0] * dist[0] + dist[1] * dist[1];
      if (DIMS == 3) r2 += dist[2] * dist[2];
      // r and 1/r from one reciprocal square root (1 ulp), so u is within a
      // few ulp of the forward's
      const double rs = r2 > 0.0 ? rsqrt(r2) : 0.0;
      const double u = r2 * rs * h_inv;
      pos_term = pos_term || (u < kSureU && A_ > 0.0);
      neg_term = neg_term || A_ < 0.0;
      double g, dg[4];
      if (fallback) {
        g = A_;
        for (int t = 0; t < 4; ++t) dg[t] = dA[t];
      } else if (u <= 1.0) {
        const double s = kshape<KERN, double>(u), sp = kshape_du<KERN>(u);
        const double irh = rs * h_inv;  // du/dx_d = dist_d / (r h)
        g = s * A_;
        for (int d = 0; d < DIMS; ++d) dg[d] = sp * (dist[d] * irh) * A_ + s * dA[d];
        if (DIMS == 2) dg[2] = 0.0;
        dg[3] = sp * (-u * h_inv) * A_ + s * dA[3];
      } else {
        g = 0.0;
        dg[0] = dg[1] = dg[2] = dg[3] = 0.0;
      }
      const int64_t idx = DIMS == 2 ? cell[0] * P + cell[1] : (cell[0] * P + cell[1]) * P + cell[2];
      double gam = A.gw[idx];
      for (int k = 0; k < nq; ++k) {
        const double gqk = A.gq[k * A.PD + idx];
        const double qk = q.scalar_zero ? 0.0 : ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + k * pt.qsk);
        gam += qk * gqk;
        sq[k] += g * gqk;
      }
      S += g;
      sgg += gam * g;
      for (int t = 0; t < 4; ++t) {
        if (DIMS == 2 && t == 2) continue;
        sgd[t] += gam * dg[t];
        sd[t] += dg[t];
      }
    }
    S = wsum(S);
    sgg = wsum(sgg);
    for (int t = 0; t < 4; ++t) {
      if (DIMS == 2 && t == 2) continue;
      sgd[t] = wsum(sgd[t]);
      sd[t] = wsum(sd[t]);
    }
    for (int k = 0; k < nq; ++k) sq[k] = wsum(sq[k]);
    if (decided || (__any_sync(full, pos_term) && !__any_sync(full, neg_term))) break;
    // the forward's renormalisation sum as a pass of its own, then the sums
    // again (recomputed rather than kept live across that pass)
    double s_w = 0.0;
    for (int64_t f = lane; f < F; f += 32) {
      const int64_t ia = f / njk, r = f - ia * njk, jb = r / nk, kc = r - jb * nk;
      double uc, a;
      cell_fp64<DIMS>(q, iMin + ia, jMin + jb, kMin + kc, &uc, &a);
      if (uc <= 1.0) s_w += kshape<KERN, double>(uc) * a;
    }
    fallback = wsum(s_w) == 0.0;
    decided = true;
  }
  const double K = DIMS == 2 ? q.area * q.wgt * q.col : q.vol * q.wgt * L;
  if (S > 0.0) {
    const double Gam = sgg / S;
    dK = Gam;
    for (int t = 0; t < 4; ++t) grad[t] = K / S * (sgd[t] - Gam * sd[t]);
    for (int k = 0; k < nq; ++k) dqk[k] = K / S * sq[k];
  }
}

// A compensated FP32 sum (s, c) reduced over the warp, as FP64.
__device__ __forceinline__ double comp_total(float s, float c) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float so = __shfl_xor_sync(0xffffffffu, s, o), co = __shfl_xor_sync(0xffffffffu, c, o);
    float t, e;
    two_sum(s, so, t, e);
    s = t;
    c = c + co + e;
  }
  return (double)s + (double)c;
}

__device__ __forceinline__ void comp_add(float& s, float& c, float v) {
  float t, e;
  two_sum(s, v, t, e);
  s = t;
  c += e;
}

// Overlap, centre offset and overlap derivatives of footprint-local pixel a
// along one axis, f the particle's offset from the footprint origin.
__device__ __forceinline__ void axis_terms_f(float f, float h, int a, float& dist, float& ov, float& dox,
                                             float& doh) {
  const float fa = (float)a;
  dist = f - fa - 0.5f;
  ov = fminf(f + h, fa + 1.0f) - fmaxf(f - h, fa);
  const bool up = f + h < fa + 1.0f, dn = f - h > fa;
  dox = (up ? 1.0f : 0.0f) - (dn ? 1.0f : 0.0f);
  doh = (up ? 1.0f : 0.0f) + (dn ? 1.0f : 0.0f);
}

// Error estimate of the FP32 path.  The image gradient gam = dL/dW +
// sum_k q_k dL/dQ_k is formed per cell from FP32 (hi, lo) pairs of its
// factors with exact products (FMA) and exact sums (TwoSum), about 48 bits
// (its parts cancel where q is near the map value), and rounded once; the
// error of that formation stays below kGamEps (|dL/dW| + sum_k |q_k dL/dQ_k|)
// and is added to each term's.  A per-cell weight or derivative
// carries a relative rounding error of about kTermEps (a few tens of FP32
// operations), amplified near the kernel edge, where (1 - u)^k turns the
// rounding of u into kEdgeEps / (1 - u).  The terms' errors are independent,
// so a sum's error is estimated as three times the root of the summed
// squared term errors.  A result is kept when that estimate is within
// kKeepRel of it (the adjoint's bar is 1e-4); otherwise the particle is
// redone in FP64.
constexpr float kTermEps = 5e-7f;
constexpr float kEdgeEps = 6e-7f;
constexpr double kKeepRel = 2e-5;
constexpr float kGamEps = 9.1e-13f;  // 2^-40: representation, cross products, low-part sums

// The warp sums of one particle on the FP32 path and their rounding
// estimates (B: of sgg, then of the four sgd; Bd of sd; Bq of sq).
struct Adj32Sums {
  double S, sgg, Gam1, sgd[4], sd[4], sq[kAdjQ32], B[5];
  float Bd[4], Bq[kAdjQ32];
};

// The FP32 path's finish of one particle, by the lane that holds the
// particle (q: its own preparation, with the factors): 1 when every result
// passes the relative test, else 2 after queueing the particle for
// k_adj_pending with its errors in output units (pos and hsml carry L, as
// the outputs do).
template <int DIMS>
__device__ __noinline__ int adj_finish32(const AdjArgs& A, int64_t p, const PrepFP64& q, const Adj32Sums& u,
                                         double grad[4], double& dK, double* dqk) {
  const int nq = A.pt.nq;
  const double S = u.S, sgg = u.sgg, Gam1 = u.Gam1;
  const double *sgd = u.sgd, *sd = u.sd, *sq = u.sq, *B = u.B;
  const float *Bd = u.Bd, *Bq = u.Bq;
  const double BG = B[0];
  const double Gam = sgg / S;
  const double relG = BG / fabs(sgg);  // relative error of Gam (S is a sum of positive terms)
  bool keep = !(relG > kKeepRel);  // (0 / 0 when every term is 0: kept)
  // sum (gam - Gam) dg = sum (gam - Gam1) dg - (Gam - Gam1) sum dg
  const double dG = Gam - Gam1;
  const double K = DIMS == 2 ? q.area * q.wgt * q.col : q.vol * q.wgt * A.mp.L;
  double val[4], err[4];
  for (int t = 0; t < 4; ++t) {
    val[t] = sgd[t] - dG * sd[t];
    err[t] = B[1 + t] + fabs(dG) * (double)Bd[t] + fabs(Gam * sd[t]) * (sgg != 0.0 ? relG : 0.0);
    if (err[t] > kKeepRel * fabs(val[t])) keep = false;
  }
  for (int k = 0; k < nq; ++k)
    if ((double)Bq[k] > kKeepRel * fabs(sq[k])) keep = false;
  dK = Gam;
  for (int t = 0; t < 4; ++t) grad[t] = K / S * val[t];
  for (int k = 0; k < nq; ++k) dqk[k] = K / S * sq[k];
  if (keep) return 1;
  AdjPending e;
  e.p = p;
  for (int t = 0; t < 4; ++t) e.e[t] = (float)(fabs(K / S) * err[t] * A.mp.L);
  e.e[4] = (float)(BG / S);
  for (int k = 0; k < kAdjQ32; ++k) e.e[5 + k] = k < nq ? (float)(fabs(K / S) * (double)Bq[k]) : 0.0f;
  e.pad = 0.0f;
  A.pend[atomicAdd(A.n_pend, 1u)] = e;
  return 2;
}

// One mapped particle on the FP32 path, the warp over its footprint (q:
// the particle's preparation, on every lane).  Returns 0 for the particles
// it leaves to the FP64 path (those the forward redoes in FP64, maps of
// more than kAdjQ32 quantities, footprints of 2^20 cells or more); else 1
// after lane 0 has stored the warp sums and their rounding estimates in
// *out for the particle's own lane to finish (adj_finish32).
template <int DIMS, int KERN>
__device__ int adj_fp32_sums(const AdjArgs& A, int64_t p, const PrepFP64& q, int lane, Adj32Sums* out) {
  const DevParticles& pt = A.pt;
  const int nq = pt.nq;
  if (nq > kAdjQ32) return 0;
  const int64_t ni = q.hi[0] - q.lo[0] + 1, nj = q.hi[1] - q.lo[1] + 1, nk = q.hi[2] - q.lo[2] + 1;
  if (ni * nj * nk >= (1 << 20)) return 0;
  const int F = (int)(ni * nj * nk), njk = (int)(nj * nk), nkk = (int)nk;
  const float inv_njk = inv_small(njk), inv_nk = inv_small(nkk);
  // the particle relative to its footprint origin (FP64 -> FP32 once)
  const float fx = (float)(q.x - (double)q.lo[0]), fy = (float)(q.y - (double)q.lo[1]);
  const float fz = DIMS == 3 ? (float)(q.z - (double)q.lo[2]) : 0.0f;
  const float h = (float)q.hsml, hinv = 1.0f / h;
  float qh[kAdjQ32], ql[kAdjQ32];  // q_k as FP32 (hi, lo)
  for (int k = 0; k < kAdjQ32; ++k) {
    const double v = (k < nq && !q.scalar_zero) ? ld_elem(pt.attr_dtype, pt.q, p * pt.qsp + k * pt.qsk) : 0.0;
    qh[k] = (float)v;
    ql[k] = (float)(v - (double)qh[k]);
  }
  const int64_t P = A.mp.P;
  const int64_t i0 = q.lo[0], j0 = q.lo[1], k0 = q.lo[2];
  const float* gh = A.g32;
  const float* gl = A.g32 + (int64_t)(nq + 1) * A.PD;
  // the image gradient at a footprint pixel (see kGamEps), rounded once;
  // mag: |dL/dW| + sum_k |q_k dL/dQ_k|, the scale of its formation error
  auto gamma_at = [&](int64_t idx, float& mag) {
    float s = gh[(int64_t)nq * A.PD + idx], e = gl[(int64_t)nq * A.PD + idx];
    mag = fabsf(s);
    for (int k = 0; k < kAdjQ32; ++k) {
      if (k >= nq) break;
      const float gqh = gh[k * A.PD + idx], gql = gl[k * A.PD + idx];
      const float pr = qh[k] * gqh, pe = fmaf(qh[k], gqh, -pr);  // qh gqh = pr + pe exactly
      const float t = s + pr, bp = t - s, se = (s - (t - bp)) + (pr - bp);  // s + pr = t + se exactly
      s = t;
      e += (se + pe) + (qh[k] * gql + ql[k] * gqh);
      mag += fabsf(pr);
    }
    return s + e;
  };
  // pass 1: renormalisation sum, the smallest u (the forward's test) and
  // the weighted mean Gam1 of gam, which pass 2 subtracts from every term
  float s1 = 0.0f, c1 = 0.0f, umin = 3.0e38f, sG1 = 0.0f, cG1 = 0.0f;
  for (int f = lane; f < F; f += 32) {
    const int a = fdiv(f, inv_njk), r = f - a * njk;
    const int b = fdiv(r, inv_nk), c = r - b * nkk;
    float dx, ox, t0, t1, dy, oy, dz = 0.0f, oz = 1.0f;
    axis_terms_f(fx, h, a, dx, ox, t0, t1);
    axis_terms_f(fy, h, b, dy, oy, t0, t1);
    if (DIMS == 3) axis_terms_f(fz, h, c, dz, oz, t0, t1);
    const float u = u_of((dx * dx + dy * dy) + dz * dz, hinv);
    umin = fminf(umin, u);
    if (u <= 1.0f) {
      const float g = kshape_f<KERN>(u) * (ox * oy * oz);
      comp_add(s1, c1, g);
      const int64_t idx = DIMS == 2 ? (i0 + a) * P + (j0 + b) : ((i0 + a) * P + (j0 + b)) * P + (k0 + c);
      float mag;
      comp_add(sG1, cG1, gamma_at(idx, mag) * g);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) umin = fminf(umin, __shfl_xor_sync(0xffffffffu, umin, o));
  const double S1 = comp_total(s1, c1);
  if (ill_conditioned((float)S1, umin)) return 0;  // warp-uniform
  const float Gam1 = (float)(comp_total(sG1, cG1) / S1);
  // pass 2: g, its derivatives and the image gradients (compensated sums)
  float aS = 0, cS = 0, aG = 0, cG = 0, agd[4] = {}, cgd[4] = {}, ad[4] = {}, cd[4] = {};
  float aq[kAdjQ32] = {}, cq[kAdjQ32] = {};
  // sums of the squared term errors: each sum's rounding estimate
  float bG = 0, bgd[4] = {}, bd[4] = {}, bq[kAdjQ32] = {};
  for (int f = lane; f < F; f += 32) {
    const int a = fdiv(f, inv_njk), r = f - a * njk;
    const int b = fdiv(r, inv_nk), c = r - b * nkk;
    float dist[3] = {0.0f, 0.0f, 0.0f}, ov[3] = {1.0f, 1.0f, 1.0f}, dox[3] = {0, 0, 0}, doh[3] = {0, 0, 0};
    axis_terms_f(fx, h, a, dist[0], ov[0], dox[0], doh[0]);
    axis_terms_f(fy, h, b, dist[1], ov[1], dox[1], doh[1]);
    if (DIMS == 3) axis_terms_f(fz, h, c, dist[2], ov[2], dox[2], doh[2]);
    const float u = u_of((dist[0] * dist[0] + dist[1] * dist[1]) + dist[2] * dist[2], hinv);
    if (!(u <= 1.0f)) continue;  // no weight, no derivative
    const float A_ = ov[0] * ov[1] * ov[2];
    float dA[4];
    dA[0] = dox[0] * ov[1] * ov[2];
    dA[1] = dox[1] * ov[0] * ov[2];
    dA[2] = DIMS == 3 ? dox[2] * ov[0] * ov[1] : 0.0f;
    dA[3] = doh[0] * ov[1] * ov[2] + doh[1] * ov[0] * ov[2] + (DIMS == 3 ? doh[2] * ov[0] * ov[1] : 0.0f);
    const float s = kshape_f<KERN>(u), sp = kshape_du_f<KERN>(u);
    const float g = s * A_;
    const float rr = u * h;  // |d|
    const float dudr = rr > 0.0f ? sp * A_ / (rr * h) : 0.0f;  // d(s A)/d(dist) per unit offset
    float dg[4];
    for (int d = 0; d < 3; ++d) dg[d] = (d < DIMS ? dudr * dist[d] : 0.0f) + s * dA[d];
    dg[3] = sp * (-u * hinv) * A_ + s * dA[3];
    const int64_t idx = DIMS == 2 ? (i0 + a) * P + (j0 + b) : ((i0 + a) * P + (j0 + b)) * P + (k0 + c);
    const float eps = kTermEps + kEdgeEps / fmaxf(1.0f - u, 1e-30f);  // this cell's terms
    for (int k = 0; k < kAdjQ32; ++k) {
      if (k >= nq) break;
      const float gqk = A.g32[k * A.PD + idx];
      comp_add(aq[k], cq[k], g * gqk);
      const float eq = eps * g * gqk;
      bq[k] = fmaf(eq, eq, bq[k]);
    }
    float mag;
    const float gam = gamma_at(idx, mag), dgam = gam - Gam1;
    const float gerr = kGamEps * mag;  // gam's formation error
    comp_add(aS, cS, g);
    comp_add(aG, cG, gam * g);
    const float tg = (eps * fabsf(gam) + gerr) * g;
    bG = fmaf(tg, tg, bG);
    // squared error weight of a term (gam - Gam1) x
    const float eg = eps * fabsf(dgam) + gerr;
    const float w2 = eg * eg;
    for (int t = 0; t < 4; ++t) {
      comp_add(agd[t], cgd[t], dgam * dg[t]);
      comp_add(ad[t], cd[t], dg[t]);
      bgd[t] = fmaf(dg[t] * dg[t], w2, bgd[t]);
      const float ed = eps * dg[t];
      bd[t] = fmaf(ed, ed, bd[t]);
    }
  }
  const double S = comp_total(aS, cS), sgg = comp_total(aG, cG);
  double sgd[4], sd[4];
  for (int t = 0; t < 4; ++t) {
    sgd[t] = comp_total(agd[t], cgd[t]);
    sd[t] = comp_total(ad[t], cd[t]);
  }
  double sq[kAdjQ32];
  for (int k = 0; k < kAdjQ32; ++k) sq[k] = comp_total(aq[k], cq[k]);
  // the rounding estimates: three times the root of the warp sums (FP32:
  // estimates of sums of squared FP32 term errors)
  const float BG = 3.0f * sqrtf(wsumf(bG));
  for (int t = 0; t < 4; ++t) {
    bgd[t] = 3.0f * sqrtf(wsumf(bgd[t]));
    bd[t] = 3.0f * sqrtf(wsumf(bd[t]));
  }
  for (int k = 0; k < kAdjQ32; ++k) bq[k] = 3.0f * sqrtf(wsumf(bq[k]));
  if (!(S > 0.0)) return 0;  // warp-uniform
  if (lane == 0) {
    out->S = S;
    out->sgg = sgg;
    out->Gam1 = (double)Gam1;
    out->B[0] = BG;
    for (int t = 0; t < 4; ++t) {
      out->sgd[t] = sgd[t];
      out->sd[t] = sd[t];
      out->B[1 + t] = bgd[t];
      out->Bd[t] = bd[t];
    }
    for (int k = 0; k < kAdjQ32; ++k) {
      out->sq[k] = sq[k];
      out->Bq[k] = bq[k];
    }
  }
  return 1;
}

// Lane 0 writes particle p's derivatives (dK, grad in pixel units, dqk)
// into the outputs and returns, in v, their magnitudes per output kind.
template <int DIMS>
__device__ void write_outputs(const AdjArgs& A, int64_t p, int state, const PrepFP64& q, const double grad[4],
                              double dK, const double* dqk, float v[kAdjScales]) {
  const DevParticles& pt = A.pt;
  const double L = A.mp.L;
  // K = w m L^3 / rho (2D), times L in 3D
  const double LD = DIMS == 2 ? L * L * L : L * L * L * L;
  const double m_in = state == kPrepMapped ? q.m_in : 0.0;
  const double rho_in = state == kPrepMapped ? q.rho_in : 1.0;
  const double w_in = state == kPrepMapped ? q.wgt : 0.0;
  const double dw = dK * m_in * LD / rho_in, dm = dK * w_in * LD / rho_in;
  const double dr = -dK * w_in * m_in * LD / (rho_in * rho_in);
  A.d_w[p] = dw;
  A.d_mass[p] = dm;
  A.d_rho[p] = dr;
  A.d_hsml[p] = grad[3] * L;
  float vp = 0.0f, vq = 0.0f;
  for (int d = 0; d < 3; ++d) {
    A.d_pos[p * pt.sp + d * pt.sc] = grad[d] * L;
    vp = fmaxf(vp, (float)fabs(grad[d] * L));
  }
  for (int k = 0; k < pt.nq; ++k) {
    A.d_q[p * pt.qsp + k * pt.qsk] = dqk[k];
    vq = fmaxf(vq, (float)fabs(dqk[k]));
  }
  v[0] = vp;
  v[1] = (float)fabs(grad[3] * L);
  v[2] = (float)fabs(dm);
  v[3] = (float)fabs(dr);
  v[4] = (float)fabs(dw);
  v[5] = vq;
}

// The largest magnitude of each output kind over a CTA's particles (each
// warp's in vmax[warp], kept by its lane 0), added to the scales with one
// atomic each.
__device__ void flush_scales(const AdjArgs& A, float (*vmax)[kAdjScales]) {
  __syncthreads();
  if (threadIdx.x < kAdjScales) {
    float m = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5) && w < 8; ++w) m = fmaxf(m, vmax[w][threadIdx.x]);
    atomicMax(A.scale + threadIdx.x, __float_as_uint(m));  // non-negative floats order as their bits
  }
}

// The FP64 path: every particle in FP64, a warp each.
template <int DIMS, int KERN>
__global__ void __launch_bounds__(256, 2) k_adj_particles(AdjArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const DevParticles& pt = A.pt;
  const int nq = pt.nq;
  __shared__ AxisTab tabs[8];
  AxisTab* tab = &tabs[threadIdx.x >> 5];
  for (int64_t p = wid; p < pt.n; p += nw) {
    PrepFP64 q;
    const int state = prep_adj<DIMS>(pt, A.mp, p, lane, &q);
    double grad[4] = {0.0, 0.0, 0.0, 0.0};  // x, y, z, h (pixel units)
    double dK = 0.0, dqk[kMaxQ];
    for (int k = 0; k < nq; ++k) dqk[k] = 0.0;
    if (state == kPrepMapped) adj_particle_fp64<DIMS, KERN>(A, p, q, lane, grad, dK, dqk, tab);
    if (lane == 0) {
      float v[kAdjScales];
      write_outputs<DIMS>(A, p, state, q, grad, dK, dqk, v);
    }
  }
}

// First pass of the FP32 path, a warp per group of 32 particles: the lanes
// prepare their particles side by side (FP64, one particle each, into
// shared memory), the warp sums each particle's footprint in FP32 (or does
// it in FP64 where the forward would), and the lanes finish their particles
// side by side again (FP64), so the per-particle FP64 work -- a small
// fraction of FP32 throughput on this GPU -- costs one warp instruction
// stream per 32 particles.  A particle whose FP32 results miss the relative
// test is written and queued for the second pass.  Maps of at most
// kAdjQ32 quantities; four warps per CTA, so a group's preparations and
// sums fit in static shared memory.
template <int DIMS, int KERN>
__global__ void __launch_bounds__(128, 4) k_adj_particles32(AdjArgs A) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = (threadIdx.x >> 5) & 3;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const DevParticles& pt = A.pt;
  const int nq = pt.nq;
  __shared__ PrepFP64 qs[4][32];
  __shared__ Adj32Sums sums[4][32];
  __shared__ float vmax[8][kAdjScales];
  float vm[kAdjScales] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const int64_t ngroups = (pt.n + 31) / 32;
  // every warp of the CTA runs the same number of rounds (the scales'
  // block reduction waits for all of them)
  const int64_t rounds = (ngroups + nw - 1) / nw;
  for (int64_t it = 0; it < rounds; ++it) {
    const int64_t g = wid + it * nw;
    if (g >= ngroups) continue;
    const int64_t g0 = g * 32;
    const int cnt = pt.n - g0 < 32 ? (int)(pt.n - g0) : 32;
    const int64_t pm = g0 + lane;
    int stm = kPrepSkip;
    {
      PrepFP64 v;
      v.x = v.y = v.z = v.hsml = v.h_inv = v.knorm = v.area = v.col = v.vol = 0.0;
      v.m_in = v.rho_in = v.wgt = 0.0;
      for (int d = 0; d < 3; ++d) v.lo[d] = v.hi[d] = 0;
      v.scalar_zero = false;
      if (lane < cnt) stm = prep_particle_fp64<DIMS>(pt, A.mp, pm, false, &v);
      qs[warp][lane] = v;
    }
    __syncwarp();
    double gm[4] = {0.0, 0.0, 0.0, 0.0}, dKm = 0.0, dqm[kAdjQ32] = {0.0, 0.0, 0.0, 0.0};
    int mode = 0;  // 1: sums of this lane's particle in sums[warp][lane]; 2: results in gm, dKm, dqm
    for (int j = 0; j < cnt; ++j) {
      if (__shfl_sync(full, stm, j) != kPrepMapped) continue;  // warp-uniform
      const PrepFP64& qj = qs[warp][j];
      if (adj_fp32_sums<DIMS, KERN>(A, g0 + j, qj, lane, &sums[warp][j])) {
        if (lane == j) mode = 1;
      } else {
        double grad[4] = {0.0, 0.0, 0.0, 0.0}, dK = 0.0, dqk[kMaxQ];
        for (int k = 0; k < nq; ++k) dqk[k] = 0.0;
        adj_particle_fp64<DIMS, KERN>(A, g0 + j, qj, lane, grad, dK, dqk, nullptr);
        if (lane == j) {
          for (int t = 0; t < 4; ++t) gm[t] = grad[t];
          dKm = dK;
          for (int k = 0; k < nq; ++k) dqm[k] = dqk[k];
          mode = 2;
        }
      }
    }
    __syncwarp();  // lane 0 stored the sums that their own lanes finish
    if (mode == 1) adj_finish32<DIMS>(A, pm, qs[warp][lane], sums[warp][lane], gm, dKm, dqm);
    if (lane < cnt) {
      float v[kAdjScales];
      write_outputs<DIMS>(A, pm, stm, qs[warp][lane], gm, dKm, dqm, v);
      for (int c = 0; c < kAdjScales; ++c) vm[c] = fmaxf(vm[c], v[c]);
    }
    __syncwarp();  // qs[warp] and sums[warp] are rewritten by the next group
  }
  for (int c = 0; c < kAdjScales; ++c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) vm[c] = fmaxf(vm[c], __shfl_xor_sync(full, vm[c], o));
    if (lane == 0) vmax[warp][c] = vm[c];
  }
  flush_scales(A, vmax);
}

// Second pass (FP32 path): a queued particle keeps its FP32 results when
// each error estimate is within kKeepRel of the larger of the value and
// 1e-3 of the largest value of its kind; otherwise it is redone in FP64.
template <int DIMS, int KERN>
__global__ void __launch_bounds__(256, 2) k_adj_pending(AdjArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const DevParticles& pt = A.pt;
  const int nq = pt.nq;
  const double L = A.mp.L;
  const int64_t np = (int64_t)*A.n_pend;
  float sc[kAdjScales];
  for (int c = 0; c < kAdjScales; ++c) sc[c] = 1e-3f * __uint_as_float(A.scale[c]);
  __shared__ AxisTab tabs[8];
  AxisTab* tab = &tabs[threadIdx.x >> 5];
  for (int64_t i = wid; i < np; i += nw) {
    const AdjPending e = A.pend[i];
    const int64_t p = e.p;
    bool ok = true;
    if (lane == 0) {
      auto pass = [&](float err, double v, float s) { return err <= (float)kKeepRel * fmaxf((float)fabs(v), s); };
      for (int d = 0; d < DIMS; ++d) ok = ok && pass(e.e[d], A.d_pos[p * pt.sp + d * pt.sc], sc[0]);
      ok = ok && pass(e.e[3], A.d_hsml[p], sc[1]);
      // dL/dK's error carried into w, m and rho by their factors
      const double m_in = ld_elem(pt.attr_dtype, pt.mass, p), rho_in = ld_elem(pt.attr_dtype, pt.rho, p);
      const double w_in = ld_elem(pt.attr_dtype, pt.w, p);
      const double LD = DIMS == 2 ? L * L * L : L * L * L * L;
      ok = ok && pass((float)(e.e[4] * fabs(w_in * LD / rho_in)), A.d_mass[p], sc[2]);
      ok = ok && pass((float)(e.e[4] * fabs(w_in * m_in * LD / (rho_in * rho_in))), A.d_rho[p], sc[3]);
      ok = ok && pass((float)(e.e[4] * fabs(m_in * LD / rho_in)), A.d_w[p], sc[4]);
      for (int k = 0; k < nq && k < kAdjQ32; ++k) ok = ok && pass(e.e[5 + k], A.d_q[p * pt.qsp + k * pt.qsk], sc[5]);
    }
    ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
    if (ok) continue;  // warp-uniform
    PrepFP64 q;
    const int state = prep_adj<DIMS>(pt, A.mp, p, lane, &q);
    double grad[4] = {0.0, 0.0, 0.0, 0.0};
    double dK = 0.0, dqk[kMaxQ];
    for (int k = 0; k < nq; ++k) dqk[k] = 0.0;
    if (state == kPrepMapped) adj_particle_fp64<DIMS, KERN>(A, p, q, lane, grad, dK, dqk, tab);
    if (lane == 0) {
      float v[kAdjScales];
      write_outputs<DIMS>(A, p, state, q, grad, dK, dqk, v);
    }
  }
}

template <int DIMS, int KERN>
void launch_adj_shape(const AdjArgs& A, int grid, int grid32, cudaStream_t s) {
  if (A.g32 && A.pt.nq <= kAdjQ32) {  // more quantities: every particle in FP64
    k_adj_particles32<DIMS, KERN><<<grid32, 128, 0, s>>>(A);
    k_adj_pending<DIMS, KERN><<<grid, 256, 0, s>>>(A);
  } else {
    k_adj_particles<DIMS, KERN><<<grid, 256, 0, s>>>(A);
  }
}

template <int DIMS>
void launch_adj_dims(int kernel, const AdjArgs& A, int grid, int grid32, cudaStream_t s) {
  switch (kernel) {
    case 0: launch_adj_shape<DIMS, 0>(A, grid, grid32, s); break;
    case 1: launch_adj_shape<DIMS, 1>(A, grid, grid32, s); break;
    case 2: launch_adj_shape<DIMS, 2>(A, grid, grid32, s); break;
    case 3: launch_adj_shape<DIMS, 3>(A, grid, grid32, s); break;
    default: launch_adj_shape<DIMS, 4>(A, grid, grid32, s); break;
  }
}

}  // namespace

cudaError_t launch_adjoint(int kernel, const DevParticles& pt, const DevMapParams& mp, const double* raw,
                           const double* grad_out, int mode, int reduce, double* gq, double* gw,
                           double* d_pos, double* d_hsml, double* d_mass, double* d_rho, double* d_w,
                           double* d_q, float* g32, void* scratch, int num_sms, cudaStream_t s) {
  const int dims = mp.dims;
  const int64_t P = mp.P;
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  int64_t g1 = (PD + 255) / 256;
  if (g1 > num_sms * 8) g1 = num_sms * 8;
  k_adj_reduce<<<(int)(g1 > 0 ? g1 : 1), 256, 0, s>>>(raw, grad_out, dims, P, pt.nq, mode, reduce, gq, gw,
                                                      g32);
  AdjArgs A;
  A.pt = pt;
  A.mp = mp;
  A.gq = gq;
  A.gw = gw;
  A.g32 = g32;
  A.PD = PD;
  A.d_pos = d_pos;
  A.d_hsml = d_hsml;
  A.d_mass = d_mass;
  A.d_rho = d_rho;
  A.d_w = d_w;
  A.d_q = d_q;
  A.st = nullptr;
  A.scale = nullptr;
  A.n_pend = nullptr;
  A.pend = nullptr;
  if (g32) {  // the second pass's scales, count and queue
    A.scale = (unsigned*)scratch;
    A.n_pend = A.scale + kAdjScales;
    A.pend = (AdjPending*)((char*)scratch + 64);
    cudaMemsetAsync(scratch, 0, 64, s);
  }
  if (pt.n > 0) {
    int64_t grid = (pt.n + 7) / 8;
    if (grid > (int64_t)num_sms * 32) grid = (int64_t)num_sms * 32;
    // FP32 first pass: a warp per 32 particles, four warps per CTA
    int64_t grid32 = (pt.n + 127) / 128;
    if (grid32 > (int64_t)num_sms * 32) grid32 = (int64_t)num_sms * 32;
    if (dims == 2) launch_adj_dims<2>(kernel, A, (int)grid, (int)grid32, s);
    else launch_adj_dims<3>(kernel, A, (int)grid, (int)grid32, s);
  }
  return cudaGetLastError();
}

size_t adjoint_scratch_bytes(int64_t n) { return 64 + (size_t)(n > 0 ? n : 1) * sizeof(AdjPending); }

}  // namespace sphg
