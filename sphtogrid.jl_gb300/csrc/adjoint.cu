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
// including the derivative of the renormalisation S.  All in FP64.
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace sphg {

namespace {

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
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

// dL/d(out) -> dL/dQ_k, dL/dW in raw row order (row = i*P + j or i*P^2 + j*P + k).
__global__ void __launch_bounds__(256) k_adj_reduce(const double* __restrict__ raw, const double* __restrict__ g,
                                                     int dims, int64_t P, int nq, int mode, int reduce,
                                                     double* __restrict__ gq, double* __restrict__ gw) {
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
  }
}

struct AdjArgs {
  DevParticles pt;
  DevMapParams mp;
  const double* gq;  // [nq][PD]
  const double* gw;  // [PD]
  int64_t PD;
  double* d_pos;     // strides of pt.pos
  double *d_hsml, *d_mass, *d_rho, *d_w;
  double* d_q;       // strides of pt.q
  DevStatus* st;
};

template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) k_adj_particles(AdjArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const DevParticles& pt = A.pt;
  const double L = A.mp.L;
  const int64_t P = A.mp.P;
  const int nq = pt.nq;
  for (int64_t p = wid; p < pt.n; p += nw) {
    PrepFP64 q;
    const int state = prep_particle_fp64<DIMS>(pt, A.mp, p, false, &q);
    double grad[4] = {0.0, 0.0, 0.0, 0.0};  // x, y, z, h (pixel units)
    double dK = 0.0, dqk[kMaxQ];
    for (int k = 0; k < nq; ++k) dqk[k] = 0.0;
    if (state == kPrepMapped) {
      const int64_t iMin = q.lo[0], jMin = q.lo[1], kMin = q.lo[2];
      const int64_t ni = q.hi[0] - iMin + 1, nj = q.hi[1] - jMin + 1, nk = q.hi[2] - kMin + 1;
      const int64_t njk = nj * nk, F = ni * njk;
      const double xs[3] = {q.x, q.y, q.z};
      const double h = q.hsml;
      // pass 1: renormalisation sum and branch (as the forward)
      double s_w = 0.0;
      for (int64_t f = lane; f < F; f += 32) {
        const int64_t ia = f / njk, r = f - ia * njk, jb = r / nk, kc = r - jb * nk;
        double u, a;
        cell_fp64<DIMS>(q, iMin + ia, jMin + jb, kMin + kc, &u, &a);
        if (u <= 1.0) s_w += kshape<KERN, double>(u) * a;
      }
      s_w = wsum(s_w);
      const bool fallback = (s_w == 0.0);
      // pass 2: recompute g and its derivatives, gather the image gradients
      double S = 0.0, sgg = 0.0, sgd[4] = {0, 0, 0, 0}, sd[4] = {0, 0, 0, 0}, sq[kMaxQ];
      for (int k = 0; k < nq; ++k) sq[k] = 0.0;
      for (int64_t f = lane; f < F; f += 32) {
        const int64_t ia = f / njk, r = f - ia * njk, jb = r / nk, kc = r - jb * nk;
        const int64_t cell[3] = {iMin + ia, jMin + jb, kMin + kc};
        double dist[3] = {0, 0, 0}, ov[3] = {1, 1, 1}, dox[3] = {0, 0, 0}, doh[3] = {0, 0, 0};
        for (int d = 0; d < DIMS; ++d) {
          cell_axis_fp64(xs[d], h, cell[d], &dist[d], &ov[d]);
          const bool up = xs[d] + h < (double)(cell[d] + 1);  // min() takes x + h
          const bool dn = xs[d] - h > (double)cell[d];        // max() takes x - h
          dox[d] = (up ? 1.0 : 0.0) - (dn ? 1.0 : 0.0);
          doh[d] = (up ? 1.0 : 0.0) + (dn ? 1.0 : 0.0);
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
        const double r2 = dist[0] * dist[0] + dist[1] * dist[1] + dist[2] * dist[2];
        const double rr = sqrt(r2);
        const double u = rr / h;
        double g, dg[4];
        if (fallback) {
          g = A_;
          for (int t = 0; t < 4; ++t) dg[t] = dA[t];
        } else if (u <= 1.0) {
          const double s = kshape<KERN, double>(u), sp = kshape_du<KERN>(u);
          g = s * A_;
          for (int d = 0; d < 3; ++d) {
            const double du = (d < DIMS && rr > 0.0) ? dist[d] / (rr * h) : 0.0;
            dg[d] = sp * du * A_ + s * dA[d];
          }
          dg[3] = sp * (-u / h) * A_ + s * dA[3];
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
          sgd[t] += gam * dg[t];
          sd[t] += dg[t];
        }
      }
      S = wsum(S);
      sgg = wsum(sgg);
      for (int t = 0; t < 4; ++t) {
        sgd[t] = wsum(sgd[t]);
        sd[t] = wsum(sd[t]);
      }
      for (int k = 0; k < nq; ++k) sq[k] = wsum(sq[k]);
      const double K = DIMS == 2 ? q.area * q.wgt * q.col : q.vol * q.wgt * L;
      if (S > 0.0) {
        const double Gam = sgg / S;
        dK = Gam;
        for (int t = 0; t < 4; ++t) grad[t] = K / S * (sgd[t] - Gam * sd[t]);
        for (int k = 0; k < nq; ++k) dqk[k] = K / S * sq[k];
      }
    }
    if (lane == 0) {
      // K = w m L^3 / rho (2D), times L in 3D
      const double LD = DIMS == 2 ? L * L * L : L * L * L * L;
      const double m_in = state == kPrepMapped ? q.m_in : 0.0;
      const double rho_in = state == kPrepMapped ? q.rho_in : 1.0;
      const double w_in = state == kPrepMapped ? q.wgt : 0.0;
      A.d_w[p] = dK * m_in * LD / rho_in;
      A.d_mass[p] = dK * w_in * LD / rho_in;
      A.d_rho[p] = -dK * w_in * m_in * LD / (rho_in * rho_in);
      A.d_hsml[p] = grad[3] * L;
      for (int d = 0; d < 3; ++d) A.d_pos[p * pt.sp + d * pt.sc] = grad[d] * L;
      for (int k = 0; k < nq; ++k) A.d_q[p * pt.qsp + k * pt.qsk] = dqk[k];
    }
  }
}

template <int DIMS>
void launch_adj_dims(int kernel, const AdjArgs& A, int grid, cudaStream_t s) {
  switch (kernel) {
    case 0: k_adj_particles<DIMS, 0><<<grid, 256, 0, s>>>(A); break;
    case 1: k_adj_particles<DIMS, 1><<<grid, 256, 0, s>>>(A); break;
    case 2: k_adj_particles<DIMS, 2><<<grid, 256, 0, s>>>(A); break;
    case 3: k_adj_particles<DIMS, 3><<<grid, 256, 0, s>>>(A); break;
    default: k_adj_particles<DIMS, 4><<<grid, 256, 0, s>>>(A); break;
  }
}

}  // namespace

cudaError_t launch_adjoint(int kernel, const DevParticles& pt, const DevMapParams& mp, const double* raw,
                           const double* grad_out, int mode, int reduce, double* gq, double* gw,
                           double* d_pos, double* d_hsml, double* d_mass, double* d_rho, double* d_w,
                           double* d_q, int num_sms, cudaStream_t s) {
  const int dims = mp.dims;
  const int64_t P = mp.P;
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  int64_t g1 = (PD + 255) / 256;
  if (g1 > num_sms * 8) g1 = num_sms * 8;
  k_adj_reduce<<<(int)(g1 > 0 ? g1 : 1), 256, 0, s>>>(raw, grad_out, dims, P, pt.nq, mode, reduce, gq, gw);
  AdjArgs A;
  A.pt = pt;
  A.mp = mp;
  A.gq = gq;
  A.gw = gw;
  A.PD = PD;
  A.d_pos = d_pos;
  A.d_hsml = d_hsml;
  A.d_mass = d_mass;
  A.d_rho = d_rho;
  A.d_w = d_w;
  A.d_q = d_q;
  A.st = nullptr;
  if (pt.n > 0) {
    int64_t grid = (pt.n + 7) / 8;
    if (grid > (int64_t)num_sms * 32) grid = (int64_t)num_sms * 32;
    if (dims == 2) launch_adj_dims<2>(kernel, A, (int)grid, s);
    else launch_adj_dims<3>(kernel, A, (int)grid, s);
  }
  return cudaGetLastError();
}

}  // namespace sphg
