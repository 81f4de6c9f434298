// healpix.cu -- all-sky HEALPix deposition (SPHtoGrid.jl
// src/healpix_interpolation/main.jl:92-227, pixel_weights.jl,
// constributing_pixels.jl) in FP64, the reference's precision.
//
// One warp per particle.  Its pixels are the HEALPix RING pixels whose
// centres lie within the projected smoothing length asin(hsml / r) of the
// particle's direction (a disc query), plus the pixel containing the
// direction; they are enumerated ring by ring, the lanes striding over each
// ring's pixel range.  Pass 1 sums the renormalisation terms (kernel weight
// times contributing area, areas, pixel counts) over the warp; pass 2
// recomputes each pixel's weight and adds it into the two maps with FP64
// atomics.  The ring geometry (Gorski et al. 2005) is restated from the
// published algorithm, as the oracle restates it.
#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace sphg {
namespace {

constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTwoPi = 6.283185307179586476925286766559005768;

struct HpRing {
  double z;
  int64_t first, nr;
  int shifted;
};

// z, first pixel, pixel count and half-pixel shift of ring ir (1 .. 4 nside - 1).
__device__ __forceinline__ HpRing hp_ring(int64_t nside, int64_t ir) {
  HpRing R;
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  const double fact2 = 4.0 / (double)npix;
  const int64_t nring = ir > 2 * nside ? 4 * nside - ir : ir;
  if (nring < nside) {
    const double tmp = (double)nring * (double)nring * fact2;
    R.z = 1.0 - tmp;
    R.nr = 4 * nring;
    R.shifted = 1;
    R.first = 2 * nring * (nring - 1);
  } else {
    R.z = (double)(2 * nside - nring) * (2.0 / (3.0 * (double)nside));
    R.nr = 4 * nside;
    R.shifted = ((nring - nside) & 1) == 0;
    R.first = ncap + (nring - nside) * R.nr;
  }
  if (nring != ir) {
    R.z = -R.z;
    R.first = npix - R.first - R.nr;
  }
  return R;
}

// Unit vector of the centre of in-ring pixel k of ring R.
__device__ __forceinline__ void hp_centre(const HpRing& R, int64_t k, double v[3]) {
  const double phi = ((double)k + (R.shifted ? 0.5 : 0.0)) * (kTwoPi / (double)R.nr);
  const double sth = sqrt((1.0 - R.z) * (1.0 + R.z));
  v[0] = sth * cos(phi);
  v[1] = sth * sin(phi);
  v[2] = R.z;
}

__device__ __forceinline__ int64_t hp_ang2pix(int64_t nside, double theta, double phi) {
  const double z = cos(theta), za = fabs(z);
  double tt = fmod(phi, kTwoPi);
  if (tt < 0.0) tt += kTwoPi;
  tt *= 2.0 / kPi;
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  if (za <= 2.0 / 3.0) {
    const double t1 = (double)nside * (0.5 + tt), t2 = (double)nside * z * 0.75;
    const int64_t jp = (int64_t)floor(t1 - t2), jm = (int64_t)floor(t1 + t2);
    const int64_t ir = nside + 1 + jp - jm;
    const int64_t kshift = 1 - (ir & 1);
    int64_t ip = (jp + jm - nside + kshift + 1) / 2;
    ip = ((ip % (4 * nside)) + 4 * nside) % (4 * nside);
    return ncap + (ir - 1) * 4 * nside + ip;
  }
  const double tp = tt - floor(tt);
  const double tmp = (double)nside * sqrt(3.0 * (1.0 - za));
  const int64_t jp = (int64_t)floor(tp * tmp), jm = (int64_t)floor((1.0 - tp) * tmp);
  const int64_t ir = jp + jm + 1;
  int64_t ip = (int64_t)floor(tt * (double)ir);
  ip = ((ip % (4 * ir)) + 4 * ir) % (4 * ir);
  return z > 0.0 ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
}

// Ring and in-ring index of pixel p.
__device__ __forceinline__ void hp_pix_ring(int64_t nside, int64_t pix, int64_t* ir, int64_t* ip) {
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  if (pix < ncap) {
    int64_t r = (int64_t)((1.0 + sqrt(1.0 + 2.0 * (double)pix)) * 0.5);
    while (2 * r * (r - 1) > pix) --r;
    while (2 * (r + 1) * r <= pix) ++r;
    *ir = r;
    *ip = pix - 2 * r * (r - 1);
  } else if (pix < npix - ncap) {
    const int64_t q = pix - ncap;
    *ir = q / (4 * nside) + nside;
    *ip = q % (4 * nside);
  } else {
    const int64_t q = npix - 1 - pix;
    int64_t r = (int64_t)((1.0 + sqrt(1.0 + 2.0 * (double)q)) * 0.5);
    while (2 * r * (r - 1) > q) --r;
    while (2 * (r + 1) * r <= q) ++r;
    *ir = 4 * nside - r;
    *ip = 4 * r - 1 - (q - 2 * r * (r - 1));
  }
}

__device__ __forceinline__ int64_t hp_ring_above(int64_t nside, double z) {
  const double az = fabs(z);
  if (az <= 2.0 / 3.0) return (int64_t)((double)nside * (2.0 - 1.5 * z));
  const int64_t ir = (int64_t)((double)nside * sqrt(3.0 * (1.0 - az)));
  return z > 0.0 ? ir : 4 * nside - ir - 1;
}

// The disc of one particle: rings irmin .. irmax with in-ring ranges
// [lo, hi] (wrapping modulo the ring size); with a pole inside the disc, the
// rings beyond irmin (north) or irmax (south) are entire.
struct HpDisc {
  double phi, z0, xa, cosrad;
  int64_t irmin, irmax, nrings;
  bool north, south;
};

__device__ __forceinline__ HpDisc hp_disc(int64_t nside, double theta, double phi, double radius) {
  HpDisc D;
  D.phi = phi;
  D.cosrad = cos(radius);
  D.z0 = cos(theta);
  D.xa = 1.0 / sqrt((1.0 - D.z0) * (1.0 + D.z0));
  D.nrings = 4 * nside - 1;
  const double rlat1 = theta - radius, rlat2 = theta + radius;
  D.irmin = hp_ring_above(nside, cos(rlat1)) + 1;
  D.irmax = hp_ring_above(nside, cos(rlat2));
  D.north = rlat1 <= 0.0;
  D.south = rlat2 >= kPi;
  return D;
}

// In-ring pixel range of ring ir within the disc: [lo, hi] (hi < lo: none).
__device__ __forceinline__ void hp_ring_range(const HpDisc& D, const HpRing& R, int64_t ir, int64_t* lo,
                                              int64_t* hi) {
  if ((D.north && ir < D.irmin) || (D.south && ir > D.irmax)) {
    *lo = 0;
    *hi = R.nr - 1;
    return;
  }
  if (ir < D.irmin || ir > D.irmax) {
    *lo = 1;
    *hi = 0;
    return;
  }
  const double x = (D.cosrad - R.z * D.z0) * D.xa, ysq = 1.0 - R.z * R.z - x * x;
  const double dphi = ysq <= 0.0 ? (x > 0.0 ? kPi : 0.0) : atan2(sqrt(ysq), x);
  const double shift = R.shifted ? 0.5 : 0.0;
  // the range in FP64 first: a whole ring when it spans the ring (or is
  // not finite), so the integer range never exceeds the ring's pixels
  const double fa = floor((double)R.nr / kTwoPi * (D.phi - dphi) - shift);
  const double fb = floor((double)R.nr / kTwoPi * (D.phi + dphi) - shift);
  if (!(fb - fa < (double)R.nr)) {
    *lo = 0;
    *hi = R.nr - 1;
    return;
  }
  *lo = (int64_t)fa + 1;
  *hi = (int64_t)fb;
}

struct HpParticle {
  double p[3], dx, dxinv, proj, hinv, area_norm, q, scale;  // scale: (ang_pix dx)^-2
  int fallback;
};

// Kernel weight and contributing area of the pixel centred at `pc`.
// Angular distance of the pixel centred at `pc` from the particle's
// direction: d / |p| as a product with the reciprocal (within an ulp of the
// quotient; where acos amplifies that, u is near 0 and the kernel flat).
__device__ __forceinline__ double hp_ddx(const HpParticle& P, const double pc[3]) {
  double d = 0.0;
  for (int c = 0; c < 3; ++c) d += P.p[c] * pc[c];
  return acos(fmin(d * P.dxinv, 1.0));
}

// Kernel weight and contributing area of a pixel at angular distance ddx.
__device__ __forceinline__ void hp_terms(int KERN_RT, int kdim, const HpParticle& P, double ddx, double ang_pix,
                                         double* wk, double* a, bool* inside) {
  const double u = ddx * P.hinv;
  *a = fmax(0.0, fmin(ang_pix, fabs(P.proj - (ddx - 0.5 * ang_pix)))) / ang_pix * P.scale;
  *inside = u <= 1.0;
  double w = 0.0;
  if (*inside) {
    const double hd = kdim == 2 ? P.hinv * P.hinv : P.hinv * P.hinv * P.hinv;
    const double nrm = kernel_sigma(KERN_RT, kdim) * hd;
    double s;
    switch (KERN_RT) {
      case 0: s = kshape<0, double>(u); break;
      case 1: s = kshape<1, double>(u); break;
      case 2: s = kshape<2, double>(u); break;
      case 3: s = kshape<3, double>(u); break;
      default: s = kshape<4, double>(u); break;
    }
    w = s * nrm;
  }
  *wk = w;
}

struct HpArgs {
  int64_t nside, n;
  int kernel, kdim, calc_mean, dtype;
  const void *pos, *hsml, *m, *rho, *q, *w;  // pos: 3 per particle
  double *allsky, *weight;
  const double* centres;  // pixel-centre unit vectors (3 per pixel), or NULL
  double* dist;           // per warp: pass 1's angular distances for pass 2, or NULL
  int dist_per_lane;      // distances kept per lane (the rest are recomputed)
  DevStatus* st;
};

// Centre of in-ring pixel kk of ring R: from the precomputed table (the same
// arithmetic, once per pixel instead of twice per particle and pixel).
__device__ __forceinline__ void pixel_centre(const HpArgs& H, const HpRing& R, int64_t kk, double pc[3]) {
  if (H.centres) {
    const double* c = H.centres + 3 * (R.first + kk);
    pc[0] = c[0];
    pc[1] = c[1];
    pc[2] = c[2];
  } else {
    hp_centre(R, kk, pc);
  }
}

// The table of pixel centres (RING order).
__global__ void __launch_bounds__(256) k_hp_centres(int64_t nside, double* centres) {
  const int64_t npix = 12 * nside * nside;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += (int64_t)gridDim.x * blockDim.x) {
    int64_t ir, ip;
    hp_pix_ring(nside, p, &ir, &ip);
    double v[3];
    hp_centre(hp_ring(nside, ir), ip, v);
    centres[3 * p] = v[0];
    centres[3 * p + 1] = v[1];
    centres[3 * p + 2] = v[2];
  }
}

// In-ring index of k, which lies within one ring size of [0, nr) (a disc's
// in-ring range): one add or subtract instead of a 64-bit modulo.
__device__ __forceinline__ int64_t ring_wrap(int64_t k, int64_t nr) {
  if (k < 0) k += nr;
  else if (k >= nr) k -= nr;
  return (k >= 0 && k < nr) ? k : ((k % nr) + nr) % nr;
}

// Calls f(R, kk) for the disc's pixels on rings r0..r1, ring by ring, the
// lanes striding over each ring's range (the same pixels in the same order
// on every call).  The rings' geometry and ranges are computed 32 at a
// time, one ring per lane, and broadcast.
template <class F>
__device__ __forceinline__ void for_disc_pixels(const HpArgs& H, const HpDisc& D, int64_t r0, int64_t r1, int lane,
                                                F&& f) {
  const unsigned full = 0xffffffffu;
  for (int64_t rb = r0; rb <= r1; rb += 32) {
    HpRing mine = {0.0, 0, 1, 0};
    int64_t lo = 1, hi = 0;
    if (rb + lane <= r1) {
      mine = hp_ring(H.nside, rb + lane);
      hp_ring_range(D, mine, rb + lane, &lo, &hi);
    }
    const int nrb = r1 - rb + 1 < 32 ? (int)(r1 - rb + 1) : 32;
    for (int q = 0; q < nrb; ++q) {
      HpRing R;
      R.z = __shfl_sync(full, mine.z, q);
      R.first = __shfl_sync(full, mine.first, q);
      R.nr = __shfl_sync(full, mine.nr, q);
      R.shifted = __shfl_sync(full, mine.shifted, q);
      const int64_t rlo = __shfl_sync(full, lo, q), rhi = __shfl_sync(full, hi, q);
      for (int64_t k = rlo + lane; k <= rhi; k += 32) f(R, ring_wrap(k, R.nr));
    }
  }
}

// One warp per particle: pass 1 (sums), pass 2 (deposit).
__global__ void __launch_bounds__(256) k_healpix(HpArgs H) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t npix = 12 * H.nside * H.nside;
  const double ang_pix = sqrt(4.0 * kPi / (double)npix);
  double c_gm = 0.0, c_pm = 0.0;
  unsigned long long c_map = 0, c_dep = 0;
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < H.n; i += nw) {
    HpParticle P;
    for (int c = 0; c < 3; ++c) P.p[c] = ld_elem(H.dtype, H.pos, 3 * i + c);
    const double h = ld_elem(H.dtype, H.hsml, i);
    P.q = ld_elem(H.dtype, H.q, i);
    if (!H.calc_mean && P.q == 0.0) continue;
    double dx = 0.0;
    for (int c = 0; c < 3; ++c) dx += P.p[c] * P.p[c];
    dx = sqrt(dx);
    if (dx < h) continue;
    P.dx = dx;
    P.dxinv = 1.0 / dx;
    P.proj = asin(h / dx);
    P.hinv = 1.0 / P.proj;
    P.scale = 1.0 / ((ang_pix * dx) * (ang_pix * dx));
    double theta = atan2(sqrt(P.p[0] * P.p[0] + P.p[1] * P.p[1]), P.p[2]);
    double phi = atan2(P.p[1], P.p[0]);
    if (phi < 0.0) phi += kTwoPi;
    if (!(isfinite(P.proj) && isfinite(theta) && isfinite(phi) && isfinite(P.q))) {
      if (lane == 0) atomicOr(&H.st->flags, kFlagNonFinite);
      continue;
    }
    const HpDisc D = hp_disc(H.nside, theta, phi, P.proj);
    // the pixel holding the direction joins when the disc misses it
    const int64_t cpix = hp_ang2pix(H.nside, theta, phi);
    int64_t cir, cip;
    hp_pix_ring(H.nside, cpix, &cir, &cip);
    bool c_in;
    {
      const HpRing R = hp_ring(H.nside, cir);
      int64_t lo, hi;
      hp_ring_range(D, R, cir, &lo, &hi);
      const int64_t off = (((cip - lo) % R.nr) + R.nr) % R.nr;  // cip - lo modulo the ring
      c_in = hi >= lo && (hi - lo + 1 >= R.nr || off <= hi - lo);
    }
    // rings that can hold disc pixels
    const int64_t r0 = D.north ? 1 : (D.irmin > 1 ? D.irmin : 1);
    const int64_t r1 = D.south ? D.nrings : (D.irmax < D.nrings ? D.irmax : D.nrings);
    // pass 1 (the lane's j-th pixel keeps its distance at dist[j * 32 + lane]
    // of the warp's slice, for pass 2)
    double* dist = H.dist ? H.dist + ((((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * H.dist_per_lane) * 32
                          : nullptr;
    double dw = 0.0, da = 0.0, swk = 0.0;
    long long nd = 0, nt = 0;
    int j = 0;
    for_disc_pixels(H, D, r0, r1, lane, [&](const HpRing& R, int64_t kk) {
      double pc[3], wk, a;
      bool in;
      pixel_centre(H, R, kk, pc);
      const double ddx = hp_ddx(P, pc);
      if (dist && j < H.dist_per_lane) dist[(int64_t)j * 32 + lane] = ddx;
      ++j;
      hp_terms(H.kernel, H.kdim, P, ddx, ang_pix, &wk, &a, &in);
      da += a;
      nt += 1;
      if (in) {
        dw += wk * a;
        nd += 1;
        swk += wk;
      }
    });
    if (!c_in && lane == 0) {
      double pc[3], wk, a;
      bool in;
      hp_centre(hp_ring(H.nside, cir), cip, pc);
      hp_terms(H.kernel, H.kdim, P, hp_ddx(P, pc), ang_pix, &wk, &a, &in);
      da += a;
      nt += 1;
      if (in) {
        dw += wk * a;
        nd += 1;
        swk += wk;
      }
    }
    dw = warp_sum_d(dw);
    da = warp_sum_d(da);
    swk = warp_sum_d(swk);
    nd = warp_sum_ll(nd);
    nt = warp_sum_ll(nt);
    // calculate_weights' factors and update_image!'s normalisation
    P.fallback = dw == 0.0;
    double wpp;
    if (P.fallback) {
      nd = nt;
      wpp = da != 0.0 ? (double)nd / da : 1.0;
      swk = (double)nt;
    } else {
      wpp = (double)nd / dw;
    }
    const double m = ld_elem(H.dtype, H.m, i), rho = ld_elem(H.dtype, H.rho, i);
    double dz = 2.0 * h;
    const double area = (m / rho) / dz;
    dz /= (ang_pix * dx) * (ang_pix * dx);
    P.area_norm = area / (double)nd * wpp * ld_elem(H.dtype, H.w, i) * dz;
    // pass 2: the same pixels in the same order
    double sa = 0.0;
    j = 0;
    for_disc_pixels(H, D, r0, r1, lane, [&](const HpRing& R, int64_t kk) {
      double wk, a;
      bool in;
      double ddx;
      if (dist && j < H.dist_per_lane) {
        ddx = dist[(int64_t)j * 32 + lane];
      } else {
        double pc[3];
        pixel_centre(H, R, kk, pc);
        ddx = hp_ddx(P, pc);
      }
      ++j;
      hp_terms(H.kernel, H.kdim, P, ddx, ang_pix, &wk, &a, &in);
      if (P.fallback) wk = 1.0;
      const double pw = P.area_norm * wk * a;
      atomicAdd(&H.allsky[R.first + kk], P.q * pw);
      atomicAdd(&H.weight[R.first + kk], pw);
      sa += a;
    });
    if (!c_in && lane == 0) {
      double pc[3], wk, a;
      bool in;
      const HpRing R = hp_ring(H.nside, cir);
      hp_centre(R, cip, pc);
      hp_terms(H.kernel, H.kdim, P, hp_ddx(P, pc), ang_pix, &wk, &a, &in);
      if (P.fallback) wk = 1.0;
      const double pw = P.area_norm * wk * a;
      atomicAdd(&H.allsky[cpix], P.q * pw);
      atomicAdd(&H.weight[cpix], pw);
      sa += a;
    }
    sa = warp_sum_d(sa);
    if (lane == 0) {
      c_gm += rho * swk * sa * dz * ((ang_pix * dx) * (ang_pix * dx));
      c_pm += m;
      c_map += 1;
      c_dep += (unsigned long long)nt;
    }
  }
  if (lane == 0 && c_map) {
    atomicAdd(&H.st->grid_mass, c_gm);
    atomicAdd(&H.st->particle_mass, c_pm);
    atomicAdd(&H.st->n_mapped, c_map);
    atomicAdd(&H.st->deposits, c_dep);
  }
}

}  // namespace

void launch_healpix(int64_t nside, int kernel, int kdim, int calc_mean, int dtype, int64_t n, const void* pos,
                    const void* hsml, const void* m, const void* rho, const void* q, const void* w,
                    double* allsky, double* weight, double* centres, bool fill_centres, double* dist,
                    int dist_per_lane, DevStatus* st, int num_sms, cudaStream_t s) {
  HpArgs H;
  H.nside = nside;
  H.n = n;
  H.kernel = kernel;
  H.kdim = kdim;
  H.calc_mean = calc_mean;
  H.dtype = dtype;
  H.pos = pos;
  H.hsml = hsml;
  H.m = m;
  H.rho = rho;
  H.q = q;
  H.w = w;
  H.allsky = allsky;
  H.weight = weight;
  H.centres = centres;
  H.dist = dist;
  H.dist_per_lane = dist ? dist_per_lane : 0;
  H.st = st;
  if (centres && fill_centres) k_hp_centres<<<num_sms * 16, 256, 0, s>>>(nside, centres);
  int64_t grid = (n * 32 + 255) / 256;
  if (grid > (int64_t)num_sms * kHpCtasPerSm) grid = (int64_t)num_sms * kHpCtasPerSm;
  if (grid < 1) grid = 1;
  k_healpix<<<(unsigned)grid, 256, 0, s>>>(H);
}

}  // namespace sphg
