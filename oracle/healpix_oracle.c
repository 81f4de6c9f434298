/* healpix_oracle.c -- TEST INFRASTRUCTURE ONLY: a CPU restatement of
 * SPHtoGrid.jl's all-sky HEALPix deposition (src/healpix_interpolation/
 * main.jl:92-227, pixel_weights.jl:1-139, constributing_pixels.jl:1-22,
 * filter_particles.jl:1-53, shared.jl:1-10), the oracle of the GPU path.
 *
 * The pixel geometry comes from Healpix.jl (not vendored here): the ring
 * scheme of Gorski et al. 2005 (ApJ 622, 759) -- pix2vec, ang2pix, vec2ang and
 * the non-inclusive disc query (pixels whose centres lie within the radius),
 * restated from the published algorithm.  PARITY UNPINNED: no reference
 * output exists here; the pixel functions are checked against the paper's
 * known pixel centres and the disc query against a brute-force search.
 *
 * Compiled with -ffp-contract=off (no FMA contraction).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define HP_PI 3.141592653589793238462643383279502884
#define HP_TWOPI 6.283185307179586476925286766559005768

/* --------------------------------------------------------- ring geometry */

/* z = cos(theta) of ring `ir` (1 .. 4 nside - 1), its first pixel, its pixel
 * count and whether its pixel centres are shifted by half a pixel. */
void hp_ring_info(int64_t nside, int64_t ir, double* z, int64_t* first, int64_t* npix_ring, int* shifted) {
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  const double fact2 = 4.0 / (double)npix;
  const int64_t northring = ir > 2 * nside ? 4 * nside - ir : ir;
  if (northring < nside) {  /* polar cap */
    const double tmp = (double)northring * (double)northring * fact2;
    *z = 1.0 - tmp;
    *npix_ring = 4 * northring;
    *shifted = 1;
    *first = 2 * northring * (northring - 1);
  } else {  /* equatorial belt */
    *z = (double)(2 * nside - northring) * (2.0 / (3.0 * (double)nside));
    *npix_ring = 4 * nside;
    *shifted = ((northring - nside) & 1) == 0;
    *first = ncap + (northring - nside) * *npix_ring;
  }
  if (northring != ir) {  /* southern hemisphere */
    *z = -*z;
    *first = npix - *first - *npix_ring;
  }
}

/* Ring index (1-based) and in-ring index of pixel `pix`. */
static void hp_pix_ring(int64_t nside, int64_t pix, int64_t* ir, int64_t* ip) {
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

/* Unit vector of the centre of pixel `pix` (RING ordering). */
void hp_pix2vec_ring(int64_t nside, int64_t pix, double v[3]) {
  int64_t ir, ip, first, nr;
  int shifted;
  double z;
  hp_pix_ring(nside, pix, &ir, &ip);
  hp_ring_info(nside, ir, &z, &first, &nr, &shifted);
  const double phi = ((double)ip + (shifted ? 0.5 : 0.0)) * (HP_TWOPI / (double)nr);
  const double sth = sqrt((1.0 - z) * (1.0 + z));
  v[0] = sth * cos(phi);
  v[1] = sth * sin(phi);
  v[2] = z;
}

/* (theta, phi) of a vector: colatitude in [0, pi], longitude in [0, 2 pi). */
void hp_vec2ang(double x, double y, double z, double* theta, double* phi) {
  *theta = atan2(sqrt(x * x + y * y), z);
  double p = atan2(y, x);
  if (p < 0.0) p += HP_TWOPI;
  *phi = p;
}

/* Pixel (RING ordering) containing the direction (theta, phi). */
int64_t hp_ang2pix_ring(int64_t nside, double theta, double phi) {
  const double z = cos(theta), za = fabs(z);
  double tt = fmod(phi, HP_TWOPI);
  if (tt < 0.0) tt += HP_TWOPI;
  tt *= 2.0 / HP_PI; /* in [0, 4) */
  const int64_t ncap = 2 * nside * (nside - 1), npix = 12 * nside * nside;
  if (za <= 2.0 / 3.0) { /* equatorial belt */
    const double t1 = (double)nside * (0.5 + tt), t2 = (double)nside * z * 0.75;
    const int64_t jp = (int64_t)floor(t1 - t2), jm = (int64_t)floor(t1 + t2);
    const int64_t ir = nside + 1 + jp - jm; /* 1 .. 2 nside + 1 */
    const int64_t kshift = 1 - (ir & 1);
    int64_t ip = (jp + jm - nside + kshift + 1) / 2;
    ip = ((ip % (4 * nside)) + 4 * nside) % (4 * nside);
    return ncap + (ir - 1) * 4 * nside + ip;
  }
  const double tp = tt - floor(tt);
  const double tmp = (double)nside * sqrt(3.0 * (1.0 - za));
  const int64_t jp = (int64_t)floor(tp * tmp), jm = (int64_t)floor((1.0 - tp) * tmp);
  const int64_t ir = jp + jm + 1; /* ring from the nearest pole */
  int64_t ip = (int64_t)floor(tt * (double)ir);
  ip = ((ip % (4 * ir)) + 4 * ir) % (4 * ir);
  return z > 0.0 ? 2 * ir * (ir - 1) + ip : npix - 2 * ir * (ir + 1) + ip;
}

/* Ring whose z is the nearest at or above `z` (0: above the first ring). */
static int64_t hp_ring_above(int64_t nside, double z) {
  const double az = fabs(z);
  if (az <= 2.0 / 3.0) return (int64_t)((double)nside * (2.0 - 1.5 * z));
  const int64_t ir = (int64_t)((double)nside * sqrt(3.0 * (1.0 - az)));
  return z > 0.0 ? ir : 4 * nside - ir - 1;
}

/* Pixels (RING ordering) whose centres lie within `radius` of
 * (theta, phi), ring by ring; returns the count (at most `cap` written). */
int64_t hp_query_disc_ring(int64_t nside, double theta, double phi, double radius, int64_t* out, int64_t cap) {
  int64_t n = 0;
#define HP_PUSH(p)            \
  do {                        \
    if (n < cap) out[n] = (p); \
    ++n;                      \
  } while (0)
  const int64_t npix = 12 * nside * nside, nrings = 4 * nside - 1;
  if (radius >= HP_PI) {
    for (int64_t p = 0; p < npix; ++p) HP_PUSH(p);
    return n;
  }
  const double cosrad = cos(radius), z0 = cos(theta);
  const double xa = 1.0 / sqrt((1.0 - z0) * (1.0 + z0));
  const double rlat1 = theta - radius, zmax = cos(rlat1);
  int64_t irmin = hp_ring_above(nside, zmax) + 1;
  if (rlat1 <= 0.0) { /* the north pole is inside: every ring above irmin entirely */
    for (int64_t ir = 1; ir < irmin; ++ir) {
      double z;
      int64_t first, nr;
      int sh;
      hp_ring_info(nside, ir, &z, &first, &nr, &sh);
      for (int64_t k = 0; k < nr; ++k) HP_PUSH(first + k);
    }
  }
  const double rlat2 = theta + radius, zmin = cos(rlat2);
  int64_t irmax = hp_ring_above(nside, zmin);
  for (int64_t ir = irmin; ir <= irmax && ir <= nrings; ++ir) {
    if (ir < 1) continue;
    double z;
    int64_t first, nr;
    int sh;
    hp_ring_info(nside, ir, &z, &first, &nr, &sh);
    const double x = (cosrad - z * z0) * xa, ysq = 1.0 - z * z - x * x;
    const double dphi = ysq <= 0.0 ? (x > 0.0 ? HP_PI : 0.0) : atan2(sqrt(ysq), x);
    if (dphi <= 0.0 && ysq <= 0.0 && x <= 0.0) continue;
    const double shift = sh ? 0.5 : 0.0;
    const double fa = floor((double)nr / HP_TWOPI * (phi - dphi) - shift);
    const double fb = floor((double)nr / HP_TWOPI * (phi + dphi) - shift);
    int64_t lo = 0, hi = nr - 1; /* a whole ring when the range spans it */
    if (fb - fa < (double)nr) {
      lo = (int64_t)fa + 1;
      hi = (int64_t)fb;
    }
    for (int64_t k = lo; k <= hi; ++k) HP_PUSH(first + ((k % nr) + nr) % nr);
  }
  if (rlat2 >= HP_PI) { /* the south pole is inside */
    for (int64_t ir = irmax + 1; ir <= nrings; ++ir) {
      double z;
      int64_t first, nr;
      int sh;
      hp_ring_info(nside, ir, &z, &first, &nr, &sh);
      for (int64_t k = 0; k < nr; ++k) HP_PUSH(first + k);
    }
  }
#undef HP_PUSH
  return n;
}

/* --------------------------------------------------------- the deposition */

double orc_kernel_value(int kernel, int kdim, double u, double h_inv); /* sph_oracle.c */

/* healpix_map's particle loop (main.jl:129-204) over particles already
 * centred, selected and ordered as filter_sort_particles leaves them.  Adds
 * into `allsky` and `weight` (12 nside^2 each, RING ordering); returns the
 * number of particles mapped, or -1 when a pixel list exceeds the scratch. */
int64_t orc_healpix_map(int64_t nside, int kernel, int kdim, int calc_mean, int64_t n, const double* pos,
                        const double* hsml, const double* m, const double* rho, const double* q,
                        const double* w, double* allsky, double* weight, double* grid_mass,
                        double* part_mass) {
  const int64_t npix = 12 * nside * nside;
  const double ang_pix = sqrt(4.0 * HP_PI / (double)npix);
  int64_t cap = 1 << 16;
  int64_t* idx = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
  double* wk = (double*)malloc((size_t)cap * sizeof(double));
  double* A = (double*)malloc((size_t)cap * sizeof(double));
  int64_t mapped = 0;
  double gm = 0.0, pm = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double* p = pos + 3 * i;
    if (!calc_mean && q[i] == 0.0) continue;
    double dx = 0.0;
    for (int d = 0; d < 3; ++d) dx += p[d] * p[d];
    dx = sqrt(dx);
    if (dx < hsml[i]) continue;
    const double proj = asin(hsml[i] / dx);
    double theta, phi;
    hp_vec2ang(p[0], p[1], p[2], &theta, &phi);
    if (!(isfinite(proj) && isfinite(theta) && isfinite(phi) && isfinite(q[i]))) continue;
    int64_t np = hp_query_disc_ring(nside, theta, phi, proj, idx, cap);
    while (np + 1 > cap) { /* grow the scratch and query again */
      cap = 2 * (np + 1);
      idx = (int64_t*)realloc(idx, (size_t)cap * sizeof(int64_t));
      wk = (double*)realloc(wk, (size_t)cap * sizeof(double));
      A = (double*)realloc(A, (size_t)cap * sizeof(double));
      np = hp_query_disc_ring(nside, theta, phi, proj, idx, cap);
    }
    /* push! the pixel holding the centre, then unique! (first occurrence kept) */
    const int64_t cpix = hp_ang2pix_ring(nside, theta, phi);
    int found = 0;
    for (int64_t k = 0; k < np; ++k)
      if (idx[k] == cpix) found = 1;
    if (!found) idx[np++] = cpix;
    /* particle_area_and_depth (main.jl:57-64) and the projection correction */
    double dz = 2.0 * hsml[i];
    const double area = (m[i] / rho[i]) / dz;
    dz /= (ang_pix * dx) * (ang_pix * dx);
    /* calculate_weights (pixel_weights.jl:93-139) */
    const double hinv = 1.0 / proj;
    int64_t n_distr = 0, n_tot = 0;
    double dw = 0.0, da = 0.0;
    for (int64_t k = 0; k < np; ++k) {
      double pc[3];
      hp_pix2vec_ring(nside, idx[k], pc);
      double d = 0.0;
      for (int c = 0; c < 3; ++c) d += p[c] * pc[c];
      const double ddx = acos(fmin(d / dx, 1.0)); /* distance_to_pixel_center */
      const double u = ddx * hinv;
      double a = fmax(0.0, fmin(ang_pix, fabs(proj - (ddx - 0.5 * ang_pix)))) / ang_pix;
      a /= (ang_pix * dx) * (ang_pix * dx);
      A[k] = a;
      da += a;
      n_tot += 1;
      if (u <= 1.0) {
        wk[k] = orc_kernel_value(kernel, kdim, u, hinv);
        dw += wk[k] * a;
        n_distr += 1;
      } else {
        wk[k] = 0.0;
      }
    }
    double wpp;
    if (dw == 0.0) {
      n_distr = n_tot;
      for (int64_t k = 0; k < np; ++k) wk[k] = 1.0;
      wpp = da != 0.0 ? (double)n_distr / da : 1.0;
    } else {
      wpp = (double)n_distr / dw;
    }
    /* update_image! (main.jl:27-46) */
    const double kernel_norm = area / (double)n_distr;
    const double area_norm = kernel_norm * wpp * w[i] * dz;
    double swk = 0.0, sa = 0.0;
    for (int64_t k = 0; k < np; ++k) {
      const double pw = area_norm * wk[k] * A[k];
      allsky[idx[k]] += q[i] * pw;
      weight[idx[k]] += pw;
      swk += wk[k];
      sa += A[k];
    }
    gm += rho[i] * swk * sa * dz * ((ang_pix * dx) * (ang_pix * dx));
    pm += m[i];
    mapped += 1;
  }
  free(idx);
  free(wk);
  free(A);
  if (grid_mass) *grid_mass = gm;
  if (part_mass) *part_mass = pm;
  return mapped;
}
