/*
 * sph_oracle.c -- FP64 CPU restatement of SPHtoGrid.jl's `sphMapping` CIC
 * deposition path (2D projection and 3D gridding with Dolag-style area /
 * volume renormalisation).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: the pytest suite,
 * `__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py` load it as
 * the oracle.  No product code path links, loads or calls it.
 *
 * Parity status: the rules restated here are pinned by the reference's own
 * self-contained tests (parameter errors, filter / shift, index bijection,
 * 2D fallback volume conservation and 3D mass conservation; see
 * tests/test_oracle_kat.py).  The kernel SHAPES come from the un-vendored
 * SPHKernels.jl package (compat "2", Project.toml:27,53) and are restated from
 * the published mathematics (cubic / quintic B-splines, Wendland C4/C6/C8);
 * the per-particle renormalisation cancels the kernel normalisation, so only
 * the shape enters the images.  The reference's only golden images
 * (test/sedov_*_reference.fits) need the downloaded `snap_sedov` input, which
 * is absent, so kernel-shape values are PARITY UNPINNED.
 *
 * Citations are to files of the reference project (SPHtoGrid.jl v0.5.3).
 * Every floating-point expression keeps the operation order of the reference
 * (compile with -ffp-contract=off) so that a second restatement in plain
 * Python reproduces this one bit for bit.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_F32 0
#define ORC_F64 1

enum { K_CUBIC = 0, K_QUINTIC = 1, K_WC4 = 2, K_WC6 = 3, K_WC8 = 4 };

enum {
  ORC_OK = 0,
  ORC_ERR_CENTER_EXTENT = 1, /* parameters.jl:67 */
  ORC_ERR_PIXELS = 2,        /* parameters.jl:98 */
  ORC_ERR_DIMS = 3,          /* sphMapping returns `nothing`: cic_interpolation.jl:148,217 */
  ORC_ERR_NONFINITE = 4,     /* floor(Integer, NaN) throws: cic_shared.jl:46-52 */
  ORC_ERR_NQ = 5,            /* 3D maps one scalar quantity: cic_3D.jl:140 */
  ORC_ERR_ALLOC = 6,
  ORC_ERR_ARG = 7
};

/* Same field order and meaning as `mappingParameters` (parameters.jl:14-27). */
typedef struct {
  double x_lim[2], y_lim[2], z_lim[2];
  double center[3];
  double halfsize[3];
  double len2pix;
  double pixelSideLength;
  int64_t Npixels[3];
  double boxsize;
  int32_t periodic;
  int32_t pad_;
} orc_params;

/* ------------------------------------------------------------------ params */

/* Constructor of mappingParameters, parameters.jl:44-125.  Sentinel values
 * (-1 for limits/centre/sizes/pixelSideLength/boxsize, 0 for Npixels) mean
 * "not given", exactly as the keyword defaults of the reference. */
int orc_mapping_parameters(const double *x_lim_in, const double *y_lim_in,
                           const double *z_lim_in, const double *center_in,
                           double x_size, double y_size, double z_size,
                           double pixelSideLength, int64_t Npixels,
                           double boxsize, orc_params *out) {
  double x_lim[2] = {x_lim_in[0], x_lim_in[1]};
  double y_lim[2] = {y_lim_in[0], y_lim_in[1]};
  double z_lim[2] = {z_lim_in[0], z_lim_in[1]};
  double center[3] = {center_in[0], center_in[1], center_in[2]};
  int xl_def = (x_lim[0] == -1.0 && x_lim[1] == -1.0);
  int yl_def = (y_lim[0] == -1.0 && y_lim[1] == -1.0);
  int zl_def = (z_lim[0] == -1.0 && z_lim[1] == -1.0);
  int c_def = (center[0] == -1.0 && center[1] == -1.0 && center[2] == -1.0);
  /* parameters.jl:58-69 */
  if (xl_def && (yl_def && zl_def)) {
    if (!c_def && (x_size != -1.0 && (y_size != -1.0 && z_size != -1.0))) {
      x_lim[0] = center[0] - 0.5 * x_size;
      x_lim[1] = center[0] + 0.5 * x_size;
      y_lim[0] = center[1] - 0.5 * y_size;
      y_lim[1] = center[1] + 0.5 * y_size;
      z_lim[0] = center[2] - 0.5 * z_size;
      z_lim[1] = center[2] + 0.5 * z_size;
    } else {
      return ORC_ERR_CENTER_EXTENT;
    }
  }
  /* parameters.jl:72-80 */
  if (x_size == -1.0) x_size = x_lim[1] - x_lim[0];
  if (y_size == -1.0) y_size = y_lim[1] - y_lim[0];
  if (z_size == -1.0) z_size = z_lim[1] - z_lim[0];
  /* parameters.jl:82-86 */
  if (c_def) {
    center[0] = x_lim[0] + 0.5 * x_size;
    center[1] = y_lim[0] + 0.5 * y_size;
    center[2] = z_lim[0] + 0.5 * z_size;
  }
  /* parameters.jl:89-99: Julia's max(a, b) for floats */
  double max_size = (x_size > y_size || isnan(x_size)) ? x_size : y_size;
  if (isnan(y_size)) max_size = y_size;
  if ((pixelSideLength == -1.0) && (Npixels != 0)) {
    pixelSideLength = max_size / (double)Npixels;
  } else if ((pixelSideLength != -1.0) && (Npixels == 0)) {
    Npixels = (int64_t)floor(max_size / pixelSideLength);
    pixelSideLength = max_size / (double)Npixels;
  } else {
    return ORC_ERR_PIXELS;
  }
  memset(out, 0, sizeof(*out));
  memcpy(out->x_lim, x_lim, sizeof(x_lim));
  memcpy(out->y_lim, y_lim, sizeof(y_lim));
  memcpy(out->z_lim, z_lim, sizeof(z_lim));
  memcpy(out->center, center, sizeof(center));
  out->halfsize[0] = 0.5 * x_size; /* parameters.jl:113 */
  out->halfsize[1] = 0.5 * y_size;
  out->halfsize[2] = 0.5 * z_size;
  out->len2pix = 1.0 / pixelSideLength; /* parameters.jl:115 */
  out->pixelSideLength = pixelSideLength;
  out->Npixels[0] = out->Npixels[1] = out->Npixels[2] = Npixels; /* :105 */
  out->boxsize = boxsize;
  out->periodic = (boxsize != -1.0); /* parameters.jl:107-111 */
  return ORC_OK;
}

/* ------------------------------------------------------- element accessors */

static inline double ld(int dtype, const void *p, int64_t i) {
  return dtype == ORC_F32 ? (double)((const float *)p)[i] : ((const double *)p)[i];
}
static inline void st(int dtype, void *p, int64_t i, double v) {
  if (dtype == ORC_F32)
    ((float *)p)[i] = (float)v; /* Julia convert(Float32, ::Float64): round to nearest */
  else
    ((double *)p)[i] = v;
}

/* ------------------------------------------------------ centring / filter */

/* center_particles, filter_shift.jl:6-32.  Shifts the caller's positions IN
 * PLACE (in their own precision) and returns the parameters re-derived around
 * centre 0, as the reference does via the constructor (filter_shift.jl:25-31). */
int orc_center_particles(int pos_dtype, void *pos, int64_t n, int64_t sp,
                         int64_t sc, const orc_params *par, orc_params *out) {
  const double cen[3] = {par->center[0], par->center[1], par->center[2]};
  for (int64_t i = 0; i < n; ++i) {
    for (int d = 0; d < 3; ++d) {
      int64_t o = i * sp + d * sc;
      st(pos_dtype, pos, o, ld(pos_dtype, pos, o) - cen[d]);
      if (par->periodic) { /* :18-21 (shifts by boxsize/2) */
        double v = ld(pos_dtype, pos, o);
        if (fabs(v) > par->boxsize / 2) {
          st(pos_dtype, pos, o, v > 0 ? v - par->boxsize / 2 : v + par->boxsize / 2);
        }
      }
    }
  }
  double xl[2] = {par->x_lim[0] - cen[0], par->x_lim[1] - cen[0]};
  double yl[2] = {par->y_lim[0] - cen[1], par->y_lim[1] - cen[1]};
  double zl[2] = {par->z_lim[0] - cen[2], par->z_lim[1] - cen[2]};
  const double c0[3] = {0.0, 0.0, 0.0};
  int64_t P = par->Npixels[0];
  if (par->Npixels[1] > P) P = par->Npixels[1];
  if (par->Npixels[2] > P) P = par->Npixels[2];
  return orc_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, P,
                                par->boxsize, out);
}

/* filter_particles_in_image, filter_shift.jl:40-58: inclusive centre-in-box
 * test in all three dimensions; the kernel extent is ignored. */
void orc_filter_particles(int pos_dtype, const void *pos, int64_t n, int64_t sp,
                          int64_t sc, const orc_params *par, uint8_t *mask) {
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = par->center[d] - par->halfsize[d];
    hi[d] = par->center[d] + par->halfsize[d];
  }
  for (int64_t i = 0; i < n; ++i) {
    int in = 1;
    for (int d = 0; d < 3; ++d) {
      double v = ld(pos_dtype, pos, i * sp + d * sc);
      if (!(lo[d] <= v && v <= hi[d])) in = 0;
    }
    mask[i] = (uint8_t)in;
  }
}

/* ---------------------------------------------------------------- indices */

/* calculate_index, indices.jl:6-8 (1-based, x slowest). */
int64_t orc_calculate_index_2d(int64_t i, int64_t j, int64_t x_pixels) {
  return i * x_pixels + j + 1;
}
/* calculate_index, indices.jl:15-17. */
int64_t orc_calculate_index_3d(int64_t i, int64_t j, int64_t k, int64_t x_pixels,
                               int64_t y_pixels) {
  return i * x_pixels * y_pixels + j * y_pixels + k + 1;
}

/* --------------------------------------------------------- kernel shapes */

/* Normalisation of the SPHKernels.jl kernels, sigma_D for support radius h
 * (u = r/h).  Derived by integrating each shape over the unit ball. */
static double kernel_sigma(int kernel, int kdim) {
  const double pi = 3.14159265358979323846;
  switch (kernel) {
  case K_CUBIC: return kdim == 2 ? 40.0 / (7.0 * pi) : 8.0 / pi;
  case K_QUINTIC: return kdim == 2 ? 15309.0 / (478.0 * pi) : 2187.0 / (40.0 * pi);
  case K_WC4: return kdim == 2 ? 9.0 / pi : 495.0 / (32.0 * pi);
  case K_WC6: return kdim == 2 ? 78.0 / (7.0 * pi) : 1365.0 / (64.0 * pi);
  default: return kdim == 2 ? 40.0 / (3.0 * pi) : 1785.0 / (64.0 * pi);
  }
}

/* 𝒲(kernel, u, h_inv) of SPHKernels.jl (called at cic_shared.jl:24).
 * Cubic: M4 B-spline (Monaghan & Lattanzio 1985) scaled to support 1.
 * Quintic: M6 B-spline (Price 2012) scaled to support 1.
 * Wendland C4/C6/C8: psi_{4,2}, psi_{5,3}, psi_{6,4} (Wendland 1995;
 * Dehnen & Aly 2012), normalised to value 1 at u = 0. */
double orc_kernel_value(int kernel, int kdim, double u, double h_inv) {
  double hd = kdim == 2 ? h_inv * h_inv : h_inv * h_inv * h_inv;
  double n = kernel_sigma(kernel, kdim) * hd;
  double t, t2;
  switch (kernel) {
  case K_CUBIC:
    if (u < 0.5) return (1.0 + 6.0 * (u - 1.0) * (u * u)) * n;
    if (u < 1.0) { t = 1.0 - u; return (2.0 * (t * t * t)) * n; }
    return 0.0;
  case K_QUINTIC: {
    double a = 1.0 - u, b = 2.0 / 3.0 - u, c = 1.0 / 3.0 - u;
    double a5 = a * a * a * a * a, b5 = b * b * b * b * b, c5 = c * c * c * c * c;
    if (u < 1.0 / 3.0) return (a5 - 6.0 * b5 + 15.0 * c5) * n;
    if (u < 2.0 / 3.0) return (a5 - 6.0 * b5) * n;
    if (u < 1.0) return a5 * n;
    return 0.0;
  }
  case K_WC4:
    if (u < 1.0) {
      t = 1.0 - u; t2 = t * t;
      return (t2 * t2 * t2 * (1.0 + 6.0 * u + 35.0 / 3.0 * (u * u))) * n;
    }
    return 0.0;
  case K_WC6:
    if (u < 1.0) {
      t = 1.0 - u; t2 = t * t; t2 = t2 * t2;
      return (t2 * t2 * (1.0 + 8.0 * u + 25.0 * (u * u) + 32.0 * (u * u * u))) * n;
    }
    return 0.0;
  default:
    if (u < 1.0) {
      t = 1.0 - u; t2 = t * t; double t4 = t2 * t2; double t8 = t4 * t4;
      double u2 = u * u;
      return (t8 * t2 *
              (1.0 + 10.0 * u + 42.0 * u2 + 90.0 * (u2 * u) + 429.0 / 5.0 * (u2 * u2))) *
             n;
    }
    return 0.0;
  }
}

/* ----------------------------------------------------- deposition helpers */

/* Julia `min`/`max` on finite floats. */
static inline double fmin_j(double a, double b) { return b < a ? b : a; }
static inline double fmax_j(double a, double b) { return b > a ? b : a; }

/* floor(Integer, v) with Julia's InexactError for non-finite / huge values. */
static inline int floor_int(double v, int64_t *out) {
  if (!(fabs(v) < 9.2e18)) return 0;
  *out = (int64_t)floor(v);
  return 1;
}

/* pix_index_min_max, cic_shared.jl:46-52. */
static inline int pix_range(double x, double h, int64_t P, int64_t *lo, int64_t *hi) {
  int64_t a, b;
  if (!floor_int(x - h, &a) || !floor_int(x + h, &b)) return 0;
  *lo = a > 0 ? a : 0;
  *hi = b < P - 1 ? b : P - 1;
  return 1;
}

typedef struct {
  int dims, kernel, kdim, calc_mean, nq;
  const orc_params *par;
  int pos_dtype, attr_dtype;
  const void *pos; int64_t sp, sc;
  const void *hsml, *m, *rho, *w, *q;
  int64_t q_sp, q_sc;
  const int64_t *order; int64_t n_order;
  double *image; /* (P^D, nq+1) column-major */
  double grid_mass, particle_mass;
  int64_t deposits;
  int status;
  double *wk, *A; int64_t cap; /* footprint scratch */
} cic_job;

static int ensure_cap(cic_job *J, int64_t need) {
  if (need <= J->cap) return 1;
  int64_t c = need * 2;
  double *a = (double *)realloc(J->wk, (size_t)c * sizeof(double));
  if (!a) return 0;
  J->wk = a;
  double *b = (double *)realloc(J->A, (size_t)c * sizeof(double));
  if (!b) return 0;
  J->A = b;
  J->cap = c;
  return 1;
}

/* cic_mapping_2D (cic_2D.jl:103-244) with calculate_weights (cic_2D.jl:11-72),
 * get_weight_per_pixel (cic_shared.jl:9-39) and update_image!
 * (cic_shared.jl:111-121); cic_mapping_3D (cic_3D.jl:110-208) for dims == 3. */
static void cic_run(cic_job *J) {
  const orc_params *par = J->par;
  const double L = par->len2pix;
  const int64_t P = par->Npixels[0];
  const int64_t PD = J->dims == 2 ? P * P : P * P * P;
  const int nq = J->nq;
  double bq[64];
  for (int64_t o = 0; o < J->n_order; ++o) {
    int64_t p = J->order[o];
    /* cic_2D.jl:154-168 / cic_3D.jl:140-144 */
    int scalar_zero = 0, allzero = 1;
    for (int k = 0; k < nq; ++k) {
      bq[k] = ld(J->attr_dtype, J->q, p * J->q_sp + k * J->q_sc);
      if (bq[k] != 0.0) allzero = 0;
    }
    if (nq > 1 && allzero) scalar_zero = 1; /* bin_q collapses to scalar 0.0 */
    if (allzero && !J->calc_mean) continue;
    double px = ld(J->pos_dtype, J->pos, p * J->sp);
    double py = ld(J->pos_dtype, J->pos, p * J->sp + J->sc);
    double pz = ld(J->pos_dtype, J->pos, p * J->sp + 2 * J->sc);
    double los_weight = ld(J->attr_dtype, J->w, p);
    double hsml, hsml_inv, area = 0.0, dz_col = 0.0, vol = 0.0;
    double rho_in = ld(J->attr_dtype, J->rho, p), m_in = ld(J->attr_dtype, J->m, p);
    if (J->dims == 2) { /* get_quantities_2D, cic_2D.jl:80-91 */
      hsml = ld(J->attr_dtype, J->hsml, p) * L;
      hsml_inv = 1.0 / hsml;
      area = (2.0 * hsml) * (2.0 * hsml);
      double rho = rho_in * (1.0 / (L * L * L));
      dz_col = m_in / rho / area;
    } else { /* get_quantities_3D, cic_3D.jl:87-97 */
      hsml = ld(J->attr_dtype, J->hsml, p) * L;
      hsml_inv = 1.0 / hsml;
      double rho = rho_in / (L * L * L);
      vol = m_in / rho;
    }
    /* get_xyz, cic_shared.jl:85-99 */
    double x = px * L, y = py * L, z = pz * L;
    x += 0.5 * (double)P;
    y += 0.5 * (double)P;
    z += 0.5 * (double)P;
    int64_t iMin, iMax, jMin, jMax, kMin = 0, kMax = 0;
    if (!pix_range(x, hsml, P, &iMin, &iMax) || !pix_range(y, hsml, P, &jMin, &jMax) ||
        (J->dims == 3 && !pix_range(z, hsml, P, &kMin, &kMax))) {
      J->status = ORC_ERR_NONFINITE;
      return;
    }
    int64_t ni = iMax - iMin + 1, nj = jMax - jMin + 1, nk = kMax - kMin + 1;
    if (ni < 0) ni = 0;
    if (nj < 0) nj = 0;
    if (nk < 0) nk = 0;
    int64_t F = J->dims == 2 ? ni * nj : ni * nj * nk;
    J->deposits += F;
    if (!ensure_cap(J, F > 0 ? F : 1)) { J->status = ORC_ERR_ALLOC; return; }
    double *wk = J->wk, *A = J->A;
    /* calculate_weights: pass 1 over the footprint */
    int64_t n_distr = 0, n_tot = 0;
    double distr_weight = 0.0, distr_area = 0.0;
    int64_t f = 0;
    for (int64_t i = iMin; i <= iMax; ++i) {
      double x_dist = x - (double)i - 0.5;
      double dx = fmin_j(x + hsml, (double)(i + 1)) - fmax_j(x - hsml, (double)i);
      for (int64_t j = jMin; j <= jMax; ++j) {
        double y_dist = y - (double)j - 0.5;
        double dy = fmin_j(y + hsml, (double)(j + 1)) - fmax_j(y - hsml, (double)j);
        if (J->dims == 2) {
          double u = sqrt(x_dist * x_dist + y_dist * y_dist) * hsml_inv;
          double dxdy = dx * dy;
          A[f] = dxdy;
          distr_area += dxdy;
          n_tot += 1;
          if (u <= 1.0) {
            double w_ = orc_kernel_value(J->kernel, J->kdim, u, hsml_inv);
            distr_weight += w_ * dxdy;
            n_distr += 1;
            wk[f] = w_;
          } else {
            wk[f] = 0.0;
          }
          ++f;
        } else {
          for (int64_t k = kMin; k <= kMax; ++k) {
            double z_dist = z - (double)k - 0.5;
            double dzz = fmin_j(z + hsml, (double)(k + 1)) - fmax_j(z - hsml, (double)k);
            double dxdydz = dx * dy * dzz;
            double u = sqrt(x_dist * x_dist + y_dist * y_dist + z_dist * z_dist) * hsml_inv;
            A[f] = dxdydz;
            distr_area += dxdydz;
            n_tot += 1;
            if (u <= 1.0) {
              double w_ = orc_kernel_value(J->kernel, J->kdim, u, hsml_inv);
              distr_weight += w_ * dxdydz;
              n_distr += 1;
              wk[f] = w_;
            } else {
              wk[f] = 0.0;
            }
            ++f;
          }
        }
      }
    }
    double weight_per_pix;
    if (distr_weight == 0.0) { /* fallback: no pixel centre inside the kernel */
      n_distr = n_tot;
      for (int64_t t = 0; t < F; ++t) wk[t] = 1.0;
      weight_per_pix = distr_area != 0.0 ? (double)n_distr / distr_area : 1.0;
    } else {
      weight_per_pix = (double)n_distr / distr_weight;
    }
    double norm;
    if (J->dims == 2) { /* cic_2D.jl:187-188 */
      double kernel_norm = area / (double)n_distr;
      norm = kernel_norm * weight_per_pix * los_weight * dz_col;
    } else { /* cic_3D.jl:168-169 */
      double kernel_norm = vol / (double)n_distr;
      norm = kernel_norm * weight_per_pix * los_weight * L;
    }
    /* pass 2: deposit */
    f = 0;
    for (int64_t i = iMin; i <= iMax; ++i) {
      for (int64_t j = jMin; j <= jMax; ++j) {
        for (int64_t k = kMin; k <= (J->dims == 2 ? kMin : kMax); ++k) {
          int64_t idx = J->dims == 2 ? i * P + j : i * P * P + j * P + k;
          double pix_weight = wk[f] * A[f] * norm;
          if (pix_weight != 0.0) {
            J->image[idx + (int64_t)nq * PD] += pix_weight;
            if (scalar_zero) {
              J->image[idx] += 0.0 * pix_weight;
            } else {
              for (int c = 0; c < nq; ++c) J->image[idx + c * PD] += bq[c] * pix_weight;
            }
          }
          if (J->dims == 3) /* cic_3D.jl:186 */
            J->grid_mass += rho_in * wk[f] * A[f] / (L * L * L);
          ++f;
        }
      }
    }
    J->particle_mass += m_in;
  }
}

static void *cic_thread(void *arg) {
  cic_run((cic_job *)arg);
  return NULL;
}

/* ----------------------------------------------------------------- reduce */

/* reduce_image_2D, reduce_image.jl:8-31: out[ix, iy, q] (column-major,
 * flat ix + P*iy + P^2*q) = Q_q / W where W > 0 (if reduce). */
void orc_reduce_image_2d(const double *image, int64_t P, int nq, int reduce,
                         double *out) {
  int64_t PD = P * P;
  for (int64_t ix = 0; ix < P; ++ix)
    for (int64_t iy = 0; iy < P; ++iy) {
      int64_t k = ix * P + iy;
      double W = image[k + (int64_t)nq * PD];
      for (int c = 0; c < nq; ++c) {
        double v = image[k + c * PD];
        if (reduce && W > 0.0) v /= W;
        out[ix + P * iy + PD * c] = v;
      }
    }
}

/* reduce_image_3D, reduce_image.jl:39-55: out[iz, iy, ix] (column-major,
 * flat iz + P*iy + P^2*ix) = Q / W only where Q > 0. */
void orc_reduce_image_3d(const double *image, int64_t P, double *out) {
  int64_t PD = P * P * P;
  for (int64_t m = 0; m < PD; ++m) {
    double v = image[m];
    if (v > 0.0) v /= image[m + PD];
    out[m] = v; /* m = ix*P^2 + iy*P + iz == iz + P*iy + P^2*ix */
  }
}

/* -------------------------------------------------------- per-particle info */

/* Integer footprint of each particle after centring/filtering (for bit-exact
 * checks of the device pre-pass): rng[6*i..] = iMin,iMax,jMin,jMax,kMin,kMax
 * (k = 0,0 in 2D); state[i] = 0 filtered out, 1 skipped (q == 0 and
 * !calc_mean), 2 mapped.  Positions must already be centred. */
int orc_footprints(int dims, const orc_params *par, int pos_dtype, const void *pos,
                   int64_t sp, int64_t sc, int attr_dtype, const void *hsml,
                   const void *q, int nq, int64_t q_sp, int64_t q_sc, int calc_mean,
                   int64_t n, int64_t *rng, int8_t *state) {
  uint8_t *mask = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
  if (!mask) return ORC_ERR_ALLOC;
  orc_filter_particles(pos_dtype, pos, n, sp, sc, par, mask);
  const double L = par->len2pix;
  const int64_t P = par->Npixels[0];
  int status = ORC_OK;
  for (int64_t p = 0; p < n; ++p) {
    for (int t = 0; t < 6; ++t) rng[6 * p + t] = 0;
    if (!mask[p]) { state[p] = 0; continue; }
    int allzero = 1;
    for (int k = 0; k < nq; ++k)
      if (ld(attr_dtype, q, p * q_sp + k * q_sc) != 0.0) allzero = 0;
    if (allzero && !calc_mean) { state[p] = 1; continue; }
    state[p] = 2;
    double h = ld(attr_dtype, hsml, p) * L;
    double c[3];
    for (int d = 0; d < 3; ++d) {
      c[d] = ld(pos_dtype, pos, p * sp + d * sc) * L;
      c[d] += 0.5 * (double)P;
    }
    for (int d = 0; d < dims; ++d)
      if (!pix_range(c[d], h, P, &rng[6 * p + 2 * d], &rng[6 * p + 2 * d + 1]))
        status = ORC_ERR_NONFINITE;
  }
  free(mask);
  return status;
}

/* ------------------------------------------------------------- sphMapping */

typedef struct { double v; int64_t i; } zkey;

/* Julia isless on Float64 (NaN greatest, -0.0 < 0.0), tie -> index. */
static int zkey_cmp(const void *a, const void *b) {
  const zkey *x = (const zkey *)a, *y = (const zkey *)b;
  int xn = isnan(x->v), yn = isnan(y->v);
  if (xn != yn) return xn ? 1 : -1;
  if (!xn) {
    if (x->v < y->v) return -1;
    if (x->v > y->v) return 1;
    if (signbit(x->v) != signbit(y->v)) return signbit(x->v) ? -1 : 1;
  }
  return x->i < y->i ? -1 : (x->i > y->i ? 1 : 0);
}

/* sphMapping, cic_interpolation.jl:35-272.  Centres `pos` in place, filters,
 * maps with `nthreads` workers (nthreads > 1 mirrors parallel=true: the
 * contiguous split of domain_decomp.jl:7-16 and the left-fold image sum of
 * cic_interpolation.jl:199,256) and reduces.  `out` receives:
 *   dims 2, return_both_maps: raw (P^2, nq+1) column-major accumulator;
 *   dims 2: (P, P, nq) [x, y, q];   dims 3: (P, P, P) [z, y, x].
 * `par_io` is replaced by the re-derived centred parameters. */
int orc_sph_mapping(orc_params *par_io, int dims, int kernel, int kdim,
                    int pos_dtype, void *pos, int64_t sp, int64_t sc, int attr_dtype,
                    const void *hsml, const void *m, const void *rho, const void *q,
                    int nq, int64_t q_sp, int64_t q_sc, const void *w, int64_t n,
                    int reduce_image, int return_both_maps, int calc_mean, int sort_z,
                    int nthreads, double *out, double *grid_mass, int64_t *deposits) {
  if (dims != 2 && dims != 3) return ORC_ERR_DIMS;
  if (nq < 1 || nq > 64) return ORC_ERR_ARG;
  if (dims == 3 && nq != 1) return ORC_ERR_NQ;
  if (dims == 3) calc_mean = 0; /* cic_mapping_3D is called without calc_mean: :219 */
  const int64_t P0 = par_io->Npixels[0];
  orc_params par;
  int st_ = orc_center_particles(pos_dtype, pos, n, sp, sc, par_io, &par);
  if (st_) return st_;
  uint8_t *mask = (uint8_t *)malloc((size_t)(n > 0 ? n : 1));
  int64_t *order = (int64_t *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
  if (!mask || !order) { free(mask); free(order); return ORC_ERR_ALLOC; }
  orc_filter_particles(pos_dtype, pos, n, sp, sc, &par, mask);
  int64_t n_sel = 0;
  if (sort_z) {
    /* filter_shift.jl:61-63: reverse(sortperm(z))[mask], mask in input order */
    zkey *keys = (zkey *)malloc((size_t)(n > 0 ? n : 1) * sizeof(zkey));
    if (!keys) { free(mask); free(order); return ORC_ERR_ALLOC; }
    for (int64_t i = 0; i < n; ++i) {
      keys[i].v = ld(pos_dtype, pos, i * sp + 2 * sc);
      keys[i].i = i;
    }
    qsort(keys, (size_t)n, sizeof(zkey), zkey_cmp);
    for (int64_t i = 0; i < n; ++i)
      if (mask[i]) order[n_sel++] = keys[n - 1 - i].i;
    free(keys);
  } else {
    for (int64_t i = 0; i < n; ++i)
      if (mask[i]) order[n_sel++] = i;
  }
  free(mask);
  const int64_t P = par.Npixels[0];
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  const int64_t img_len = PD * (nq + 1);
  int T = nthreads < 1 ? 1 : nthreads;
  cic_job *jobs = (cic_job *)calloc((size_t)T, sizeof(cic_job));
  double *img = (double *)calloc((size_t)img_len * (size_t)T, sizeof(double));
  if (!jobs || !img) { free(jobs); free(img); free(order); return ORC_ERR_ALLOC; }
  int64_t bsize = n_sel / T;
  for (int t = 0; t < T; ++t) {
    cic_job *J = &jobs[t];
    J->dims = dims; J->kernel = kernel; J->kdim = kdim; J->calc_mean = calc_mean;
    J->nq = nq; J->par = &par; J->pos_dtype = pos_dtype; J->attr_dtype = attr_dtype;
    J->pos = pos; J->sp = sp; J->sc = sc; J->hsml = hsml; J->m = m; J->rho = rho;
    J->w = w; J->q = q; J->q_sp = q_sp; J->q_sc = q_sc;
    int64_t b0 = (int64_t)t * bsize, b1 = (t == T - 1) ? n_sel : (int64_t)(t + 1) * bsize;
    J->order = order + b0; J->n_order = b1 - b0;
    J->image = img + (size_t)t * (size_t)img_len;
  }
  if (T == 1) {
    cic_run(&jobs[0]);
  } else {
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)T);
    for (int t = 0; t < T; ++t) pthread_create(&th[t], NULL, cic_thread, &jobs[t]);
    for (int t = 0; t < T; ++t) pthread_join(th[t], NULL);
    free(th);
    for (int t = 1; t < T; ++t) { /* sum(fetch.(futures)): left fold */
      double *dst = img, *src = img + (size_t)t * (size_t)img_len;
      for (int64_t e = 0; e < img_len; ++e) dst[e] += src[e];
    }
  }
  int status = ORC_OK;
  double gm = 0.0;
  int64_t dep = 0;
  for (int t = 0; t < T; ++t) {
    if (jobs[t].status) status = jobs[t].status;
    gm += jobs[t].grid_mass;
    dep += jobs[t].deposits;
    free(jobs[t].wk);
    free(jobs[t].A);
  }
  if (status == ORC_OK) {
    if (dims == 2) {
      if (return_both_maps)
        memcpy(out, img, (size_t)img_len * sizeof(double));
      else
        orc_reduce_image_2d(img, P0, nq, reduce_image, out);
    } else if (return_both_maps == 2) {
      /* raw (P^3, 2) accumulator: not an output of the reference (its 3D path
       * always reduces); used to check adjoints */
      memcpy(out, img, (size_t)img_len * sizeof(double));
    } else {
      if (!reduce_image)
        for (int64_t e = 0; e < PD; ++e) img[PD + e] = 1.0; /* :230-232 */
      orc_reduce_image_3d(img, P0, out);
    }
  }
  if (grid_mass) *grid_mass = gm;
  if (deposits) *deposits = dep;
  *par_io = par;
  free(jobs);
  free(img);
  free(order);
  return status;
}

/* ------------------------------------------------- one particle's weights */

/* Weights pw of ONE particle (attributes given as doubles, position already
 * centred) on its footprint pixels: idx[t] (flat, x slowest) and pw[t] for
 * t < return value (-1 on error / capacity).  The same arithmetic as
 * cic_run, used to take finite differences of a loss particle by particle. */
int64_t orc_particle_contrib(int dims, const orc_params *par, int kernel, int kdim, double px,
                             double py, double pz, double hsml_in, double m_in, double rho_in,
                             double w_in, int64_t cap, int64_t *idx, double *pw) {
  const int64_t P = par->Npixels[0];
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  double pos[3] = {px, py, pz};
  double one = 1.0;
  int64_t order = 0;
  double *img = (double *)calloc((size_t)PD * 2, sizeof(double));
  if (!img) return -1;
  cic_job J;
  memset(&J, 0, sizeof(J));
  J.dims = dims; J.kernel = kernel; J.kdim = kdim; J.calc_mean = 0; J.nq = 1;
  J.par = par; J.pos_dtype = ORC_F64; J.attr_dtype = ORC_F64;
  J.pos = pos; J.sp = 3; J.sc = 1;
  J.hsml = &hsml_in; J.m = &m_in; J.rho = &rho_in; J.w = &w_in; J.q = &one;
  J.q_sp = 1; J.q_sc = 0; J.order = &order; J.n_order = 1; J.image = img;
  cic_run(&J);
  free(J.wk);
  free(J.A);
  int64_t n = 0;
  if (J.status == ORC_OK) {
    for (int64_t e = 0; e < PD; ++e) {
      if (img[PD + e] != 0.0) {
        if (n >= cap) { n = -1; break; }
        idx[n] = e;
        pw[n] = img[PD + e];
        ++n;
      }
    }
  } else {
    n = -1;
  }
  free(img);
  return n;
}
