// tiled_kernels.cuh -- templates of the per-kernel-shape passes of the
// FP32-compensated tiled deposition: K3 k_norm_fill and K4 k_deposit (see
// tiled.cuh).  Each tiled_k<K>.cu instantiates them for one SPHKernels shape
// so the build compiles the shapes in parallel.
#pragma once

#include <cuda_runtime.h>

#include <climits>

#include "internal.h"
#include "tiled.cuh"

namespace sphg {
namespace tiled_detail {

// Maps with at most this many tiles count a CTA's (particle, tile) overlaps
// in shared memory first, then add them to the global counts once per tile
// touched (a dense map of few tiles otherwise serialises its particles on
// a few global counters).
constexpr int kTileHist = 4096;

// m 2^e as a double, for m a float in [2^-6, 2] and |e| < 1000 (the
// exponent field of (double)m raised by e; no FP64 arithmetic).
__device__ __forceinline__ double scale_to_double(float m, int e) {
  return __longlong_as_double(__double_as_longlong((double)m) + ((long long)e << 52));
}

// The record's weight factor numerator (w m L^3 / rho, times L in 3D) and
// 3D mass factor (rho / L^3 * sigma / h^kdim) to FP32 accuracy over the
// whole FP64 range: FP32 products of the inputs' mantissas, their binary
// exponents summed as integers.  False (the caller takes FP64) for a zero,
// subnormal or non-finite input.
template <int DIMS>
__device__ __forceinline__ bool factors_f32(const DevMapParams& mp, const PrepLite& q, double* cp, double* aux) {
  if (!q.f32 || !mp.fac_ok) return false;
  float wm, mm, rm, hm;
  int we, me, re, he;
  split_f(q.w32, wm, we);
  split_f(q.m32, mm, me);
  split_f(q.rho32, rm, re);
  split_f(q.g[3], hm, he);
  const auto normal = [](float m) { return m >= 0.5f && m < 1.0f; };  // split_f leaves others as they are
  if (!(normal(fabsf(wm)) && normal(fabsf(mm)) && normal(fabsf(rm)) && normal(fabsf(hm)))) return false;
  const float Lm = mp.fac_m[0], L3m = mp.fac_m[1], sm = mp.fac_m[2];
  const int Le = mp.fac_e[0], L3e = mp.fac_e[1], se = mp.fac_e[2];
  float c = (wm * mm) * L3m / rm;  // [2^-3, 2]
  int ce = we + me + L3e - re;
  if (DIMS == 3) {
    c *= Lm;
    ce += Le;
  }
  const float hk = mp.kernel_dim == 2 ? hm * hm : hm * hm * hm;
  const float a = (rm * sm) / (hk * L3m);  // [2^-2, 2^4], scaled by 2^-4 below
  const int ae = re + se - (mp.kernel_dim == 2 ? 2 : 3) * he - L3e + 4;
  if (!(abs(ce) < 1000 && abs(ae) < 1000)) return false;
  *cp = scale_to_double(c, ce);
  *aux = scale_to_double(a * 0.0625f, ae);
  return true;
}

// K1 body: this CTA's threads take particles base0 + threadIdx.x, then
// every `stride` further, below `end` (a whole CTA enters each iteration
// together).
struct PrepShared {
  int hist[kTileHist];  // overlaps per tile (maps of few tiles)
  int list[kTileHist];  // tiles touched by this CTA, once each
  int nlist;
};

template <int DIMS>
__device__ void prep_count(const TiledArgs& A, int64_t base0, int64_t stride, PrepShared& sh,
                           int64_t end = INT64_MAX) {
  int* const s_hist = sh.hist;
  int* const s_list = sh.list;
  const bool hist = A.n_tiles <= kTileHist;  // uniform across the CTA
  if (hist) {
    for (int i = threadIdx.x; i < (int)A.n_tiles; i += blockDim.x) s_hist[i] = 0;
    if (threadIdx.x == 0) sh.nlist = 0;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  unsigned long long c_mapped = 0, c_dep = 0;
  double c_pm = 0.0;
  unsigned flags = 0;
  const int64_t stop = end < A.pt.n ? end : A.pt.n;
  for (int64_t base = base0; base < stop; base += stride) {
    const int64_t p = base + threadIdx.x;
    PrepLite q;
    int state = kPrepSkip;
    if (p < A.pt.n) state = prep_particle_lite<DIMS>(A.pt, A.mp, p, true, &q);
    if (state == kPrepNonFinite) flags |= kFlagNonFinite;
    int ni = 0, nj = 0, nk = 0;
    if (state == kPrepMapped) {
      ni = (int)(q.hi[0] - q.lo[0] + 1);
      nj = (int)(q.hi[1] - q.lo[1] + 1);
      nk = (int)(q.hi[2] - q.lo[2] + 1);
      c_mapped += 1;
      c_dep += (unsigned long long)ni * nj * nk;
      c_pm += q.mass();
    }
    const bool rec = state == kPrepMapped && ni > 0 && nj > 0 && nk > 0;
    // warp-aggregated slot allocation
    const unsigned bal = __ballot_sync(0xffffffffu, rec);
    int slot0 = 0;
    if (bal) {
      const int leader = __ffs(bal) - 1;
      if (lane == leader) slot0 = atomicAdd(A.n_rec, __popc(bal));
      slot0 = __shfl_sync(0xffffffffu, slot0, leader);
    }
    if (rec) {
      const int r = slot0 + __popc(bal & lanemask_lt());
      const int i0 = (int)q.lo[0], j0 = (int)q.lo[1], k0 = (int)q.lo[2];
      A.box[r] = make_int4(i0, j0, k0, 0);
      A.dimv[r] = make_int4(ni, nj, nk, (int)p);
      A.geo[r] = make_float4(q.g[0], q.g[1], q.g[2], q.g[3]);
      // weight factor numerator, area*w*dz (cic_2D.jl:187-188) = w m / rho_pix
      // or vol*w*L (cic_3D.jl:168-169) = w m L / rho_pix, with
      // rho_pix = rho / L^3; FP32 accuracy suffices here (the FP32 method
      // derives FP32 factors from it; ill-conditioned records redo it in
      // FP64), so no FP64 division
      double cpv, auxv;
      if (!factors_f32<DIMS>(A.mp, q, &cpv, &auxv)) {
        const double L = A.mp.L, L3 = L * L * L;
        const double wm_rho = q.weight() * q.mass() * L3 * rcp_approx(q.rho());
        cpv = DIMS == 2 ? wm_rho : wm_rho * L;
        // 3D mass diagnostic factor rho/L^3 * kernel normalisation
        const double hi_ = rcp_approx(q.h());
        auxv = q.rho() * (A.mp.sigma * (A.mp.kernel_dim == 2 ? hi_ * hi_ : hi_ * hi_ * hi_)) * rcp_approx(L3);
      }
      A.cp[r] = cpv;
      A.aux[r] = auxv;
      for (int k = 0; k < A.pt.nq; ++k)
        A.qv[(int64_t)k * A.cap + r] = q.scalar_zero ? 0.0f
            : A.pt.attr_dtype == 0 ? __ldg((const float*)A.pt.q + p * A.pt.qsp + k * A.pt.qsk)
                                   : __double2float_rn(ld_elem(A.pt.attr_dtype, A.pt.q, p * A.pt.qsp + k * A.pt.qsk));
      if ((int64_t)ni * nj * nk > A.large_cells) A.large[atomicAdd(A.n_large, 1)] = r;
      // (particle, tile) overlaps
      const int tx0 = i0 / A.tdim[0], tx1 = (i0 + ni - 1) / A.tdim[0];
      const int ty0 = j0 / A.tdim[1], ty1 = (j0 + nj - 1) / A.tdim[1];
      const int tz0 = k0 / A.tdim[2], tz1 = (k0 + nk - 1) / A.tdim[2];
      for (int tx = tx0; tx <= tx1; ++tx)
        for (int ty = ty0; ty <= ty1; ++ty)
          for (int tz = tz0; tz <= tz1; ++tz) {
            const int64_t t = ((int64_t)tx * A.ntile[1] + ty) * A.ntile[2] + tz;
            if (!hist) atomicAdd(&A.tile_count[t], 1);
            else if (atomicAdd(&s_hist[t], 1) == 0) s_list[atomicAdd(&sh.nlist, 1)] = (int)t;
          }
    }
  }
  if (hist) {
    __syncthreads();
    for (int i = threadIdx.x; i < sh.nlist; i += blockDim.x) atomicAdd(&A.tile_count[s_list[i]], s_hist[s_list[i]]);
  }
  c_pm = warp_sum_d(c_pm);
  c_mapped = (unsigned long long)warp_sum_ll((long long)c_mapped);
  c_dep = (unsigned long long)warp_sum_ll((long long)c_dep);
  flags = __reduce_or_sync(0xffffffffu, flags);
  if (lane == 0) {
    if (c_mapped) {
      atomicAdd(&A.st->n_mapped, c_mapped);
      atomicAdd(&A.st->deposits, c_dep);
      atomicAdd(&A.st->particle_mass, c_pm);
    }
    if (flags) atomicOr(&A.st->flags, flags);
  }
}

// K2 body: exclusive scan of the tile counts by one CTA of 1024 threads.
__device__ inline void scan_tiles(const TiledArgs& A, long long* part) {
  const int64_t n = A.n_tiles;
  const int64_t per = (n + blockDim.x - 1) / blockDim.x;
  const int64_t b = (int64_t)threadIdx.x * per, e = b + per < n ? b + per : n;
  long long s = 0;
  for (int64_t i = b; i < e; ++i) s += A.tile_count[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // Hillis-Steele inclusive scan
    long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  long long run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int64_t i = b; i < e; ++i) {
    A.tile_start[i] = run;
    run += A.tile_count[i];
  }
  if (threadIdx.x == blockDim.x - 1) {
    A.tile_start[n] = part[blockDim.x - 1];
    if (part[blockDim.x - 1] > A.pair_cap) atomicOr(&A.st->flags, kFlagOverflow);
  }
  // chunk prefix of the large records (few: a serial pass by one warp)
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nl = *A.n_large;
    long long run = 0;
    for (int base = 0; base < nl; base += 32) {
      const int i = base + threadIdx.x;
      long long c = 0;
      if (i < nl) {
        const int4 dm = A.dimv[A.large[i]];
        c = ((int64_t)dm.x * dm.y * dm.z + kChunkCells - 1) / kChunkCells;
      }
      long long incl = c;  // inclusive warp scan
      for (int o = 1; o < 32; o <<= 1) {
        const long long v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)threadIdx.x >= o) incl += v;
      }
      if (i < nl) A.large_start[i] = run + incl - c;
      run += __shfl_sync(0xffffffffu, incl, 31);
    }
    if (threadIdx.x == 0) {
      A.large_start[nl] = run;
      if (run > A.chunk_cap) atomicOr(&A.st->flags, kFlagOverflow);
    }
  }
}


// FP32 renormalisation partial sum of record cells [f0, f1) with stride
// `step` starting at f0 + first, compensated (TwoSum per addition), and the
// smallest u seen.
template <int DIMS, int KERN>
__device__ __forceinline__ void cell_term(int kern, float2 ex, float2 ey, float2 ez, float hinv, float& s,
                                          float& comp, float& umin) {
  const float u = u_of((ex.x + ey.x) + ez.x, hinv);
  umin = fminf(umin, u);
  if (u <= 1.0f) {
    float t, e;
    two_sum(s, shape_f<KERN>(kern, u) * (ex.y * ey.y * ez.y), t, e);
    s = t;
    comp += e;
  }
}

template <int DIMS, int KERN>
__device__ __forceinline__ void cell_sum_fp32(int kern, const float4 g, float h, float hinv, int a, int b, int c,
                                              float& s, float& comp, float& umin) {
  const float2 ez = DIMS == 3 ? axis_sq(g.z, h, c) : make_float2(0.0f, 1.0f);
  cell_term<DIMS, KERN>(kern, axis_sq(g.x, h, a), axis_sq(g.y, h, b), ez, hinv, s, comp, umin);
}

template <int DIMS, int KERN>
__device__ __forceinline__ void record_sum_fp32(int kern, const float4 g, const int4 dm, int64_t f0, int64_t f1,
                                                int first, int step, float& s, float& comp, float& umin) {
  const int njk = dm.y * dm.z;
  const float h = g.w, hinv = 1.0f / g.w;
  if (f1 + njk < (1 << 20)) {
    // 32-bit cell index, decomposed with float reciprocals (exact here)
    const float inv_njk = inv_small(njk), inv_nz = inv_small(dm.z);
    for (int f = (int)f0 + first; f < (int)f1; f += step) {
      const int a = fdiv(f, inv_njk);
      const int rr = f - a * njk;
      const int b = fdiv(rr, inv_nz), c = rr - b * dm.z;
      cell_sum_fp32<DIMS, KERN>(kern, g, h, hinv, a, b, c, s, comp, umin);
    }
  } else {
    for (int64_t f = f0 + first; f < f1; f += step) {
      const int a = (int)(f / njk);
      const int rr = (int)(f - (int64_t)a * njk);
      const int b = rr / dm.z, c = rr - b * dm.z;
      cell_sum_fp32<DIMS, KERN>(kern, g, h, hinv, a, b, c, s, comp, umin);
    }
  }
}

// Per-warp axis tables of the renormalisation pass (footprints with every
// side at most kNormTab cells).
constexpr int kNormTab = 64;

// 3D footprints with at most this many (x, y) columns also get a per-warp
// plane table.
constexpr int kNormPlane = 256;

// A cell from its (x, y) plane entry {sx + sy, ox * oy} and its z term: the
// same operations in the same order as cell_term, so the same u and weight.
template <int DIMS, int KERN>
__device__ __forceinline__ void cell_term_plane(int kern, float2 pxy, float2 ez, float hinv, float& s,
                                                float& comp, float& umin) {
  const float u = u_of(pxy.x + ez.x, hinv);
  umin = fminf(umin, u);
  if (u <= 1.0f) {
    float t, e;
    two_sum(s, shape_f<KERN>(kern, u) * (pxy.y * ez.y), t, e);
    s = t;
    comp += e;
  }
}

// Per-warp scratch of the renormalisation pass (one instance per kernel,
// shared by every specialisation it inlines).
// Per-warp: the 3D plane table while the warp sums a group's records, then
// the group's pair sources (PairSrc, five uint4 each) while it writes their
// pair records.
union NormWarpShared {
  float2 plane[kNormPlane];
  uint4 src[32][5];
};
struct NormShared {
  float2 tabs[8][3][kNormTab];
  NormWarpShared w[8];
};

// The whole footprint of one record from per-axis tables filled by the warp
// (3D footprints with few columns: from a plane table too, one index
// division per cell instead of two).
template <int DIMS, int KERN>
__device__ __forceinline__ void record_sum_tab(int kern, const float4 g, const int4 dm, int lane, float2 (*tab)[kNormTab],
                                               float2* plane, float& s, float& comp, float& umin) {
  const float h = g.w, hinv = 1.0f / g.w;
  const int ntab = dm.x + dm.y + (DIMS == 3 ? dm.z : 0);
  for (int i = lane; i < ntab; i += 32) {  // axis and offset by selects (no divergence)
    const int ax = i < dm.x ? 0 : (i < dm.x + dm.y ? 1 : 2);
    const int k = i - (ax == 0 ? 0 : (ax == 1 ? dm.x : dm.x + dm.y));
    tab[ax][k] = axis_sq(ax == 0 ? g.x : (ax == 1 ? g.y : g.z), h, k);
  }
  __syncwarp();
  if (DIMS == 3 && dm.x * dm.y <= kNormPlane) {
    // Only the columns whose (x, y) offset can be within h: a column with
    // sx + sy above h^2 (with a margin far above the FP32 rounding of the
    // per-cell test u <= 1) has no cell inside the support.  A sphere's
    // columns fill about three quarters of its footprint's.
    const int nab = dm.x * dm.y;
    const float inv_ny = inv_small(dm.y);
    const float R2 = h * h * (1.0f + 0x1p-10f);
    int ncol = 0;
    for (int i0 = 0; i0 < nab; i0 += 32) {
      const int i = i0 + lane;
      float2 pxy = make_float2(0.0f, 0.0f);
      bool keep = false;
      if (i < nab) {
        const int a = fdiv(i, inv_ny), b = i - a * dm.y;
        const float2 ex = tab[0][a], ey = tab[1][b];
        pxy = make_float2(ex.x + ey.x, ex.y * ey.y);
        keep = !(pxy.x > R2);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) plane[ncol + __popc(bal & lanemask_lt())] = pxy;
      ncol += __popc(bal);
    }
    __syncwarp();
    const int F = ncol * dm.z;
    const float inv_nz = inv_small(dm.z);
    for (int f = lane; f < F; f += 32) {
      const int ab = fdiv(f, inv_nz), c = f - ab * dm.z;
      cell_term_plane<DIMS, KERN>(kern, plane[ab], tab[2][c], hinv, s, comp, umin);
    }
    __syncwarp();  // the tables are refilled for the next record
    return;
  }
  const int njk = dm.y * dm.z;
  const int F = dm.x * njk;
  const float inv_njk = inv_small(njk), inv_nz = inv_small(dm.z);
  for (int f = lane; f < F; f += 32) {
    const int a = fdiv(f, inv_njk);
    const int rr = f - a * njk;
    const int b = DIMS == 3 ? fdiv(rr, inv_nz) : rr, c = DIMS == 3 ? rr - b * dm.z : 0;
    const float2 ez = DIMS == 3 ? tab[2][c] : make_float2(0.0f, 1.0f);
    cell_term<DIMS, KERN>(kern, tab[0][a], tab[1][b], ez, hinv, s, comp, umin);
  }
  __syncwarp();  // the tables are refilled for the next record
}

// Lane 0 derives the particle's FP64 quantities (prep_particle_fp64) and
// broadcasts the ones the cell loops need: FP64 is a small fraction of FP32
// throughput on GB300, so the other lanes do not repeat it.
template <int DIMS>
__device__ __forceinline__ void prep_bcast(const DevParticles& pt, const DevMapParams& mp, int64_t p, int lane,
                                           PrepFP64* q) {
  PrepFP64 v;
  v.x = v.y = v.z = v.hsml = v.h_inv = v.knorm = v.area = v.col = v.vol = v.m_in = v.rho_in = v.wgt = 0.0;
  if (lane == 0) prep_particle_fp64<DIMS>(pt, mp, p, false, &v);
  const unsigned full = 0xffffffffu;
  q->x = __shfl_sync(full, v.x, 0);
  q->y = __shfl_sync(full, v.y, 0);
  q->z = __shfl_sync(full, v.z, 0);
  q->hsml = __shfl_sync(full, v.hsml, 0);
  q->h_inv = __shfl_sync(full, v.h_inv, 0);
  q->knorm = __shfl_sync(full, v.knorm, 0);
  q->area = v.area;  // lane 0 only: the per-particle factors
  q->col = v.col;
  q->vol = v.vol;
  q->m_in = v.m_in;
  q->rho_in = v.rho_in;
  q->wgt = v.wgt;
}

// Compensated butterfly reduction of (s, comp) and min of umin over a warp.
// u is never negative, so the order of its bit patterns as unsigned
// integers is the order of the values: one warp-wide integer min instead of
// five shuffle rounds.
__device__ __forceinline__ void warp_reduce_comp(float& s, float& comp, float& umin) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float so = __shfl_xor_sync(0xffffffffu, s, o);
    const float co = __shfl_xor_sync(0xffffffffu, comp, o);
    float t, e;
    two_sum(s, so, t, e);
    s = t;
    comp = comp + co + e;
  }
  umin = __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(umin)));
}

// Stores the finished weight factor cpv of record r (FP64, and as FP32
// mantissa and exponent for the deposit) in place of its numerator, and
// raises the channel exponents by the record's largest per-cell weight
// `bound`.  Returns the FP32 mantissa and exponent through cm_out / ce_out.
__device__ __forceinline__ void store_factor(const TiledArgs& A, int64_t r, double cpv, double bound, int fl,
                                             int* emax, float* cm_out = nullptr, int* ce_out = nullptr) {
  // Dolag renormalisation makes the record's deposits into W sum to the
  // numerator; the deterministic mode bounds its tile sums with it
  A.aux[r] = fabs(A.cp[r]);
  A.cp[r] = cpv;
  int ce = 0;
  const float cm = (float)frexp(cpv, &ce);
  A.cpm[r] = cm;
  A.cpe[r] = ce;
  if (cm_out) *cm_out = cm;
  if (ce_out) *ce_out = ce;
  if (fl) A.box[r].w = fl;
  int e;
  if (bound > 0.0 && bound < 1e300) {
    frexp(bound, &e);
    emax[A.pt.nq] = max(emax[A.pt.nq], e);
    for (int k = 0; k < A.pt.nq; ++k) {
      const double qa = fabs((double)A.qv[(int64_t)k * A.cap + r]);
      if (qa > 0.0 && qa < 1e300) {
        frexp(bound * qa, &e);
        emax[k] = max(emax[k], e);
      }
    }
  }
}

// Weight factor of a well-conditioned record from its compensated FP32 sum
// S + S_err, by the one thread that holds it (weight numerator / S,
// cic_2D.jl:187-188 and cic_3D.jl:168-169).
__device__ __forceinline__ void finish_scalar(const TiledArgs& A, int64_t r, float S, float S_err, double& c_gm,
                                              int* emax, float* cm = nullptr, int* ce = nullptr) {
  const double Sd = (double)S + (double)S_err;
  const double cpv = A.cp[r] / Sd;
  c_gm += A.aux[r] * Sd;
  store_factor(A, r, cpv, fabs(cpv), 0, emax, cm, ce);
}

// Ill-conditioned record (every pixel centre near or beyond the kernel edge,
// or a zero FP32 sum): the reference's FP64 arithmetic with the whole warp,
// as in the plain path, including its fallback when no centre is inside
// (cic_2D.jl:196-205, cic_3D.jl:175-184).
template <int DIMS, int KERN>
__device__ void finish_fp64_warp(const TiledArgs& A, int64_t r, int lane, double& c_gm, int* emax, double* x64) {
  const int4 bx = A.box[r];
  const int4 dm = A.dimv[r];
  const int njk = dm.y * dm.z;
  const int64_t F = (int64_t)dm.x * njk;
  PrepFP64 q;
  prep_bcast<DIMS>(A.pt, A.mp_re, dm.w, lane, &q);
  double s_w = 0.0, s_a = 0.0;
  long long n_d = 0, n_t = 0;
  for (int64_t f = lane; f < F; f += 32) {
    const int a = (int)(f / njk);
    const int rr = (int)(f - (int64_t)a * njk);
    const int b = rr / dm.z, c = rr - b * dm.z;
    double u, ar;
    cell_fp64<DIMS>(q, bx.x + a, bx.y + b, bx.z + c, &u, &ar);
    s_a += ar;
    n_t += 1;
    if (u <= 1.0) {
      s_w += shape_d<KERN>(A.kern, u) * q.knorm * ar;
      n_d += 1;
    }
  }
  s_w = warp_sum_d(s_w);
  s_a = warp_sum_d(s_a);
  n_d = warp_sum_ll(n_d);
  n_t = warp_sum_ll(n_t);
  if (lane == 0) {  // per-particle factors (the scalars of prep_bcast live on lane 0)
    const bool fallback = (s_w == 0.0);
    double wpp;
    if (fallback) {
      n_d = n_t;
      wpp = s_a != 0.0 ? (double)n_d / s_a : 1.0;
    } else {
      wpp = (double)n_d / s_w;
    }
    const double cpv = DIMS == 2 ? q.area / (double)n_d * wpp * q.wgt * q.col
                                 : q.vol / (double)n_d * wpp * q.wgt * A.mp.L;
    c_gm += q.rho_in / (A.mp.L * A.mp.L * A.mp.L) * (fallback ? s_a : s_w);
    store_factor(A, r, cpv, fabs(cpv) * (fallback ? 1.0 : q.knorm), kRecFP64 | (fallback ? kRecFallback : 0),
                 emax);
  }
  // the FP64 preparation the record's pairs carry (every lane holds it)
  x64[0] = q.x;
  x64[1] = q.y;
  x64[2] = DIMS == 2 ? q.hsml : q.z;
  x64[3] = DIMS == 2 ? q.h_inv : q.hsml;
}

// Tile-range of record r.
struct TileSpan {
  int tx0, ty0, tz0, nty, ntz, nt;
};
__device__ __forceinline__ TileSpan tile_span(const TiledArgs& A, int4 bx, int4 dm) {
  TileSpan t;
  t.tx0 = bx.x / A.tdim[0];
  t.ty0 = bx.y / A.tdim[1];
  t.tz0 = bx.z / A.tdim[2];
  const int tx1 = (bx.x + dm.x - 1) / A.tdim[0];
  const int ty1 = (bx.y + dm.y - 1) / A.tdim[1];
  const int tz1 = (bx.z + dm.z - 1) / A.tdim[2];
  t.nty = ty1 - t.ty0 + 1;
  t.ntz = tz1 - t.tz0 + 1;
  t.nt = (tx1 - t.tx0 + 1) * t.nty * t.ntz;
  return t;
}

// Narrows the footprint-local cell ranges [k0[d], k1[d]) of a (record, tile)
// intersection to the cells whose pixel centres can lie within the kernel
// support (offset at most h), with margins far above the FP32 rounding of
// the per-cell test u <= 1, which still decides each cell.  A sphere (disc)
// fills about a third (three quarters) of its footprint box, and a tile at
// the box's corner often misses it altogether.  Returns false when no cell
// of the intersection can be inside.  g = {x, y, z offsets from the
// footprint start, h}, FP32 record geometry (finite, h > 0).
template <int DIMS>
__device__ __forceinline__ void support_min2(const float* f, const int* k0, const int* k1, float* m2) {
#pragma unroll
  for (int d = 0; d < 3; ++d) {  // smallest squared centre offset per axis
    const float first = f[d] - (float)k0[d] - 0.5f, last = f[d] - (float)(k1[d] - 1) - 0.5f;
    m2[d] = (d >= DIMS || (last <= 0.0f && first >= 0.0f)) ? 0.0f : fminf(first * first, last * last);
  }
}

// Whether any cell of the intersection can be inside the support (the test
// of support_box without the narrowing: no square root).
template <int DIMS>
__device__ __forceinline__ bool support_hits(const float4 g, const int* k0, const int* k1) {
  const float f[3] = {g.x, g.y, g.z};
  float m2[3];
  support_min2<DIMS>(f, k0, k1, m2);
  return !((m2[0] + m2[1]) + m2[2] > g.w * g.w * (1.0f + 0x1p-10f));
}

template <int DIMS>
__device__ __forceinline__ bool support_box(const float4 g, int* k0, int* k1) {
  const float f[3] = {g.x, g.y, g.z};
  float m2[3];
  support_min2<DIMS>(f, k0, k1, m2);
  const float R2 = g.w * g.w * (1.0f + 0x1p-10f);
#pragma unroll
  for (int d = 0; d < DIMS; ++d) {
    float rem = R2;
#pragma unroll
    for (int j = 0; j < DIMS; ++j)
      if (j != d) rem -= m2[j];
    if (!(rem >= 0.0f)) return false;
    const float R = sqrtf(rem) * (1.0f + 0x1p-10f) + 0x1p-10f;
    const int lo = (int)ceilf(f[d] - 0.5f - R), hi = (int)floorf(f[d] - 0.5f + R);
    k0[d] = max(k0[d], lo);
    k1[d] = min(k1[d], hi + 1);
    if (k1[d] <= k0[d]) return false;
  }
  return true;
}

// Intersection of record box bx (sides dm) with the tile at (ox, oy, oz),
// footprint-local.
__device__ __forceinline__ void tile_cut(int4 bx, int4 dm, int ox, int oy, int oz, int tx, int ty, int tz,
                                         int* k0, int* k1) {
  k0[0] = max(0, ox - bx.x);
  k0[1] = max(0, oy - bx.y);
  k0[2] = max(0, oz - bx.z);
  k1[0] = min(dm.x, ox + tx - bx.x);
  k1[1] = min(dm.y, oy + ty - bx.y);
  k1[2] = min(dm.z, oz + tz - bx.z);
}

// x 2^k for |k| <= 2044 by two exact power-of-two factors (no ldexp call).
__device__ __forceinline__ double scale_pow2(double x, int k) {
  const int k1 = k / 2, k2 = k - k1;
  return x * __longlong_as_double((long long)(k1 + 1023) << 52) * __longlong_as_double((long long)(k2 + 1023) << 52);
}

// What every pair record of one record repeats (PairRec, tiled.cuh).
struct PairSrc {
  int4 bx, dm;      // footprint start {iMin, jMin, kMin, flags} and sides
  float4 g;         // geometry {x - iMin, y - jMin, z - kMin, h}
  float hinv;       // 1 / h, as the renormalisation pass forms it
  float cpm;        // FP32 record: factor mantissa
  int cpe;          // FP32 record: factor exponent; FP64 record: record index
  float tot;        // FP32 record: |numerator| * 2^-cpe
  uint4 q;          // quantities 0-3 (more channels: the record index in q.x)
  bool tight;       // FP32 record: only tiles and cells the support can reach
  bool x64;         // FP64 record: g and q hold its FP64 preparation (kPackX64)
};

// An FP64 record's source with its FP64 preparation in place of g and q.
__device__ __forceinline__ void set_x64(PairSrc& s, const double* v) {
  s.x64 = true;
  s.g = make_float4(__int_as_float(__double2loint(v[0])), __int_as_float(__double2hiint(v[0])),
                    __int_as_float(__double2loint(v[1])), __int_as_float(__double2hiint(v[1])));
  s.q = make_uint4((unsigned)__double2loint(v[2]), (unsigned)__double2hiint(v[2]), (unsigned)__double2loint(v[3]),
                   (unsigned)__double2hiint(v[3]));
}

// The source of record r's pair records, by the lane that finished it
// (cm, ce: its FP32 factor; FP64 records read their own from memory).
__device__ __forceinline__ PairSrc pair_src(const TiledArgs& A, int64_t r, bool tight, float cm, int ce) {
  PairSrc s;
  s.bx = A.box[r];
  s.dm = A.dimv[r];
  s.g = A.geo[r];
  s.hinv = 1.0f / s.g.w;
  s.tight = tight;
  s.x64 = false;
  s.cpm = cm;
  s.cpe = tight ? ce : (int)r;
  // |numerator| relative to 2^cpe (|cpm| S: within the FP32 range for every
  // FP32 record, whatever the units); FP64 records: read from aux
  s.tot = tight ? (float)scale_pow2(A.aux[r], -ce) : 0.0f;
  const int nq = A.pt.nq;
  float qv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  if (nq <= 4)
    for (int k = 0; k < nq; ++k) qv[k] = A.qv[(int64_t)k * A.cap + r];
  s.q = make_uint4(nq <= 4 ? __float_as_uint(qv[0]) : (unsigned)r, __float_as_uint(qv[1]), __float_as_uint(qv[2]),
                   __float_as_uint(qv[3]));
  return s;
}

// Writes the pair record of record `src` and the t-th tile of its span into
// the tile's slot range, unless `tight` (an FP32 record) and no pixel centre
// of their intersection can lie within the kernel support; an FP32 record's
// cell box is narrowed to the support's bounding box (support_box).  FP64
// records may take the fallback weights, which cover every footprint cell,
// so they keep every tile and cell; their records fill the slot range from
// its end.
template <int DIMS>
__device__ __forceinline__ void write_pair(const TiledArgs& A, const TileSpan& s, int t, const PairSrc& src) {
  const int ta = t / (s.nty * s.ntz), tb = (t / s.ntz) % s.nty, tc = t % s.ntz;
  const int ox = (s.tx0 + ta) * A.tdim[0], oy = (s.ty0 + tb) * A.tdim[1], oz = (s.tz0 + tc) * A.tdim[2];
  int k0[3], k1[3];
  tile_cut(src.bx, src.dm, ox, oy, oz, A.tdim[0], A.tdim[1], A.tdim[2], k0, k1);
  if (src.tight && !support_box<DIMS>(src.g, k0, k1)) return;
  const int64_t tile = ((int64_t)(s.tx0 + ta) * A.ntile[1] + (s.ty0 + tb)) * A.ntile[2] + (s.tz0 + tc);
  const int lbase = ((src.bx.x + k0[0] - ox) * A.tdim[1] + (src.bx.y + k0[1] - oy)) * A.tdim[2] +
                    (src.bx.z + k0[2] - oz);
  const unsigned pack = (unsigned)lbase | (unsigned)(k1[0] - k0[0] - 1) << 10 | (unsigned)(k1[1] - k0[1] - 1) << 15 |
                        (unsigned)(k1[2] - k0[2] - 1) << 20 | (src.tight ? 0u : (unsigned)kPackFP64) |
                        (src.x64 ? (unsigned)kPackX64 : 0u);
  const long long slot = src.tight ? A.tile_start[tile] + atomicAdd(&A.tile_fill[tile], 1)
                                   : A.tile_start[tile + 1] - 1 - atomicAdd(&A.tile_fill64[tile], 1);
  uint4* w = A.prec + slot * kPairRecWords;
  w[0] = make_uint4(__float_as_uint(src.g.x), __float_as_uint(src.g.y), __float_as_uint(src.g.z),
                    __float_as_uint(src.g.w));
  w[1] = make_uint4(__float_as_uint(src.hinv), __float_as_uint(src.cpm), (unsigned)src.cpe, pack);
  w[2] = make_uint4((unsigned)k0[0], (unsigned)k0[1], (unsigned)k0[2], __float_as_uint(src.tot));
  w[3] = src.q;
}

// Warp-wide channel maxima and sums before lane 0 flushes them.
__device__ __forceinline__ void flush_stats(const TiledArgs& A, int lane, int dims, double c_gm, int* emax) {
  c_gm = warp_sum_d(c_gm);
  for (int c = 0; c < A.pt.nq + 1; ++c) emax[c] = __reduce_max_sync(0xffffffffu, emax[c]);
  if (lane == 0) {
    if (dims == 3 && c_gm != 0.0) atomicAdd(&A.st->grid_mass, c_gm);
    for (int c = 0; c < A.pt.nq + 1; ++c)
      if (emax[c] != INT_MIN) atomicMax(&A.exps[c], emax[c]);
  }
}

__device__ __forceinline__ void src_store(uint4* d, const PairSrc& s) {
  d[0] = make_uint4((unsigned)s.bx.x, (unsigned)s.bx.y, (unsigned)s.bx.z, (s.tight ? 1u : 0u) | (s.x64 ? 2u : 0u));
  d[1] = make_uint4((unsigned)s.dm.x, (unsigned)s.dm.y, (unsigned)s.dm.z, (unsigned)s.dm.w);
  d[2] = make_uint4(__float_as_uint(s.g.x), __float_as_uint(s.g.y), __float_as_uint(s.g.z), __float_as_uint(s.g.w));
  d[3] = make_uint4(__float_as_uint(s.hinv), __float_as_uint(s.cpm), (unsigned)s.cpe, __float_as_uint(s.tot));
  d[4] = s.q;
}
__device__ __forceinline__ PairSrc src_load(const uint4* d) {
  PairSrc s;
  const uint4 a = d[0], b = d[1], g = d[2], f = d[3];
  s.bx = make_int4((int)a.x, (int)a.y, (int)a.z, 0);
  s.tight = (a.w & 1u) != 0;
  s.x64 = (a.w & 2u) != 0;
  s.dm = make_int4((int)b.x, (int)b.y, (int)b.z, (int)b.w);
  s.g = make_float4(__uint_as_float(g.x), __uint_as_float(g.y), __uint_as_float(g.z), __uint_as_float(g.w));
  s.hinv = __uint_as_float(f.x);
  s.cpm = __uint_as_float(f.y);
  s.cpe = (int)f.z;
  s.tot = __uint_as_float(f.w);
  s.q = d[4];
  return s;
}

// Pair records of a group of 32 records, lane j holding record j (`mine`)
// and having put its source into srcs[j].  The group's (record, tile) pairs
// are spread over the lanes, so a record with many tiles does not hold up
// the warp.
template <int DIMS>
__device__ __forceinline__ void fill_group(const TiledArgs& A, bool mine, int4 bx, int4 dm,
                                           const uint4 (*srcs)[5], int lane) {
  const unsigned full = 0xffffffffu;
  TileSpan sp = {0, 0, 0, 1, 1, 0};
  if (mine) sp = tile_span(A, bx, dm);
  int incl = sp.nt;  // inclusive scan of the tile counts
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(full, incl, 31);
  for (int base = 0; base < total; base += 32) {
    const int f = base + lane;
    int j = 0;  // first lane whose inclusive count exceeds f
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
      const int v = __shfl_sync(full, incl, j + step - 1);
      if (v <= f) j += step;
    }
    j = j < 31 ? j : 31;
    TileSpan s;
    s.tx0 = __shfl_sync(full, sp.tx0, j);
    s.ty0 = __shfl_sync(full, sp.ty0, j);
    s.tz0 = __shfl_sync(full, sp.tz0, j);
    s.nty = __shfl_sync(full, sp.nty, j);
    s.ntz = __shfl_sync(full, sp.ntz, j);
    const int first = __shfl_sync(full, incl - sp.nt, j);
    if (f < total) write_pair<DIMS>(A, s, f - first, src_load(srcs[j]));
  }
  __syncwarp();  // the sources' shared memory is reused by the next group's sums
}

// K3 body: the warp `wid` of `nw` takes groups of 32 consecutive records
// (those with a footprint of at most large_cells cells).  The warp sums each
// record's footprint together; lane j keeps record j's sum, and the 32 lanes
// then finish their records side by side, so the FP64 division (a small
// fraction of FP32 throughput on GB300) costs one warp instruction sequence
// per 32 records.  The warp then writes the group's pair records.
template <int DIMS, int KERN>
__device__ void norm_records(const TiledArgs& A, int64_t wid, int64_t nw, int lane, NormShared& sh) {
  const int nrec = *A.n_rec;
  const bool overflow = (A.st->flags & kFlagOverflow) != 0;
  double c_gm = 0.0;
  int emax[kMaxQ + 1];
  for (int c = 0; c <= A.pt.nq; ++c) emax[c] = INT_MIN;
  float2(*tab)[kNormTab] = sh.tabs[(threadIdx.x >> 5) & 7];  // one set per warp of a 256-thread CTA
  float2* plane = sh.w[(threadIdx.x >> 5) & 7].plane;
  uint4(*srcs)[5] = sh.w[(threadIdx.x >> 5) & 7].src;
  for (int64_t g0 = wid * 32; g0 < nrec; g0 += nw * 32) {
    const int cnt = nrec - g0 < 32 ? (int)(nrec - g0) : 32;
    float my_s = 0.0f, my_c = 0.0f, my_u = 0.0f;
    bool mine = false;
    for (int j = 0; j < cnt; ++j) {
      const int4 dm = A.dimv[g0 + j];
      const int64_t F = (int64_t)dm.x * dm.y * dm.z;
      if (F > A.large_cells) continue;  // two-phase path (k_large_partials)
      float s = 0.0f, comp = 0.0f, umin = 3.0e38f;
      if (dm.x <= kNormTab && dm.y <= kNormTab && dm.z <= kNormTab) {
        const float4 g = A.geo[g0 + j];
        // a run-time kernel shape is dispatched once per record, so the
        // cell loop evaluates a compile-time shape
        if (KERN >= 0) record_sum_tab<DIMS, KERN>(A.kern, g, dm, lane, tab, plane, s, comp, umin);
        else if (A.kern == 0) record_sum_tab<DIMS, 0>(0, g, dm, lane, tab, plane, s, comp, umin);
        else if (A.kern == 1) record_sum_tab<DIMS, 1>(1, g, dm, lane, tab, plane, s, comp, umin);
        else if (A.kern == 2) record_sum_tab<DIMS, 2>(2, g, dm, lane, tab, plane, s, comp, umin);
        else if (A.kern == 3) record_sum_tab<DIMS, 3>(3, g, dm, lane, tab, plane, s, comp, umin);
        else record_sum_tab<DIMS, 4>(4, g, dm, lane, tab, plane, s, comp, umin);
      } else {
        record_sum_fp32<DIMS, KERN>(A.kern, A.geo[g0 + j], dm, 0, F, lane, 32, s, comp, umin);
      }
      warp_reduce_comp(s, comp, umin);
      if (lane == j) {
        my_s = s;
        my_c = comp;
        my_u = umin;
        mine = true;
      }
    }
    const int64_t r = g0 + lane;
    const bool ill = mine && ill_conditioned(my_s, my_u);
    double my64[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned m = __ballot_sync(0xffffffffu, ill); m; m &= m - 1) {
      const int j = __ffs(m) - 1;
      double v[4];
      finish_fp64_warp<DIMS, KERN>(A, g0 + j, lane, c_gm, emax, v);
      if (lane == j)
        for (int k = 0; k < 4; ++k) my64[k] = v[k];
    }
    float cm = 0.0f;
    int ce = 0;
    if (mine && !ill) finish_scalar(A, r, my_s, my_c, c_gm, emax, &cm, &ce);
    __syncwarp();  // lane 0's FP64 finishes are read by the records' own lanes
    if (!overflow) {
      int4 bx = make_int4(0, 0, 0, 0), dm = bx;
      if (mine) {
        PairSrc src = pair_src(A, r, !ill, cm, ce);
        if (ill) set_x64(src, my64);
        bx = src.bx;
        dm = src.dm;
        src_store(srcs[lane], src);
      }
      __syncwarp();
      fill_group<DIMS>(A, mine, bx, dm, srcs, lane);
    }
  }
  flush_stats(A, lane, DIMS, c_gm, emax);
}

// K3: one warp per group of 32 small records.
template <int DIMS, int KERN>
__global__ void __launch_bounds__(256, 4) k_norm_fill(TiledArgs A) {
  __shared__ NormShared sh;
  norm_records<DIMS, KERN>(A, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                           ((int64_t)gridDim.x * blockDim.x) >> 5, threadIdx.x & 31, sh);
}

// K3L phase 1: every CTA takes chunks of kChunkCells cells of the large
// records (a persistent loop over the chunk list) and writes the chunk's
// compensated partial sum and smallest u.
template <int DIMS, int KERN>
__device__ void large_partials(const TiledArgs& A, int64_t bid, int64_t nblocks, float (*red)[8]) {
  const int nl = *A.n_large;
  const long long total = A.large_start[nl];
  const bool overflow = (A.st->flags & kFlagOverflow) != 0;
  if (overflow) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (long long w = bid; w < total; w += nblocks) {
    int lo = 0, hi = nl - 1;  // record whose chunk range holds w
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (A.large_start[mid] <= w) lo = mid;
      else hi = mid - 1;
    }
    const int64_t r = A.large[lo];
    const int4 dm = A.dimv[r];
    const int64_t F = (int64_t)dm.x * dm.y * dm.z;
    const int64_t f0 = (w - A.large_start[lo]) * kChunkCells;
    const int64_t f1 = f0 + kChunkCells < F ? f0 + kChunkCells : F;
    float s = 0.0f, comp = 0.0f, umin = 3.0e38f;
    record_sum_fp32<DIMS, KERN>(A.kern, A.geo[r], dm, f0, f1, threadIdx.x, blockDim.x, s, comp, umin);
    warp_reduce_comp(s, comp, umin);
    if (lane == 0) {
      red[0][warp] = s;
      red[1][warp] = comp;
      red[2][warp] = umin;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      float S = red[0][0], C = red[1][0], U = red[2][0];
      for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
        float t, e;
        two_sum(S, red[0][k], t, e);
        S = t;
        C = C + red[1][k] + e;
        U = fminf(U, red[2][k]);
      }
      A.partials[w] = make_float4(S, C, U, 0.0f);
    }
    __syncthreads();
  }
}

template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) k_large_partials(TiledArgs A) {
  __shared__ float red[3][8];
  large_partials<DIMS, KERN>(A, blockIdx.x, gridDim.x, red);
}

// K3L phase 2: one warp per large record sums its chunk partials in a fixed
// order and finishes the record.
template <int DIMS, int KERN>
__device__ void large_finish(const TiledArgs& A, int64_t wid, int64_t nw, int lane) {
  const int nl = *A.n_large;
  const bool overflow = (A.st->flags & kFlagOverflow) != 0;
  double c_gm = 0.0;
  int emax[kMaxQ + 1];
  for (int c = 0; c <= A.pt.nq; ++c) emax[c] = INT_MIN;
  if (!overflow) {
    for (int64_t i = wid; i < nl; i += nw) {
      const int64_t r = A.large[i];
      float s = 0.0f, comp = 0.0f, umin = 3.0e38f;
      for (long long w = A.large_start[i] + lane; w < A.large_start[i + 1]; w += 32) {
        const float4 pv = A.partials[w];
        float t, e;
        two_sum(s, pv.x, t, e);
        s = t;
        comp = comp + pv.y + e;
        umin = fminf(umin, pv.z);
      }
      warp_reduce_comp(s, comp, umin);
      const bool ill = ill_conditioned(s, umin);
      double v[4];
      if (ill) finish_fp64_warp<DIMS, KERN>(A, r, lane, c_gm, emax, v);
      else if (lane == 0) finish_scalar(A, r, s, comp, c_gm, emax);
      __syncwarp();  // lane 0 wrote the factor
      const bool tight = (A.box[r].w & kRecFP64) == 0;
      PairSrc src = pair_src(A, r, tight, A.cpm[r], A.cpe[r]);
      if (ill) set_x64(src, v);
      const TileSpan sp = tile_span(A, src.bx, src.dm);
      for (int t = lane; t < sp.nt; t += 32) write_pair<DIMS>(A, sp, t, src);
    }
  }
  flush_stats(A, lane, DIMS, c_gm, emax);
}

template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) k_large_finish(TiledArgs A) {
  large_finish<DIMS, KERN>(A, ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                           ((int64_t)gridDim.x * blockDim.x) >> 5, threadIdx.x & 31);
}

// v rounded to the nearest int64 (|v| < 2^62) with 32-bit conversions:
// below 2^31 one rounding conversion; above, v is an integer (24 significant
// bits) and splits exactly into h 2^31 + r.  Cheaper than the 64-bit
// conversion where a cell takes many channels (2D), dearer with two (3D).
__device__ __forceinline__ long long float_to_ll_split(float v) {
  if (fabsf(v) < 0x1p31f) return (long long)__float2int_rn(v);
  const int h = __float2int_rz(v * 0x1p-31f);
  return (long long)h * 2147483648LL + (long long)__float2int_rz(fmaf(-(float)h, 0x1p31f, v));
}

// Tiles (or chunks of split tiles) of at most this many pairs accumulate the
// deterministic mode's fixed point as three 21-bit chunks: a cell takes at
// most one value per pair, each chunk of a value is at most 2^20 in
// magnitude, so no 32-bit chunk sum can overflow.
constexpr int kChunkPairs = 2047;

// v (|v| < 2^62) rounded to the nearest integer x = x2 2^42 + x1 2^21 + x0,
// |xk| <= 2^20, by FP32 additions alone: a float of magnitude below
// 2^(22+k) added to 1.5 2^(23+k) leaves round(v / 2^k) in the sum's low
// mantissa bits (its ulp is 2^k), and each remainder is exact.  The sum of
// the three parts is round(v) with ties to even, as a 64-bit conversion
// rounds, since x2 2^42 + x1 2^21 is even.
__device__ __forceinline__ void fixed_chunks(float v, int& x0, int& x1, int& x2) {
  const float C42 = 0x1.8p65f, C21 = 0x1.8p44f, C0 = 0x1.8p23f;
  const float t2 = v + C42;
  const float r1 = v - (t2 - C42);
  const float t1 = r1 + C21;
  const float r0 = r1 - (t1 - C21);
  const float t0 = r0 + C0;
  x2 = __float_as_int(t2) - __float_as_int(C42);
  x1 = __float_as_int(t1) - __float_as_int(C21);
  x0 = __float_as_int(t0) - __float_as_int(C0);
}

// Adds one cell value to a tile accumulator (see k_deposit).  DET: an exact
// int64 fixed-point sum.  Shared-memory atomics on 32-bit integers are single
// native instructions, while 64-bit and FP32 ones are compiled to load /
// compare-and-swap loops.  With c2 (a tile of at most kChunkPairs pairs) the
// value's three chunks go into the planes hi, lo and c2 as signed 32-bit
// sums, three reductions that return nothing; otherwise the low and high
// words go into hi and lo, the low word's add returning its old value, from
// which the carry into the high word follows.  Both add exactly whatever the
// order of the additions.
template <bool DET, bool SPLIT = false>
__device__ __forceinline__ void acc_cell(float* hi, float* lo, int* c2, int i, float v) {
  if (DET) {
    if (c2) {
      int x0, x1, x2;
      fixed_chunks(v, x0, x1, x2);
      atomicAdd((int*)hi + i, x0);
      atomicAdd((int*)lo + i, x1);
      atomicAdd(c2 + i, x2);
    } else {
      const unsigned long long x = (unsigned long long)(SPLIT ? float_to_ll_split(v) : __float2ll_rn(v));
      const unsigned xl = (unsigned)x;
      const unsigned old = atomicAdd((unsigned*)hi + i, xl);
      const unsigned xh = (unsigned)(x >> 32) + (old + xl < old ? 1u : 0u);
      if (xh != 0u) atomicAdd((unsigned*)lo + i, xh);
    }
  } else {
    acc_twosum(&hi[i], &lo[i], v);
  }
}

// The exact int64 value of a DET accumulator cell.
__device__ __forceinline__ long long fixed_value(const float* hi, const float* lo, const int* c2, int i) {
  if (c2)
    return (long long)c2[i] * (1LL << 42) + (long long)((const int*)lo)[i] * (1LL << 21) + ((const int*)hi)[i];
  return (long long)(((unsigned long long)((const unsigned*)lo)[i] << 32) | ((const unsigned*)hi)[i]);
}

template <bool DET>
__device__ __forceinline__ double cell_value(const float* hi, const float* lo, const int* c2, int i) {
  if (DET) return (double)fixed_value(hi, lo, c2, i);
  return (double)hi[i] + (double)lo[i];
}

// K4: one CTA per image tile.  DET selects exact int64 fixed-point tile sums
// (bitwise reproducible) instead of TwoSum-compensated FP32 (hi, lo) pairs;
// both use 8 bytes per channel and tile pixel.

// Deposit of one FP64 pair (an ill-conditioned record, its pair record's
// words m = w[1], o = w[2]): per-cell weights in the reference's FP64
// arithmetic over the pair's whole cell box, lane-strided.  Out of line: its
// FP64 state stays out of the register budget of the FP32 pair loop.
template <int DIMS, int KERN, int TY, int TZ, bool DET>
__device__ __noinline__ void deposit_pair_fp64(const TiledArgs& A, const uint4* R, int nq, int TV,
                                               float* hi, float* lo, int* c2, const double* s_scale,
                                               int lane) {
  const uint4 m = R[1], o = R[2];
  const int r = (int)m.z;
  const unsigned pack = m.w;
  const int na = (int)((pack >> 10) & 31u) + 1, nb = (int)((pack >> 15) & 31u) + 1, nc = (int)((pack >> 20) & 31u) + 1;
  const int lbase = (int)(pack & 1023u);
  const int n = na * nb * nc;
  const int4 bx = A.box[r];
  const int4 dm = A.dimv[r];
  PrepFP64 q;
  if (pack & (unsigned)kPackX64) {
    // the renormalisation pass's FP64 preparation; 1/hsml and the kernel
    // normalisation as prep_particle_fp64 forms them
    const uint4 g = R[0], q4 = R[3];
    q.x = __hiloint2double((int)g.y, (int)g.x);
    q.y = __hiloint2double((int)g.w, (int)g.z);
    const double a = __hiloint2double((int)q4.y, (int)q4.x), b = __hiloint2double((int)q4.w, (int)q4.z);
    q.z = DIMS == 2 ? 0.0 : a;
    q.hsml = DIMS == 2 ? a : b;
    q.h_inv = DIMS == 2 ? b : 1.0 / q.hsml;
    const double hd = A.mp_re.kernel_dim == 2 ? q.h_inv * q.h_inv : q.h_inv * q.h_inv * q.h_inv;
    q.knorm = A.mp_re.sigma * hd;
  } else {
    prep_bcast<DIMS>(A.pt, A.mp_re, dm.w, lane, &q);
  }
  const bool fb = (bx.w & kRecFallback) != 0;
  const double cpv = A.cp[r];
  const double scw = s_scale[nq];
  const float inv_nc = inv_small(nc), inv_nb = inv_small(nb);
  for (int e = lane; e < n; e += 32) {
    const int bc = fdiv(e, inv_nc);
    const int c = e - bc * nc;
    const int a = fdiv(bc, inv_nb);
    const int b = bc - a * nb;
    double u, ar;
    cell_fp64<DIMS>(q, bx.x + (int)o.x + a, bx.y + (int)o.y + b, bx.z + (int)o.z + c, &u, &ar);
    const double wk = fb ? 1.0 : (u <= 1.0 ? shape_d<KERN>(A.kern, u) * q.knorm : 0.0);
    const double pw = wk * ar * cpv;
    if (pw != 0.0) {
      const int li = lbase + (a * TY + b) * TZ + c;
      acc_cell<DET, DIMS == 2>(hi, lo, c2, nq * TV + li, __double2float_rn(pw * scw));
      for (int k = 0; k < nq; ++k)
        acc_cell<DET, DIMS == 2>(hi, lo, c2, k * TV + li,
                                 __double2float_rn(pw * s_scale[k] * (double)A.qv[(int64_t)k * A.cap + r]));
    }
  }
}

// Pair records per bulk copy into a warp's staging buffer (1 KB).
constexpr int kStage = 16;
// Bound on the polls of a bulk copy's completion (each poll may suspend the
// thread for a while in hardware); a copy of 1 KB completes in microseconds.
constexpr int kSpinLimit = 1 << 22;

// Per-CTA scratch of the tile deposit besides the accumulators: one
// instance per kernel, shared by every specialisation the kernel inlines.
struct DepositShared {
  double scale[kMaxQ + 1];  // 2^shift per channel
  double unscale[kMaxQ + 1];  // 2^-shift per channel, for the flush (exact)
  int shift[kMaxQ + 1];
  double bnd[kMaxQ + 1][8];  // deterministic mode: per-warp tile bounds
  float2 tabs[8][3][32];     // per-warp axis tables of the current pair
  uint4 small[8][16][4];     // per-warp constants of the packed small pairs (deposit_small)
  uint4 stage[8][2][kStage * kPairRecWords];  // per-warp double buffer of pair records
  unsigned long long bar[8][2];               // mbarriers of the staging buffers
  unsigned phase[8];         // per warp: bit b, the parity buffer b's barrier waits for next
  int last;                  // split tile: this CTA finished it
};

// Bulk copies (the non-tensor TMA path) into shared memory, completed on an
// mbarrier that counts the bytes.
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// Orders this thread's earlier shared-memory accesses (generic proxy: data
// reads, mbarrier initialisation) before later bulk copies and their
// completions (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// `bytes` a multiple of 16, both addresses 16-byte aligned.
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// The whole warp waits for the phase of parity `parity` to complete; false
// when it has not after `limit` polls (warp-uniform).
__device__ __forceinline__ bool mbar_wait_warp(unsigned long long* bar, unsigned parity, int limit = kSpinLimit) {
  for (int it = 0; it < limit; ++it)
    if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
  return false;
}

// Once per CTA, before its first tile: each warp's lane 0 initialises the
// warp's two staging barriers, which then live for the CTA (a barrier that
// bulk copies have completed on is not initialised again).
__device__ __forceinline__ void deposit_init(DepositShared& sh) {
  const int warp = (threadIdx.x >> 5) & 7;
  if ((threadIdx.x & 31) == 0) {
    mbar_init(&sh.bar[warp][0], 1);
    mbar_init(&sh.bar[warp][1], 1);
    sh.phase[warp] = 0;
    fence_proxy_async_smem();  // the initialised barriers, as the bulk copies see them
    fence_mbar_init();
  }
  __syncwarp();
}

// Writes one output pixel (i, j, k) from its W and channel values q(c) in
// the output's layout (raw accumulator, 3D reduced or 2D reduced).
template <int DIMS, class QFn>
__device__ __forceinline__ void store_cell(const TiledArgs& A, int64_t P, int64_t PD, int i, int j, int k, int nq,
                                           double W, QFn q) {
  if (A.mode == 1) {  // raw (P^D, nq+1) accumulator
    const int64_t row = DIMS == 2 ? (int64_t)i * P + j : ((int64_t)i * P + j) * P + k;
    A.out[row + (int64_t)nq * PD] = W;
    for (int c = 0; c < nq; ++c) A.out[row + c * PD] = q(c);
  } else if (DIMS == 3) {
    // reduce_image_3D divides wherever Q > 0 (reduce_image.jl:49-51); a
    // weight sum that vanished in the tile accumulator (below the
    // deterministic mode's fixed-point quantum, or FP32 underflow) leaves
    // the cell empty rather than infinite
    double Q = q(0);
    if (Q > 0.0 && !A.w_is_one) Q = W > 0.0 ? Q / W : 0.0;
    A.out[((int64_t)i * P + j) * P + k] = Q;
  } else {
    for (int c = 0; c < nq; ++c) {
      double Q = q(c);
      if (A.reduce && W > 0.0) Q /= W;
      A.out[(int64_t)i + P * j + PD * c] = Q;
    }
  }
}

// Tile cell v of the flush walk: its tile-local index li and pixel (i, j, k).
// The reduced 2D output is x-fastest, so that walk is x-fastest.
template <int DIMS, int TX, int TY, int TZ>
__device__ __forceinline__ void flush_cell(const TiledArgs& A, int v, int ox, int oy, int oz, bool xfast, int& li,
                                           int& i, int& j, int& k) {
  if (DIMS == 2 && xfast) {
    const int ix = v % TX, iy = v / TX;
    li = ix * TY + iy;
    i = ox + ix;
    j = oy + iy;
    k = 0;
  } else {
    li = v;
    i = ox + v / (TY * TZ);
    j = oy + (v / TZ) % TY;
    k = oz + v % TZ;
  }
}

// FP32 factor of a channel of quantity q for a record of factor
// cpm 2^cpe: cpm q 2^(cpe + shift), with q split into mantissa and exponent
// so no intermediate leaves the FP32 range (each factor is at most 2^62 / S
// of its channel's scale).
__device__ __forceinline__ float channel_factor(float q, float cpm, int cpe, int shift) {
  float qm;
  int qe;
  split_f(q, qm, qe);
  return (cpm * qm) * pow2f(cpe + qe + shift);
}

// One cell (a, b, c) of a pair's box.
template <int DIMS, int KERN, int NQ, int TY, int TZ, bool DET>
__device__ __forceinline__ void deposit_cell(const float2 (*tab)[32], int a, int b, int c, int lbase, float hinv,
                                             float cw, const float* cq, int nq, int TV, float* hi, float* lo,
                                             int* c2) {
  // 2D: the z term is the constant {0, 1} (the same u and weight as the
  // renormalisation pass forms)
  {
    const float2 ex = tab[0][a], ey = tab[1][b], ez = DIMS == 3 ? tab[2][c] : make_float2(0.0f, 1.0f);
    const float u = u_of((ex.x + ey.x) + ez.x, hinv);
    if (u <= 1.0f) {
      const float gw = kshape_f<KERN>(u) * (ex.y * ey.y * ez.y);
      const int li = lbase + (a * TY + b) * TZ + c;
      acc_cell<DET, DIMS == 2>(hi, lo, c2, nq * TV + li, gw * cw);
#pragma unroll
      for (int k = 0; k < (NQ > 0 ? NQ : kMaxQ); ++k) {
        if (NQ == 0 && k >= nq) break;
        acc_cell<DET, DIMS == 2>(hi, lo, c2, k * TV + li, gw * cq[k]);
      }
    }
  }
}

// The cells of one (record, tile) pair: the intersection's n = na nb nc
// cells, lane-strided, from the per-axis tables.  KERN is a compile-time
// shape here.
template <int DIMS, int KERN, int NQ, int TY, int TZ, bool DET>
__device__ __forceinline__ void deposit_cells(const float2 (*tab)[32], int n, int nb, int nc, int lbase, float hinv,
                                              float cw, const float* cq, int nq, int TV, float* hi, float* lo,
                                              int* c2, int lane) {
  const float inv_nc = inv_small(nc), inv_nb = inv_small(nb);
  for (int e = lane; e < n; e += 32) {
    const int bc = DIMS == 3 ? fdiv(e, inv_nc) : e;  // 2D: nc == 1
    const int cc = DIMS == 3 ? e - bc * nc : 0;
    const int ca = fdiv(bc, inv_nb);
    const int cb = bc - ca * nb;
    deposit_cell<DIMS, KERN, NQ, TY, TZ, DET>(tab, ca, cb, cc, lbase, hinv, cw, cq, nq, TV, hi, lo, c2);
  }
}

// One FP32 pair from its staged record R (PairRec): per-axis tables of its
// cell box, then its cells.  Uniform across the warp.
template <int DIMS, int KERN, int NQ, int TY, int TZ, bool DET>
__device__ __forceinline__ void deposit_pair32(const TiledArgs& A, const uint4* R, int nq, int TV, const int* s_shift,
                                               float2 (*tab)[32], float* hi, float* lo, int* c2,
                                               int lane) {
  const uint4 g = R[0], m = R[1], o = R[2];
  const unsigned pack = m.w;
  const int na = (int)((pack >> 10) & 31u) + 1, nb = (int)((pack >> 15) & 31u) + 1;
  const int nc = DIMS == 3 ? (int)((pack >> 20) & 31u) + 1 : 1;
  const int lbase = (int)(pack & 1023u);
  const float h = __uint_as_float(g.w), hinv = __uint_as_float(m.x), cpm = __uint_as_float(m.y);
  const int cpe = (int)m.z;
  const float cw = cpm * pow2f(cpe + s_shift[nq]);
  float cq[NQ > 0 ? NQ : kMaxQ];
  {
    const uint4 q4 = R[3];
    const unsigned qa[4] = {q4.x, q4.y, q4.z, q4.w};
    if (NQ > 0 && NQ <= 4) {
#pragma unroll
      for (int k = 0; k < (NQ > 0 && NQ <= 4 ? NQ : 1); ++k)
        cq[k] = channel_factor(__uint_as_float(qa[k]), cpm, cpe, s_shift[k]);
    } else {  // channel count known at run time: up to four in the record, more by record index
      for (int k = 0; k < nq; ++k)
        cq[k] = channel_factor(nq <= 4 ? __uint_as_float(qa[k & 3]) : A.qv[(int64_t)k * A.cap + (int)q4.x], cpm,
                               cpe, s_shift[k]);
    }
  }
  for (int i = lane; i < na + nb + nc; i += 32) {  // separable per-axis terms; axis by selects
    const int ax = i < na ? 0 : (i < na + nb ? 1 : 2);
    const int k = i - (ax == 0 ? 0 : (ax == 1 ? na : na + nb));
    const int c = k + (int)(ax == 0 ? o.x : (ax == 1 ? o.y : o.z));
    tab[ax][k] = (DIMS == 2 && ax == 2)
                     ? make_float2(0.0f, 1.0f)
                     : axis_sq(__uint_as_float(ax == 0 ? g.x : (ax == 1 ? g.y : g.z)), h, c);
  }
  __syncwarp();
  const int n = na * nb * nc;
  // a run-time kernel shape is dispatched once per pair, so the cell loop
  // evaluates a compile-time shape
#define SPHG_CELLS(K) \
  deposit_cells<DIMS, K, NQ, TY, TZ, DET>(tab, n, nb, nc, lbase, hinv, cw, cq, nq, TV, hi, lo, c2, lane)
  if (KERN >= 0) SPHG_CELLS(KERN >= 0 ? KERN : 0);
  else if (A.kern == 0) SPHG_CELLS(0);
  else if (A.kern == 1) SPHG_CELLS(1);
  else if (A.kern == 2) SPHG_CELLS(2);
  else if (A.kern == 3) SPHG_CELLS(3);
  else SPHG_CELLS(4);
#undef SPHG_CELLS
  __syncwarp();  // the tables are refilled for the next pair
}

// Pairs of at most this many cells are deposited packed (64: measured best
// of 32, 64 and 128 on the 3D and batched workloads): the small pairs of
// a staged chunk share the warp's iterations, lanes taking consecutive cells
// across them, instead of one pair (and its axis tables) per iteration.
constexpr int kSmallCells = 64;

// The per-pair constants of a packed small pair, prepared by its lane
// (four uint4): {fx, fy, fz, h}, {1/h, cw, a0, b0}, {c0, pack, inv_nc,
// inv_nbc}, {cq[0..3]} -- the channel factors with this tile's shifts.
template <int DIMS, int NQ>
__device__ __forceinline__ void small_header(const uint4* R, const int* s_shift, int nq, uint4* H) {
  const uint4 g = R[0], m = R[1], o = R[2], q4 = R[3];
  const unsigned pack = m.w;
  const int nb = (int)((pack >> 15) & 31u) + 1;
  const int nc = DIMS == 3 ? (int)((pack >> 20) & 31u) + 1 : 1;
  const float cpm = __uint_as_float(m.y);
  const int cpe = (int)m.z;
  const float cw = cpm * pow2f(cpe + s_shift[nq]);
  const unsigned qa[4] = {q4.x, q4.y, q4.z, q4.w};
  float cq[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < (NQ > 0 && NQ <= 4 ? NQ : 1); ++k) cq[k] = channel_factor(__uint_as_float(qa[k]), cpm, cpe, s_shift[k]);
  H[0] = g;
  H[1] = make_uint4(m.x, __float_as_uint(cw), o.x, o.y);
  H[2] = make_uint4(o.z, pack, __float_as_uint(inv_small(nc)), __float_as_uint(inv_small(nb * nc)));
  H[3] = make_uint4(__float_as_uint(cq[0]), __float_as_uint(cq[1]), __float_as_uint(cq[2]), __float_as_uint(cq[3]));
}

// The small pairs of a staged chunk (lanes set in smask; lane j holds pair
// j's cell count nj), packed: cell t of the concatenation belongs to the
// first pair whose inclusive count exceeds t.  Per cell the axis terms are
// formed directly with axis_sq, the same operations the tables hold, so u
// and the weight equal those of the renormalisation pass.  Cells of two
// pairs may meet in one step; the accumulation is atomic.
template <int DIMS, int KERN, int NQ, int TY, int TZ, bool DET>
__device__ __forceinline__ void deposit_small(const uint4* R, unsigned smask, int nj, const int* s_shift, int nq,
                                              int TV, uint4 (*hdr)[4], float* hi, float* lo, int* c2,
                                              int lane) {
  const unsigned full = 0xffffffffu;
  const bool mine = (smask >> lane) & 1u;
  if (mine) small_header<DIMS, NQ>(R + lane * kPairRecWords, s_shift, nq, hdr[lane]);
  int incl = mine ? nj : 0;  // inclusive scan of the small pairs' cell counts
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(full, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(full, incl, 31);
  __syncwarp();
  for (int base = 0; base < total; base += 32) {
    const int t = base + lane;
    int j = 0;  // the first pair (lane) whose inclusive count exceeds t
#pragma unroll
    for (int step = 8; step > 0; step >>= 1) {
      const int v = __shfl_sync(full, incl, j + step - 1);
      if (v <= t) j += step;
    }
    const int start = __shfl_sync(full, incl - (mine ? nj : 0), j);
    if (t >= total) continue;
    const uint4 g = hdr[j][0], h1 = hdr[j][1], h2 = hdr[j][2];
    const int e = t - start;
    const int bc = DIMS == 3 ? fdiv(e, __uint_as_float(h2.z)) : e;
    const int c = DIMS == 3 ? e - bc * (int)(((h2.y >> 20) & 31u) + 1) : 0;
    const int nb = (int)((h2.y >> 15) & 31u) + 1;
    const int a = fdiv(e, __uint_as_float(h2.w));
    const int b = bc - a * nb;
    const float h = __uint_as_float(g.w);
    const float2 ex = axis_sq(__uint_as_float(g.x), h, (int)h1.z + a);
    const float2 ey = axis_sq(__uint_as_float(g.y), h, (int)h1.w + b);
    const float2 ez = DIMS == 3 ? axis_sq(__uint_as_float(g.z), h, (int)h2.x + c) : make_float2(0.0f, 1.0f);
    const float u = u_of((ex.x + ey.x) + ez.x, __uint_as_float(h1.x));
    if (u <= 1.0f) {
      const float gw = kshape_f<KERN>(u) * (ex.y * ey.y * ez.y);
      const int li = (int)(h2.y & 1023u) + (a * TY + b) * TZ + c;
      acc_cell<DET, DIMS == 2>(hi, lo, c2, nq * TV + li, gw * __uint_as_float(h1.y));
      const uint4 q4 = hdr[j][3];
      const float cq[4] = {__uint_as_float(q4.x), __uint_as_float(q4.y), __uint_as_float(q4.z), __uint_as_float(q4.w)};
#pragma unroll
      for (int k = 0; k < (NQ > 0 && NQ <= 4 ? NQ : 1); ++k) acc_cell<DET, DIMS == 2>(hi, lo, c2, k * TV + li, gw * cq[k]);
    }
  }
  __syncwarp();  // the headers are rewritten for the next chunk
}

template <int DIMS, int KERN, int NQ, int TX, int TY, int TZ, bool DET>
__device__ void deposit_tile(const TiledArgs& A, int64_t t, unsigned char* smem_raw, DepositShared& sh,
                             int chunk = 0) {
  constexpr int TV = TX * TY * TZ;
  const int nq = NQ > 0 ? NQ : A.pt.nq;
  const int nch = nq + 1;
  // FP32C: hi [nch][TV], lo [nch][TV]; DET: three planes [nch][TV] (see
  // acc_cell), the third used when the tile has at most kChunkPairs pairs
  float* hi = (float*)smem_raw;
  float* lo = hi + nch * TV;
  const int tz = (int)(t % A.ntile[2]);
  const int ty = (int)((t / A.ntile[2]) % A.ntile[1]);
  const int tx = (int)(t / ((int64_t)A.ntile[2] * A.ntile[1]));
  const int ox = tx * TX, oy = ty * TY, oz = tz * TZ;
  for (int v = threadIdx.x; v < (DET ? 3 : 2) * nch * TV; v += blockDim.x) hi[v] = 0.0f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  // after an overflow of the pair list the lists are incomplete: deposit
  // nothing (the host grows the list and maps again); nor after a staging
  // copy timed out (the call fails)
  // (read from L2: a timeout raised by an earlier tile of this CTA must be seen)
  const bool overflow = (__ldcg(&A.st->flags) & (kFlagOverflow | kFlagTimeout)) != 0;
  // the tile's slots hold the pairs the renormalisation pass kept: FP32
  // pairs from the start, FP64 pairs from the end
  const long long p0 = A.tile_start[t], pe = A.tile_start[t + 1];
  const int n32 = overflow ? 0 : A.tile_fill[t], n64 = overflow ? 0 : A.tile_fill64[t];
  const uint4* rec32 = A.prec + p0 * kPairRecWords;
  const uint4* rec64 = A.prec + (pe - n64) * kPairRecWords;
  const bool split = A.split > 1;
  // this CTA's pairs: all of the tile's, or its chunk of each kind
  const int f0 = split ? (int)((long long)n32 * chunk / A.split) : 0;
  const int f1 = split ? (int)((long long)n32 * (chunk + 1) / A.split) : n32;
  const int d0 = split ? (int)((long long)n64 * chunk / A.split) : 0;
  const int d1 = split ? (int)((long long)n64 * (chunk + 1) / A.split) : n64;
  int* const c2 = (DET && (f1 - f0) + (d1 - d0) <= kChunkPairs) ? (int*)(lo + nch * TV) : nullptr;
  // channel scales (powers of two): 2^s_shift as double for the flush
  double* s_scale = sh.scale;
  double* s_unscale = sh.unscale;
  int* s_shift = sh.shift;
  if (DET) {
    // this tile's bound per channel: the sum over its pairs of the record's
    // whole deposit (|numerator| * |q|), so every partial sum of the tile
    // stays below 2^62 in int64 fixed point
    double(*s_bnd)[8] = sh.bnd;
    double bnd[kMaxQ + 1];
    for (int c = 0; c < nch; ++c) bnd[c] = 0.0;
    for (int s = threadIdx.x; s < n32 + n64; s += blockDim.x) {
      const uint4* R = s < n32 ? rec32 + (int64_t)s * kPairRecWords : rec64 + (int64_t)(s - n32) * kPairRecWords;
      const uint4 m = R[1];
      const uint4 q4 = R[3];
      const unsigned qa[4] = {q4.x, q4.y, q4.z, q4.w};
      const bool p64 = (m.w & (unsigned)kPackFP64) != 0;
      const int r = p64 ? (int)m.z : (int)q4.x;  // the record index, where the record holds it
      const double tot = p64 ? A.aux[r] : scale_pow2((double)__uint_as_float(R[2].w), (int)m.z);
      bnd[nq] += tot;
      for (int k = 0; k < nq; ++k) {
        const float qk = (!p64 && nq <= 4) ? __uint_as_float(qa[k & 3]) : A.qv[(int64_t)k * A.cap + r];
        bnd[k] += tot * fabs((double)qk);
      }
    }
    for (int c = 0; c < nch; ++c) {
      const double v = warp_sum_d(bnd[c]);
      if (lane == 0) s_bnd[c][warp & 7] = v;
    }
    __syncthreads();
    if (threadIdx.x < nch) {
      double b = 0.0;
      for (int w = 0; w < (nwarp < 8 ? nwarp : 8); ++w) b += s_bnd[threadIdx.x][w];
      // widened for the FP32 rounding of the cell values and of S
      b *= 1.0 + 0x1p-18;
      int e = 0;
      if (b > 0.0 && b < 1e300) frexp(b, &e);  // b < 2^e
      const int sh = (b > 0.0 && b < 1e300) ? 62 - e : 0;
      s_shift[threadIdx.x] = sh;
      s_scale[threadIdx.x] = ldexp(1.0, sh);
      s_unscale[threadIdx.x] = ldexp(1.0, -sh);
    }
  } else if (threadIdx.x < nch) {
    const int e = A.exps[threadIdx.x];  // initialised far below any real exponent
    const int sh = e < -100000 ? 0 : kScaleTop - e;
    s_shift[threadIdx.x] = sh;
    s_scale[threadIdx.x] = ldexp(1.0, sh);
    s_unscale[threadIdx.x] = ldexp(1.0, -sh);
  }
  __syncthreads();
  float2(*tab)[32] = sh.tabs[warp & 7];
  {
    // FP32 pairs: warp w takes chunks w, w + nwarp, ... of kStage pair
    // records, each staged into shared memory by one bulk copy while the
    // warp deposits the previous chunk (two buffers per warp)
    uint4* stage[2] = {sh.stage[warp & 7][0], sh.stage[warp & 7][1]};
    unsigned long long* bar = sh.bar[warp & 7];
    const int nchunk = (f1 - f0 + kStage - 1) / kStage;
    auto issue = [&](int c, int b) {
      if (lane == 0 && c < nchunk) {
        const int s0 = f0 + c * kStage;
        const int cnt = f1 - s0 < kStage ? f1 - s0 : kStage;
        mbar_expect_tx(&bar[b], (unsigned)(cnt * kPairRecBytes));
        bulk_copy_g2s(stage[b], rec32 + (int64_t)s0 * kPairRecWords, (unsigned)(cnt * kPairRecBytes), &bar[b]);
      }
    };
    issue(warp, 0);
    // bit b: the phase buffer b waits for next (the barriers live for the
    // CTA, initialised once by deposit_init; every copy of an earlier tile
    // was waited for)
    unsigned parity = sh.phase[warp & 7];
    int b = 0;
    for (int c = warp; c < nchunk; c += nwarp) {
      issue(c + nwarp, b ^ 1);  // the other buffer was released at the end of the last round
      if (!mbar_wait_warp(&bar[b], (parity >> b) & 1u)) {
        // a bulk copy that never completes: record it, wait (bounded) for
        // the other buffer's copy in flight, deposit nothing more
        if (lane == 0) atomicOr(&A.st->flags, kFlagTimeout);
        if (c + nwarp < nchunk) mbar_wait_warp(&bar[b ^ 1], (parity >> (b ^ 1)) & 1u);
        break;
      }
      parity ^= 1u << b;
      const int s0 = f0 + c * kStage;
      const int cnt = f1 - s0 < kStage ? f1 - s0 : kStage;
      const uint4* R = stage[b];
      unsigned smask = 0;
      if (NQ > 0 && NQ <= 4) {  // pairs of at most kSmallCells cells go packed
        int nj = 0;
        if (lane < cnt) {
          const unsigned pk = R[lane * kPairRecWords + 1].w;
          nj = (int)(((pk >> 10) & 31u) + 1) * (int)(((pk >> 15) & 31u) + 1) *
               (DIMS == 3 ? (int)(((pk >> 20) & 31u) + 1) : 1);
        }
        smask = __ballot_sync(0xffffffffu, lane < cnt && nj <= kSmallCells);
        if (smask) {
#define SPHG_SMALL(K) \
  deposit_small<DIMS, K, NQ, TY, TZ, DET>(R, smask, nj, s_shift, nq, TV, sh.small[warp & 7], hi, lo, c2, lane)
          if (KERN >= 0) SPHG_SMALL(KERN >= 0 ? KERN : 0);
          else if (A.kern == 0) SPHG_SMALL(0);
          else if (A.kern == 1) SPHG_SMALL(1);
          else if (A.kern == 2) SPHG_SMALL(2);
          else if (A.kern == 3) SPHG_SMALL(3);
          else SPHG_SMALL(4);
#undef SPHG_SMALL
        }
      }
      for (int j = 0; j < cnt; ++j)
        if (!((smask >> j) & 1u))
          deposit_pair32<DIMS, KERN, NQ, TY, TZ, DET>(A, R + j * kPairRecWords, nq, TV, s_shift, tab, hi, lo, c2,
                                                      lane);
      __syncwarp();
      if (lane == 0) fence_proxy_async_smem();  // this buffer's reads before its next bulk copy
      b ^= 1;
    }
    __syncwarp();
    if (lane == 0) sh.phase[warp & 7] = parity;
  }
  // FP64 pairs (ill-conditioned records), warp per pair
  for (int j = d0 + warp; j < d1; j += nwarp) {
    const uint4* R = rec64 + (int64_t)j * kPairRecWords;
    deposit_pair_fp64<DIMS, KERN, TY, TZ, DET>(A, R, nq, TV, hi, lo, c2, s_scale, lane);
    __syncwarp();
  }
  __syncthreads();
  const int64_t P = A.mp.P;
  const int64_t PD = DIMS == 2 ? P * P : P * P * P;
  const double inv_w = s_unscale[nq];
  if (split) {
    // add this chunk's sums to the tile's raw partial sums (exact int64 in
    // the deterministic mode: every chunk of the tile has the same scale)
    for (int v = threadIdx.x; v < TV; v += blockDim.x) {
      int li, i, j, k;
      flush_cell<DIMS, TX, TY, TZ>(A, v, ox, oy, oz, false, li, i, j, k);
      if (i >= P || j >= P || (DIMS == 3 && k >= P)) continue;
      const int64_t row = DIMS == 2 ? (int64_t)i * P + j : ((int64_t)i * P + j) * P + k;
      for (int c = 0; c <= nq; ++c) {
        if (DET) {
          const unsigned long long x = (unsigned long long)fixed_value(hi, lo, c2, c * TV + li);
          if (x) atomicAdd((unsigned long long*)A.acc + row + c * PD, x);
        } else {
          const double x = cell_value<DET>(hi, lo, c2, c * TV + li);
          if (x != 0.0) atomicAdd(A.acc + row + c * PD, x * s_unscale[c]);
        }
      }
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) sh.last = atomicAdd(A.done + t, 1) == A.split - 1;
    __syncthreads();
    if (sh.last) {  // every chunk of the tile has added its sums: write the output
      __threadfence();
      for (int v = threadIdx.x; v < TV; v += blockDim.x) {
        int li, i, j, k;
        flush_cell<DIMS, TX, TY, TZ>(A, v, ox, oy, oz, DIMS == 2 && A.mode == 0, li, i, j, k);
        if (i >= P || j >= P || (DIMS == 3 && k >= P)) continue;
        const int64_t row = DIMS == 2 ? (int64_t)i * P + j : ((int64_t)i * P + j) * P + k;
        auto sum = [&](int c) {
          if (DET) return (double)(long long)__ldcg((const unsigned long long*)A.acc + row + c * PD) * s_unscale[c];
          return __ldcg(A.acc + row + c * PD);
        };
        store_cell<DIMS>(A, P, PD, i, j, k, nq, sum(nq), sum);
      }
    }
    __syncthreads();  // the shared accumulators are reused by the next tile
    return;
  }
  // flush: FP64 values straight into the output layout
  for (int v = threadIdx.x; v < TV; v += blockDim.x) {
    int li, i, j, k;
    flush_cell<DIMS, TX, TY, TZ>(A, v, ox, oy, oz, DIMS == 2 && A.mode == 0, li, i, j, k);
    if (i >= P || j >= P || (DIMS == 3 && k >= P)) continue;
    const double W = cell_value<DET>(hi, lo, c2, nq * TV + li) * inv_w;
    store_cell<DIMS>(A, P, PD, i, j, k, nq, W,
                     [&](int c) { return cell_value<DET>(hi, lo, c2, c * TV + li) * s_unscale[c]; });
  }
  __syncthreads();  // the shared accumulators are reused by the next tile
}

template <int DIMS, int KERN, int NQ, int TX, int TY, int TZ, bool DET>
// Launch bounds: five CTAs per SM (48 registers); at six (40 registers) the
// pair loop spills to local memory.
__global__ void __launch_bounds__(256, 5) k_deposit(TiledArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ DepositShared sh;
  deposit_init(sh);
  deposit_tile<DIMS, KERN, NQ, TX, TY, TZ, DET>(A, blockIdx.x, smem_raw, sh);
}

template <int DIMS, int KERN, int NQ, bool DET>
void launch_deposit_det(const TiledArgs& A, cudaStream_t s) {
  // the tile accumulators are dynamic shared memory beside DepositShared;
  // above the default 48 KB in all the kernel opts in
  if (DIMS == 2) {
    constexpr int TX = 16, TY = 16;
    const size_t sm = (DET ? 3 : 2) * (size_t)(A.pt.nq + 1) * TX * TY * sizeof(float);
    if (sm + sizeof(DepositShared) > 48 * 1024)
      cudaFuncSetAttribute(k_deposit<2, KERN, NQ, TX, TY, 1, DET>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_deposit<2, KERN, NQ, TX, TY, 1, DET><<<(unsigned)A.n_tiles, 256, sm, s>>>(A);
  } else {
    constexpr int TX = kTile3X, TY = kTile3Y, TZ = kTile3Z;
    const size_t sm = (DET ? 3 : 2) * (size_t)(A.pt.nq + 1) * TX * TY * TZ * sizeof(float);
    if (sm + sizeof(DepositShared) > 48 * 1024)
      cudaFuncSetAttribute(k_deposit<3, KERN, NQ, TX, TY, TZ, DET>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sm);
    k_deposit<3, KERN, NQ, TX, TY, TZ, DET><<<(unsigned)A.n_tiles, 256, sm, s>>>(A);
  }
}

template <int DIMS, int KERN, int NQ>
void launch_deposit_nq(const TiledArgs& A, cudaStream_t s) {
  if (A.det) launch_deposit_det<DIMS, KERN, NQ, true>(A, s);
  else launch_deposit_det<DIMS, KERN, NQ, false>(A, s);
}

template <int DIMS, int KERN>
inline void launch_kern(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev) {
  k_norm_fill<DIMS, KERN><<<grid_rec, 256, 0, s>>>(A);
  k_large_partials<DIMS, KERN><<<A.large_grid, 256, 0, s>>>(A);
  k_large_finish<DIMS, KERN><<<A.large_grid, 256, 0, s>>>(A);
  if (ev) cudaEventRecord(ev[2], s);
  switch (DIMS == 3 ? 1 : A.pt.nq) {
    case 1: launch_deposit_nq<DIMS, KERN, 1>(A, s); break;
    case 2: launch_deposit_nq<DIMS, KERN, 2>(A, s); break;
    case 3: launch_deposit_nq<DIMS, KERN, 3>(A, s); break;
    case 4: launch_deposit_nq<DIMS, KERN, 4>(A, s); break;
    default: launch_deposit_nq<DIMS, KERN, 0>(A, s); break;
  }
}

}  // namespace tiled_detail

// Instantiates launch_norm_deposit_<K> (declared in internal.h).
#define SPHG_TILED_SHAPE(K)                                                                     \
  void launch_norm_deposit_##K(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev) { \
    if (A.mp.dims == 2) tiled_detail::launch_kern<2, K>(A, grid_rec, s, ev);                   \
    else tiled_detail::launch_kern<3, K>(A, grid_rec, s, ev);                                  \
  }

}  // namespace sphg
