// tiled.cuh -- the FP32-compensated, image-tiled deposition.
//
// Pipeline for one map (all on one stream):
//   K1 k_prep_count   one thread per input particle: centring, filter, quantity
//                     skip and FP64 pixel ranges exactly as the reference
//                     (prep_particle_fp64); compacts mapped particles into
//                     records with FP32 local coordinates and counts the
//                     (particle, tile) overlaps per image tile.
//   K2 k_scan_tiles   exclusive scan of the tile counts (one CTA).
//   K3 k_norm_fill    one warp per record: the renormalisation sum
//                     S = sum(w(u) A) over the whole footprint (calculate_weights,
//                     cic_2D.jl:11-72) in FP32 with compensated lane sums; tiny,
//                     ill-conditioned particles (no pixel centre well inside the
//                     kernel) are redone in the reference's FP64 arithmetic.
//                     Writes one 64-byte pair record per (record, tile) pair
//                     whose cells can reach the kernel support into the
//                     tile's slot range.
//   K4 k_deposit      one CTA per image tile: the tile's pair records are
//                     staged into shared memory by bulk copies (TMA, one per
//                     16 records, double-buffered per warp); every pair adds
//                     w(u) A c_p (and q times it) to shared-memory accumulators;
//                     the tile is then flushed once, in FP64, straight into the
//                     output layout (reduce_image_2D/3D fused: reduce_image.jl:8-55).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

namespace sphg {

enum : int { kRecFP64 = 1, kRecFallback = 2 };

// Footprints above kLargeCells cells (the default of TiledArgs::large_cells)
// take the two-phase (multi-CTA) renormalisation in chunks of kChunkCells
// cells.
constexpr int64_t kLargeCells = 8192;
constexpr int64_t kChunkCells = 4096;

// Scale exponent target: the largest per-cell contribution of a channel is
// brought to about 2^kScaleTop before it enters FP32 accumulators.
constexpr int kScaleTop = 24;

// 3D deposit tile (cells per axis), shared by the single-map and batched
// paths so that deterministic sums agree bit for bit between them.
constexpr int kTile3X = 8, kTile3Y = 8, kTile3Z = 8;

// One (record, tile) pair as the deposit consumes it, written once by the
// renormalisation pass into the tile's slot range: 64 bytes (two DRAM
// sectors), so a tile's pairs form one contiguous stream that the deposit
// stages into shared memory with bulk copies.
//   w[0]  {fx, fy, fz, h}: the record's position offsets from its footprint
//         start and its smoothing length, pixel units (FP32)
//   w[1]  {1/h, factor mantissa, factor exponent, pack}; an FP64 pair holds
//         the record index in place of the exponent
//   w[2]  {a0, b0, c0, tot}: the start of the pair's cell box, footprint-
//         local, and the record's whole deposit |numerator| 2^-exponent
//         (FP32, the deterministic mode's tile bound)
//   w[3]  {q0, q1, q2, q3}: the quantities (more than four channels: the
//         record index in w[3].x, the deposit reads them by record)
// pack: tile-local index of the box start (10 bits), the box sides minus one
// (5 bits each, x y z), the FP64 flag and the X64 flag.  An FP64 pair with
// the X64 flag carries its particle's FP64 preparation in place of w[0] and
// w[3]: w[0] = {x, y} and w[3] = {hsml, 1/hsml} (2D) or {z, hsml} (3D), the
// pixel coordinates and smoothing length as doubles, so the deposit does
// not prepare the particle again.
constexpr int kPairRecWords = 4;  // uint4 per pair record
constexpr int kPackFP64 = 1 << 25;
constexpr int kPackX64 = 1 << 26;
constexpr size_t kPairRecBytes = kPairRecWords * 16;

// Counter ints of one map: tile_count, tile_fill and tile_fill64 per tile,
// then the record and large-record counters.
inline int64_t tiled_counter_ints(int64_t n_tiles) { return 3 * n_tiles + 2; }

struct TiledArgs {
  DevParticles pt;
  DevMapParams mp;
  int kern;         // SPHKernels shape (used where the shape is a runtime value)
  int large_cells;  // footprints above this many cells take the two-phase path
  DevMapParams mp_re;  // re-derivation after K1 (positions already centred in place)
  int tdim[3];      // tile extent per axis (1 on the unused 2D axis)
  int ntile[3];     // tiles per axis
  int64_t n_tiles;
  int64_t cap;      // record capacity
  int* n_rec;       // number of records (device counter)
  int4* box;        // {iMin, jMin, kMin, flags}
  int4* dimv;       // {ni, nj, nk, source particle}
  float4* geo;      // {x - iMin, y - jMin, z - kMin, h} in pixel units
  double* cp;       // K1: numerator of the weight factor; K3: the factor
  float* cpm;       // K3: the factor as FP32 mantissa ...
  int* cpe;         //     ... and binary exponent (cp = cpm * 2^cpe)
  double* aux;      // K1: rho / L^3 * kernel normalisation (3D mass diagnostic);
                    // K3: |numerator|, the record's total deposit into W
  float* qv;        // quantities, qv[k * cap + r]
  int* tile_count;  // per tile, zeroed before K1
  int* tile_fill;   // per tile, zeroed before K3: FP32 pairs, from the start of the tile's slots
  int* tile_fill64; // per tile, zeroed before K3: FP64 pairs, from the end of the tile's slots
  long long* tile_start;  // n_tiles + 1
  uint4* prec;      // pair records, kPairRecWords uint4 per slot (PairRec)
  long long pair_cap;
  // large records (two-phase renormalisation)
  int* n_large;             // count (device counter)
  int* large;               // record indices
  long long* large_start;   // chunk prefix per large record (n_large + 1)
  float4* partials;         // per chunk: compensated sum, error term, min u
  long long chunk_cap;
  int large_grid;
  int* exps;        // per channel max exponent (channels 0..nq-1 = Q, nq = W)
  // deterministic mode: exact int64 fixed-point tile sums, scaled per tile
  int det;
  DevStatus* st;
  // output
  double* out;
  int mode;         // 0: 2D reduced, 1: raw (P^D, nq+1) accumulator, 2: 3D reduced
  int reduce;       // 2D reduce_image
  int w_is_one;     // 3D !reduce_image
  // tiles split over several CTAs (split > 1): chunk c of a tile deposits
  // pairs [c n / split, (c + 1) n / split) of its n and adds its partial
  // sums to `acc`; the tile's last chunk writes the output from there
  int split;
  double* acc;      // raw (P^D, nq+1) partial sums: FP64, or the int64 fixed-point
                    // bits in the deterministic mode (one scale per tile)
  int* done;        // chunks finished per tile
};

// Points A's counters (A.n_tiles set) into `base`, tiled_counter_ints(n_tiles)
// ints laid out as tile_count, tile_fill, tile_fill64, n_rec, n_large.
inline void bind_counters(TiledArgs& A, int* base) {
  A.tile_count = base;
  A.tile_fill = base + A.n_tiles;
  A.tile_fill64 = base + 2 * A.n_tiles;
  A.n_rec = base + 3 * A.n_tiles;
  A.n_large = A.n_rec + 1;
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Error-free sum of two floats (Knuth's TwoSum): a + b == s + e exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// Compensated accumulation into a shared-memory (hi, lo) pair: the atomic add
// returns the value it added to, so the rounding error of that very addition
// is recovered exactly with TwoSum and accumulated in `lo`.
__device__ __forceinline__ void acc_twosum(float* hi, float* lo, float v) {
  const float old = atomicAdd(hi, v);
  float s, e;
  two_sum(old, v, s, e);
  if (e != 0.0f) atomicAdd(lo, e);
}

// The same compensated accumulation into an adjacent (hi, lo) pair with one
// 64-bit compare-and-swap per attempt: the pair is read, v is added to hi
// with TwoSum and its error to lo, and both words are swapped in together
// if the pair is unchanged (else the attempt repeats on the pair it found;
// some thread's swap succeeds on every round, so the loop ends).  One loop
// per channel instead of the two FP32 atomics' loops, but measured slower in
// the deposit (3D 7.33 against 6.97 ms, 96-map batch 97.6 against 80.5 ms);
// kept for the accumulation microbenchmark (sphg_probe_smem_rate kind 4).
__device__ __forceinline__ void acc_pair(float2* p, float v) {
  unsigned long long* a = reinterpret_cast<unsigned long long*>(p);
  unsigned long long seen = *a;
  for (;;) {
    const float hi = __uint_as_float((unsigned)seen), lo = __uint_as_float((unsigned)(seen >> 32));
    float s, e;
    two_sum(hi, v, s, e);
    const unsigned long long want =
        (unsigned long long)__float_as_uint(s) | ((unsigned long long)__float_as_uint(lo + e) << 32);
    const unsigned long long was = atomicCAS(a, seen, want);
    if (was == seen) return;
    seen = was;
  }
}


// A record is redone in FP64 when every pixel centre is near or beyond the
// kernel edge (FP32 cancellation in 1 - u), when its FP32 sum is 0 (the
// reference's fallback branch) or below 2^-40 (its per-cell factor numerator
// / S would leave the FP32 range once scaled for the tile accumulators).
__device__ __forceinline__ bool ill_conditioned(float S, float umin) {
  return umin > 0.9f || !(S >= 0x1p-40f);
}

// FP32 kernel shape (no normalisation) via fused multiply-adds.
template <int KERN>
__device__ __forceinline__ float kshape_f(float u) {
  if (KERN == 0) {
    if (u < 0.5f) return fmaf(6.0f * (u - 1.0f), u * u, 1.0f);
    const float t = 1.0f - u;
    return 2.0f * t * t * t;
  } else if (KERN == 1) {
    const float a = 1.0f - u, b = (2.0f / 3.0f) - u, c = (1.0f / 3.0f) - u;
    const float a2 = a * a, b2 = b * b, c2 = c * c;
    const float a5 = a2 * a2 * a, b5 = b2 * b2 * b, c5 = c2 * c2 * c;
    if (u < 1.0f / 3.0f) return fmaf(15.0f, c5, fmaf(-6.0f, b5, a5));
    if (u < 2.0f / 3.0f) return fmaf(-6.0f, b5, a5);
    return a5;
  } else if (KERN == 2) {
    const float t = 1.0f - u, t2 = t * t;
    return t2 * t2 * t2 * fmaf(u, fmaf(35.0f / 3.0f, u, 6.0f), 1.0f);
  } else if (KERN == 3) {
    const float t = 1.0f - u, t2 = t * t, t4 = t2 * t2;
    return t4 * t4 * fmaf(u, fmaf(u, fmaf(32.0f, u, 25.0f), 8.0f), 1.0f);
  } else {
    const float t = 1.0f - u, t2 = t * t, t4 = t2 * t2;
    return t4 * t4 * t2 * fmaf(u, fmaf(u, fmaf(u, fmaf(429.0f / 5.0f, u, 90.0f), 42.0f), 10.0f), 1.0f);
  }
}

// Distance in units of h from the squared distance (shared by the
// renormalisation and the deposit so both see the same u).
__device__ __forceinline__ float u_of(float d2, float hinv) {
  return d2 > 0.0f ? d2 * rsqrtf(d2) * hinv : 0.0f;
}

// Kernel shape with the shape chosen at compile time (KERN >= 0) or at run
// time (KERN < 0: `kern`, uniform across a warp).
template <int KERN>
__device__ __forceinline__ float shape_f(int kern, float u) {
  if (KERN >= 0) return kshape_f<(KERN < 0 ? 0 : KERN)>(u);
  switch (kern) {
    case 0: return kshape_f<0>(u);
    case 1: return kshape_f<1>(u);
    case 2: return kshape_f<2>(u);
    case 3: return kshape_f<3>(u);
    default: return kshape_f<4>(u);
  }
}

template <int KERN>
__device__ __forceinline__ double shape_d(int kern, double u) {
  if (KERN >= 0) return kshape<(KERN < 0 ? 0 : KERN), double>(u);
  switch (kern) {
    case 0: return kshape<0, double>(u);
    case 1: return kshape<1, double>(u);
    case 2: return kshape<2, double>(u);
    case 3: return kshape<3, double>(u);
    default: return kshape<4, double>(u);
  }
}

// Overlap of [f - h, f + h] with local pixel a and the pixel-centre offset.
__device__ __forceinline__ void axis_f(float f, float h, int a, float* dist, float* ov) {
  const float fa = (float)a;
  *dist = f - fa - 0.5f;
  *ov = fminf(f + h, fa + 1.0f) - fmaxf(f - h, fa);
}

// Separable per-axis part of a cell: (squared pixel-centre offset, overlap).
// The squared distance of a cell is (sx + sy) + sz, in that order, wherever
// it is formed (tables or direct), so every pass sees the same u.
__device__ __forceinline__ float2 axis_sq(float f, float h, int a) {
  float dist, ov;
  axis_f(f, h, a, &dist, &ov);
  return make_float2(dist * dist, ov);
}

// q = m * 2^e with m in [0.5, 1) for normal floats, by bit operations (no
// branches); zero, subnormal and non-finite q are returned as m = q, e = 0.
__device__ __forceinline__ void split_f(float q, float& m, int& e) {
  const unsigned b = __float_as_uint(q);
  const int be = (int)((b >> 23) & 0xffu);
  const bool normal = be != 0 && be != 255;
  m = normal ? __uint_as_float((b & 0x807fffffu) | (126u << 23)) : q;
  e = normal ? be - 126 : 0;
}

// Divide small non-negative integers with a float reciprocal: with inv_d
// within 2^-21 (relative) of 1/d, trunc((e + 0.5) * inv_d) == e / d for
// 0 <= e < 2^20, since (e + 0.5) / d stays at least 0.5 / d away from an
// integer and the error of the product is below (e + 0.5) * 2^-20 / d.
__device__ __forceinline__ int fdiv(int e, float inv_d) { return __float2int_rz(((float)e + 0.5f) * inv_d); }

// Reciprocal of a positive integer for fdiv: the approximate reciprocal
// (within 2 ulp), one instruction instead of the correctly rounded division.
__device__ __forceinline__ float inv_small(int d) { return __fdividef(1.0f, (float)d); }

// 2^k as a float for -126 <= k <= 127, 0 below (the values scaled by it are
// then below 2^-126 of the channel's largest and do not change the sums),
// infinity above; exact, without the special-case branches of ldexpf.
__device__ __forceinline__ float pow2f(int k) {
  const int kc = k < -127 ? -127 : (k > 128 ? 128 : k);
  return __int_as_float((kc + 127) << 23);
}

}  // namespace sphg
