// tiled_fp32.cu -- K1/K2 and the host launcher of the FP32-compensated tiled
// deposition (see tiled.cuh for the pipeline; K3/K4 are in tiled_kernels.cuh).  Compiled with --fmad=false so
// that the FP64 arithmetic shared with the plain path rounds exactly as the
// reference; the FP32 hot loops use explicit fmaf.
#include <cuda_runtime.h>

#include <climits>

#include "internal.h"
#include "tiled.cuh"

namespace sphg {

namespace {

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// K1: one thread per input particle.
template <int DIMS>
__global__ void __launch_bounds__(256) k_prep_count(TiledArgs A) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  unsigned long long c_mapped = 0, c_dep = 0;
  double c_pm = 0.0;
  unsigned flags = 0;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < A.pt.n; base += stride) {
    const int64_t p = base + threadIdx.x;
    PrepFP64 q;
    int state = kPrepSkip;
    if (p < A.pt.n) state = prep_particle_fp64<DIMS>(A.pt, A.mp, p, true, &q);
    if (state == kPrepNonFinite) flags |= kFlagNonFinite;
    int ni = 0, nj = 0, nk = 0;
    if (state == kPrepMapped) {
      ni = (int)(q.hi[0] - q.lo[0] + 1);
      nj = (int)(q.hi[1] - q.lo[1] + 1);
      nk = (int)(q.hi[2] - q.lo[2] + 1);
      c_mapped += 1;
      c_dep += (unsigned long long)ni * nj * nk;
      c_pm += q.m_in;
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
      A.geo[r] = make_float4(__double2float_rn(q.x - (double)i0), __double2float_rn(q.y - (double)j0),
                             DIMS == 3 ? __double2float_rn(q.z - (double)k0) : 0.0f,
                             __double2float_rn(q.hsml));
      // weight factor numerator: area*w*dz (cic_2D.jl:187-188) / vol*w*L (cic_3D.jl:168-169)
      A.cp[r] = DIMS == 2 ? q.area * q.wgt * q.col : q.vol * q.wgt * A.mp.L;
      A.aux[r] = q.rho_in * q.knorm / (A.mp.L * A.mp.L * A.mp.L);
      for (int k = 0; k < A.pt.nq; ++k)
        A.qv[(int64_t)k * A.cap + r] = q.scalar_zero ? 0.0f
            : __double2float_rn(ld_elem(A.pt.attr_dtype, A.pt.q, p * A.pt.qsp + k * A.pt.qsk));
      if (A.det) {  // exponent of the particle's total per channel
        const double num = fabs(A.cp[r]);
        int e;
        if (num > 0.0 && num < 1e300) {
          frexp(num, &e);
          atomicMax(&A.kexp[A.pt.nq], e);
          for (int k = 0; k < A.pt.nq; ++k) {
            const double qa = fabs((double)A.qv[(int64_t)k * A.cap + r]);
            if (qa > 0.0 && qa < 1e300) {
              frexp(num * qa, &e);
              atomicMax(&A.kexp[k], e);
            }
          }
        }
      }
      if ((int64_t)ni * nj * nk > kLargeCells) A.large[atomicAdd(A.n_large, 1)] = r;
      // (particle, tile) overlaps
      const int tx0 = i0 / A.tdim[0], tx1 = (i0 + ni - 1) / A.tdim[0];
      const int ty0 = j0 / A.tdim[1], ty1 = (j0 + nj - 1) / A.tdim[1];
      const int tz0 = k0 / A.tdim[2], tz1 = (k0 + nk - 1) / A.tdim[2];
      for (int tx = tx0; tx <= tx1; ++tx)
        for (int ty = ty0; ty <= ty1; ++ty)
          for (int tz = tz0; tz <= tz1; ++tz)
            atomicAdd(&A.tile_count[((int64_t)tx * A.ntile[1] + ty) * A.ntile[2] + tz], 1);
    }
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

// K2: exclusive scan of the tile counts (one CTA of 1024 threads).
__global__ void __launch_bounds__(1024) k_scan_tiles(TiledArgs A) {
  __shared__ long long part[1024];
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

}  // namespace

void tiled_geometry(int dims, int64_t P, int tdim[3], int ntile[3], int64_t* n_tiles) {
  if (dims == 2) {
    tdim[0] = 16; tdim[1] = 16; tdim[2] = 1;
  } else {
    tdim[0] = 8; tdim[1] = 8; tdim[2] = 8;
  }
  for (int d = 0; d < 3; ++d) ntile[d] = (d < dims) ? (int)((P + tdim[d] - 1) / tdim[d]) : 1;
  *n_tiles = (int64_t)ntile[0] * ntile[1] * ntile[2];
}

// Launches K1..K4 on `s`.  With `ev` (4 events) the phases prep+scan,
// norm+fill and deposit are bracketed for timing.  Returns the number of
// kernels launched through `n_launch`.
cudaError_t launch_tiled_fp32(int kernel, const TiledArgs& A, int num_sms, cudaStream_t s,
                              cudaEvent_t* ev, int* n_launch) {
  const int dims = A.mp.dims;
  int grid = ceil_div(A.pt.n, 256);
  if (grid > num_sms * 8) grid = num_sms * 8;
  if (grid < 1) grid = 1;
  if (ev) cudaEventRecord(ev[0], s);
  if (dims == 2) k_prep_count<2><<<grid, 256, 0, s>>>(A);
  else k_prep_count<3><<<grid, 256, 0, s>>>(A);
  k_scan_tiles<<<1, 1024, 0, s>>>(A);
  if (ev) cudaEventRecord(ev[1], s);
  int grid_rec = ceil_div(A.pt.n, 8);
  if (grid_rec > num_sms * 16) grid_rec = num_sms * 16;
  if (grid_rec < 1) grid_rec = 1;
  switch (kernel) {
    case 0: launch_norm_deposit_0(A, grid_rec, s, ev); break;
    case 1: launch_norm_deposit_1(A, grid_rec, s, ev); break;
    case 2: launch_norm_deposit_2(A, grid_rec, s, ev); break;
    case 3: launch_norm_deposit_3(A, grid_rec, s, ev); break;
    default: launch_norm_deposit_4(A, grid_rec, s, ev); break;
  }
  if (ev) cudaEventRecord(ev[3], s);
  if (n_launch) *n_launch = 6;
  return cudaGetLastError();
}

}  // namespace sphg
