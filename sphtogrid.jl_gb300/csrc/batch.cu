// batch.cu -- many maps of uneven particle counts, resolutions, quantity
// counts and kernel shapes in one pipeline: one launch per phase for all maps
// and one persistent deposit launch that pulls image tiles of every map from
// a work queue (largest maps first).  The whole sequence is captured once in
// a CUDA graph and replayed; an autotuner picks the 2D tile shape, the
// deposit's CTAs per SM and the large-footprint threshold.
//
// Compiled with --fmad=false (see tiled_fp32.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/sphgrid.h"
#include "internal.h"
#include "tiled_kernels.cuh"

namespace sphg {
using namespace tiled_detail;

namespace {

struct BatchDev {
  const TiledArgs* maps;
  int n_maps;
  const int* blk_base;         // K1: first CTA of each map (n_maps + 1)
  const long long* tile_base;  // K4: first queue slot of each position (n_maps + 1)
  const int* order;            // K4: map at each position of the queue
  unsigned long long* queue;   // K4: next queue slot
  long long total_tiles;
};

__device__ __forceinline__ int find_seg_ll(const long long* base, int n, long long x) {
  int lo = 0, hi = n - 1;  // largest i with base[i] <= x
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_seg_i(const int* base, int n, int x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Particles of one map per K1 CTA (four rounds of 256 threads): the CTA's
// set-up (its map, the shared tile counts) is paid once per 1024 particles.
constexpr int64_t kPrepSpan = 1024;

__global__ void __launch_bounds__(256, 4) kb_prep(BatchDev B) {
  const int m = find_seg_i(B.blk_base, B.n_maps, blockIdx.x);
  const TiledArgs& A = B.maps[m];
  const int64_t base = (int64_t)(blockIdx.x - B.blk_base[m]) * kPrepSpan;
  __shared__ PrepShared sh;
  if (A.mp.dims == 2) prep_count<2>(A, base, blockDim.x, sh, base + kPrepSpan);
  else prep_count<3>(A, base, blockDim.x, sh, base + kPrepSpan);
}

__global__ void __launch_bounds__(1024) kb_scan(BatchDev B) {
  __shared__ long long part[1024];
  scan_tiles(B.maps[blockIdx.x], part);
}

// The renormalisation phase runs once per (dimensions, kernel shape) that
// the batch holds, over that shape's maps: each launch evaluates one
// compile-time shape, so its code stays small (one launch over every shape
// inlined all of them and stalled on instruction fetch).
template <int DIMS, int KERN>
__global__ void __launch_bounds__(256, 4) kb_norm(BatchDev B) {
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  __shared__ NormShared sh;
  for (int m = 0; m < B.n_maps; ++m) {
    const TiledArgs& A = B.maps[m];
    if (A.mp.dims == DIMS && A.kern == KERN) norm_records<DIMS, KERN>(A, wid, nw, threadIdx.x & 31, sh);
  }
}

template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) kb_large_partials(BatchDev B) {
  __shared__ float red[3][8];
  for (int m = 0; m < B.n_maps; ++m) {
    const TiledArgs& A = B.maps[m];
    if (A.mp.dims == DIMS && A.kern == KERN) large_partials<DIMS, KERN>(A, blockIdx.x, gridDim.x, red);
  }
}

template <int DIMS, int KERN>
__global__ void __launch_bounds__(256) kb_large_finish(BatchDev B) {
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int m = 0; m < B.n_maps; ++m) {
    const TiledArgs& A = B.maps[m];
    if (A.mp.dims == DIMS && A.kern == KERN) large_finish<DIMS, KERN>(A, wid, nw, threadIdx.x & 31);
  }
}

template <int DIMS, int KERN>
void launch_norm_shape(const BatchDev& d, int num_sms, cudaStream_t s) {
  kb_norm<DIMS, KERN><<<num_sms * 16, 256, 0, s>>>(d);
  kb_large_partials<DIMS, KERN><<<num_sms * 4, 256, 0, s>>>(d);
  kb_large_finish<DIMS, KERN><<<num_sms * 4, 256, 0, s>>>(d);
}

template <int DIMS>
void launch_norm_dims(int kern, const BatchDev& d, int num_sms, cudaStream_t s) {
  switch (kern) {
    case 0: launch_norm_shape<DIMS, 0>(d, num_sms, s); break;
    case 1: launch_norm_shape<DIMS, 1>(d, num_sms, s); break;
    case 2: launch_norm_shape<DIMS, 2>(d, num_sms, s); break;
    case 3: launch_norm_shape<DIMS, 3>(d, num_sms, s); break;
    default: launch_norm_shape<DIMS, 4>(d, num_sms, s); break;
  }
}

// One tile of one map, for a compile-time channel count.  Out of line: the
// persistent kernel dispatches among several specialisations, and a call per
// tile keeps each one's register use inside its own cell loop.
template <int DIMS, int NQ, int TX, int TY, int TZ, bool DET>
__device__ __noinline__ void tile_call(const TiledArgs& A, long long t, int chunk, unsigned char* smem_raw,
                                       DepositShared& sh) {
  deposit_tile<DIMS, -1, NQ, TX, TY, TZ, DET>(A, t, smem_raw, sh, chunk);
}

// The persistent deposit: every CTA takes the next tile from the queue until
// the queue is empty.
template <int TX, int TY, bool DET>
__global__ void __launch_bounds__(256, 6) kb_deposit(BatchDev B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ DepositShared sh;
  __shared__ long long t_sh;
  deposit_init(sh);
  for (;;) {
    if (threadIdx.x == 0) t_sh = (long long)atomicAdd(B.queue, 1ull);
    __syncthreads();
    const long long t = t_sh;
    __syncthreads();
    if (t >= B.total_tiles) break;
    const int pos = find_seg_ll(B.tile_base, B.n_maps, t);
    const TiledArgs& A = B.maps[B.order[pos]];
    // a split map's queue slots are (chunk, tile), chunk-major, so the
    // chunks of one tile run apart in time
    const long long slot = t - B.tile_base[pos];
    const long long local = A.split > 1 ? slot % A.n_tiles : slot;
    const int chunk = A.split > 1 ? (int)(slot / A.n_tiles) : 0;
    // the map's channel count as a compile-time constant keeps the per-pair
    // factors in registers (3D maps carry one quantity)
    if (A.mp.dims == 3) {
      tile_call<3, 1, kTile3X, kTile3Y, kTile3Z, DET>(A, local, chunk, smem_raw, sh);
    } else {
      switch (A.pt.nq) {
        case 1: tile_call<2, 1, TX, TY, 1, DET>(A, local, chunk, smem_raw, sh); break;
        case 2: tile_call<2, 2, TX, TY, 1, DET>(A, local, chunk, smem_raw, sh); break;
        case 3: tile_call<2, 3, TX, TY, 1, DET>(A, local, chunk, smem_raw, sh); break;
        case 4: tile_call<2, 4, TX, TY, 1, DET>(A, local, chunk, smem_raw, sh); break;
        default: tile_call<2, 0, TX, TY, 1, DET>(A, local, chunk, smem_raw, sh); break;
      }
    }
  }
}

template <int TX, int TY>
void launch_kb_deposit_shape(const BatchDev& B, bool det, int grid, size_t smem, cudaStream_t s, bool prepare) {
  if (det) {
    if (prepare) cudaFuncSetAttribute(kb_deposit<TX, TY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    else kb_deposit<TX, TY, true><<<grid, 256, smem, s>>>(B);
  } else {
    if (prepare) cudaFuncSetAttribute(kb_deposit<TX, TY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    else kb_deposit<TX, TY, false><<<grid, 256, smem, s>>>(B);
  }
}

// Launches the persistent deposit for a 2D tile shape (prepare: only set its
// dynamic shared-memory limit, outside any graph capture).
bool launch_kb_deposit(int tx, int ty, const BatchDev& B, bool det, int grid, size_t smem, cudaStream_t s,
                       bool prepare = false) {
  if (tx == 16 && ty == 16) launch_kb_deposit_shape<16, 16>(B, det, grid, smem, s, prepare);
  else if (tx == 32 && ty == 16) launch_kb_deposit_shape<32, 16>(B, det, grid, smem, s, prepare);
  else if (tx == 32 && ty == 32) launch_kb_deposit_shape<32, 32>(B, det, grid, smem, s, prepare);
  else return false;
  return true;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Pairs per (chunk of a) tile above which a map's tiles are split over
// several CTAs, and the most chunks per tile.  A map of many particles on
// few pixels has few, heavy tiles; one CTA each would leave the rest of
// the GPU idle while they finish.
constexpr double kSplitPairs = 4096.0;
constexpr int kMaxSplit = 64;

}  // namespace

// ------------------------------------------------------------------ host

struct BatchMapHost {
  sphg_map_desc desc;
  sphg_params cpar;
  int64_t n_tiles = 0;
  long long pair_cap = 0, chunk_cap = 0;
  int split = 1;  // chunks per tile (CTAs sharing each tile's pairs)
};

// Chunks per tile of a map from its expected pairs per tile (about 1.5
// tiles per particle in 2D, 3 in 3D, for footprints small next to a tile).
inline int split_of(const BatchMapHost& M) {
  if (M.n_tiles <= 0) return 1;
  const double per_tile = (double)M.desc.parts.n * (M.desc.opt.dimensions == 2 ? 1.5 : 3.0) / (double)M.n_tiles;
  const double k = std::ceil(per_tile / kSplitPairs);
  return k < 1.0 ? 1 : (k > kMaxSplit ? kMaxSplit : (int)k);
}

struct BatchPlan {
  int tile_x = 16, tile_y = 16, ctas_per_sm = 4, large_cells = (int)kLargeCells;
  void* mem = nullptr;  // one device allocation for everything
  size_t mem_size = 0;
  std::vector<TiledArgs> args;
  std::vector<int> blk_base;
  std::vector<long long> tile_base;
  std::vector<int> order;
  BatchDev dev{};
  TiledArgs* d_args = nullptr;
  DevStatus* d_status = nullptr;  // per map
  char* counters = nullptr;
  size_t counters_bytes = 0;
  int* exps = nullptr;            // per map kMaxQ + 1
  size_t smem = 0;
  bool det = false;
  int k1_grid = 0;
  std::vector<int> shapes;  // (dimensions, kernel shape) pairs present: dims * 8 + shape
  std::vector<std::pair<char*, size_t>> zero;  // split maps' partial sums, zeroed per run
};

}  // namespace sphg

struct sphg_batch {
  sphg_context* ctx = nullptr;
  int device = 0;
  int num_sms = 0;
  std::vector<sphg::BatchMapHost> maps;
  sphg::BatchPlan plan;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t stream = nullptr;  // own stream (capture and synchronous work)
  cudaStream_t side = nullptr;    // second stream: renormalisation shapes run side by side
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaStream_t last = nullptr;    // stream of the last launch
  std::vector<sphg::DevStatus> h_status;
  std::string err;
  float tuned_ms = 0.0f;
};

namespace sphg {
namespace {

int bfail(sphg_batch* b, int st, const std::string& m) {
  b->err = std::string(sphg_status_string(st)) + (m.empty() ? "" : ": " + m);
  return st;
}

#define BCK(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      cudaGetLastError();                                                            \
      return bfail(b, SPHG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    }                                                                                \
  } while (0)

void free_plan(BatchPlan& p) {
  if (p.mem) cudaFree(p.mem);
  p.mem = nullptr;
  p.mem_size = 0;
}

// Lays out every map's buffers in one device allocation and fills the
// per-map TiledArgs.
int build_plan(sphg_batch* b) {
  BatchPlan& p = b->plan;
  const int nm = (int)b->maps.size();
  free_plan(p);
  p.args.assign(nm, TiledArgs());
  p.zero.clear();
  for (BatchMapHost& M : b->maps) M.split = split_of(M);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  struct Off {
    size_t box, dim, geo, cp, cpm, cpe, aux, qv, start, pairs, large, lstart, part, acc;
  };
  std::vector<Off> offs(nm);
  // shared regions first: counters, exponents, bounds, statuses + queue
  size_t cnt_bytes = 0;
  std::vector<size_t> cnt_off(nm);
  for (int m = 0; m < nm; ++m) {
    cnt_off[m] = cnt_bytes;
    cnt_bytes += tiled_counter_ints(b->maps[m].n_tiles) * sizeof(int);
  }
  const size_t o_cnt = take(cnt_bytes);
  const size_t o_exps = take((size_t)nm * (kMaxQ + 1) * sizeof(int));
  const size_t o_stat = take((size_t)nm * sizeof(DevStatus) + sizeof(unsigned long long));
  const size_t o_args = take((size_t)nm * sizeof(TiledArgs));
  const size_t o_meta = take((size_t)(nm + 1) * sizeof(int) + (size_t)(nm + 1) * sizeof(long long) +
                             (size_t)nm * sizeof(int) + 64);
  size_t smem = 0;
  for (int m = 0; m < nm; ++m) {
    const BatchMapHost& M = b->maps[m];
    const int64_t cap = M.desc.parts.n > 0 ? M.desc.parts.n : 1;
    const int nq = M.desc.parts.n_q;
    Off& o = offs[m];
    o.box = take(cap * sizeof(int4));
    o.dim = take(cap * sizeof(int4));
    o.geo = take(cap * sizeof(float4));
    o.cp = take(cap * sizeof(double));
    o.cpm = take(cap * sizeof(float));
    o.cpe = take(cap * sizeof(int));
    o.aux = take(cap * sizeof(double));
    o.qv = take(cap * nq * sizeof(float));
    o.start = take((M.n_tiles + 1) * sizeof(long long));
    o.pairs = take(M.pair_cap * kPairRecBytes);
    o.large = take(cap * sizeof(int));
    o.lstart = take((cap + 1) * sizeof(long long));
    o.part = take(M.chunk_cap * sizeof(float4));
    // tiles split over several CTAs: the raw partial sums and chunk counters
    const int64_t P = M.desc.par.Npixels[0];
    const int64_t PD = M.desc.opt.dimensions == 2 ? P * P : P * P * P;
    o.acc = M.split > 1 ? take((size_t)PD * (nq + 1) * sizeof(double) + M.n_tiles * sizeof(int)) : 0;
    const size_t tv = M.desc.opt.dimensions == 2 ? (size_t)p.tile_x * p.tile_y
                                                 : (size_t)kTile3X * kTile3Y * kTile3Z;
    smem = std::max(smem, (p.det ? 3 : 2) * (size_t)(nq + 1) * tv * sizeof(float));
  }
  cudaError_t e = cudaMalloc(&p.mem, off);
  if (e != cudaSuccess) {
    cudaGetLastError();
    p.mem = nullptr;
    return bfail(b, SPHG_ERR_ALLOC, "batch workspace of " + std::to_string(off) + " bytes");
  }
  p.mem_size = off;
  char* base = (char*)p.mem;
  p.counters = base + o_cnt;
  p.counters_bytes = cnt_bytes;
  p.exps = (int*)(base + o_exps);
  p.d_status = (DevStatus*)(base + o_stat);
  p.d_args = (TiledArgs*)(base + o_args);
  p.smem = smem;
  // queue order: maps by particle count, largest first
  p.order.resize(nm);
  for (int m = 0; m < nm; ++m) p.order[m] = m;
  std::stable_sort(p.order.begin(), p.order.end(), [&](int a, int c) {
    return b->maps[a].desc.parts.n > b->maps[c].desc.parts.n;
  });
  p.blk_base.assign(nm + 1, 0);
  p.tile_base.assign(nm + 1, 0);
  for (int m = 0; m < nm; ++m) {
    const BatchMapHost& M = b->maps[m];
    const int64_t n = M.desc.parts.n;
    p.blk_base[m + 1] = p.blk_base[m] + (int)std::max<int64_t>(1, (n + kPrepSpan - 1) / kPrepSpan);
  }
  for (int i = 0; i < nm; ++i) {
    const BatchMapHost& M = b->maps[p.order[i]];
    p.tile_base[i + 1] = p.tile_base[i] + M.n_tiles * M.split;
  }
  p.k1_grid = p.blk_base[nm];
  p.shapes.clear();  // kernel ids are validated (0-4) when the maps are added
  for (int m = 0; m < nm; ++m) p.shapes.push_back(b->maps[m].desc.opt.dimensions * 8 + b->maps[m].desc.opt.kernel);
  std::sort(p.shapes.begin(), p.shapes.end());
  p.shapes.erase(std::unique(p.shapes.begin(), p.shapes.end()), p.shapes.end());
  for (int m = 0; m < nm; ++m) {
    const BatchMapHost& M = b->maps[m];
    const sphg_map_desc& D = M.desc;
    const Off& o = offs[m];
    TiledArgs& A = p.args[m];
    std::memset(&A, 0, sizeof(A));
    const int dims = D.opt.dimensions;
    const int64_t P = D.par.Npixels[0];
    A.pt.n = D.parts.n;
    A.pt.pos_dtype = D.parts.pos_dtype;
    A.pt.attr_dtype = D.parts.attr_dtype;
    A.pt.pos = D.parts.pos;
    A.pt.sp = D.parts.pos_stride_p;
    A.pt.sc = D.parts.pos_stride_c;
    A.pt.hsml = D.parts.hsml;
    A.pt.mass = D.parts.mass;
    A.pt.rho = D.parts.rho;
    A.pt.w = D.parts.weights;
    A.pt.q = D.parts.bin_q;
    A.pt.nq = D.parts.n_q;
    A.pt.qsp = D.parts.q_stride_p;
    A.pt.qsk = D.parts.q_stride_k;
    DevMapParams& mp = A.mp;
    for (int k = 0; k < 3; ++k) {
      mp.cen[k] = D.par.center[k];
      mp.lo[k] = M.cpar.center[k] - M.cpar.halfsize[k];
      mp.hi[k] = M.cpar.center[k] + M.cpar.halfsize[k];
    }
    mp.boxsize = D.par.boxsize;
    mp.periodic = D.par.periodic;
    mp.center_mode = D.opt.center;
    mp.filter = D.opt.filter;
    mp.calc_mean = dims == 2 ? D.opt.calc_mean : 0;
    mp.kernel_dim = D.opt.kernel_dim;
    mp.dims = dims;
    mp.L = M.cpar.len2pix;
    mp.P = P;
    mp.sigma = kernel_sigma(D.opt.kernel, D.opt.kernel_dim);
    set_lite_params(mp);
    A.mp_re = mp;
    A.kern = D.opt.kernel;
    A.large_cells = p.large_cells;
    if (dims == 2) {
      A.tdim[0] = p.tile_x;
      A.tdim[1] = p.tile_y;
      A.tdim[2] = 1;
    } else {
      A.tdim[0] = kTile3X;
      A.tdim[1] = kTile3Y;
      A.tdim[2] = kTile3Z;
    }
    for (int d = 0; d < 3; ++d) A.ntile[d] = d < dims ? (int)((P + A.tdim[d] - 1) / A.tdim[d]) : 1;
    A.n_tiles = M.n_tiles;
    A.cap = D.parts.n > 0 ? D.parts.n : 1;
    A.box = (int4*)(base + o.box);
    A.dimv = (int4*)(base + o.dim);
    A.geo = (float4*)(base + o.geo);
    A.cp = (double*)(base + o.cp);
    A.cpm = (float*)(base + o.cpm);
    A.cpe = (int*)(base + o.cpe);
    A.aux = (double*)(base + o.aux);
    A.qv = (float*)(base + o.qv);
    bind_counters(A, (int*)(p.counters + cnt_off[m]));
    A.tile_start = (long long*)(base + o.start);
    A.prec = (uint4*)(base + o.pairs);
    A.pair_cap = M.pair_cap;
    A.large = (int*)(base + o.large);
    A.large_start = (long long*)(base + o.lstart);
    A.partials = (float4*)(base + o.part);
    A.chunk_cap = M.chunk_cap;
    A.exps = p.exps + (size_t)m * (kMaxQ + 1);
    A.det = p.det ? 1 : 0;
    A.st = p.d_status + m;
    A.out = D.out;
    A.split = M.split;
    if (M.split > 1) {
      const int64_t PD = dims == 2 ? P * P : P * P * P;
      const size_t acc_bytes = (size_t)PD * (D.parts.n_q + 1) * sizeof(double);
      A.acc = (double*)(base + o.acc);
      A.done = (int*)(base + o.acc + acc_bytes);
      p.zero.push_back({base + o.acc, acc_bytes + M.n_tiles * sizeof(int)});
    }
    const bool raw = D.opt.raw_accumulator || (dims == 2 && D.opt.return_both_maps);
    A.mode = raw ? 1 : (dims == 3 ? 2 : 0);
    A.reduce = D.opt.reduce_image;
    A.w_is_one = D.opt.reduce_image ? 0 : 1;
  }
  // device copies of the tables (8-byte entries first: natural alignment)
  char* meta = base + o_meta;
  long long* d_tb = (long long*)meta;
  int* d_blk = (int*)(meta + (nm + 1) * sizeof(long long));
  int* d_order = d_blk + (nm + 1);
  if (smem > 227 * 1024) return bfail(b, SPHG_ERR_UNSUPPORTED, "tile accumulators exceed shared memory");
  if (!launch_kb_deposit(p.tile_x, p.tile_y, p.dev, p.det, 0, smem, nullptr, true))
    return bfail(b, SPHG_ERR_ARG, "tile shape must be 16x16, 32x16 or 32x32");
  BCK(cudaMemcpy(p.d_args, p.args.data(), (size_t)nm * sizeof(TiledArgs), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(d_blk, p.blk_base.data(), (size_t)(nm + 1) * sizeof(int), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(d_tb, p.tile_base.data(), (size_t)(nm + 1) * sizeof(long long), cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(d_order, p.order.data(), (size_t)nm * sizeof(int), cudaMemcpyHostToDevice));
  p.dev.maps = p.d_args;
  p.dev.n_maps = nm;
  p.dev.blk_base = d_blk;
  p.dev.tile_base = d_tb;
  p.dev.order = d_order;
  p.dev.queue = (unsigned long long*)(p.d_status + nm);
  p.dev.total_tiles = p.tile_base[nm];
  return SPHG_OK;
}

// All launches of one batch run on `s` (graph-capturable: no host sync).
int enqueue(sphg_batch* b, cudaStream_t s) {
  BatchPlan& p = b->plan;
  const int nm = (int)b->maps.size();
  BCK(cudaMemsetAsync(p.counters, 0, p.counters_bytes, s));
  BCK(cudaMemsetAsync(p.exps, 0x80, (size_t)nm * (kMaxQ + 1) * sizeof(int), s));
  BCK(cudaMemsetAsync(p.d_status, 0, (size_t)nm * sizeof(DevStatus) + sizeof(unsigned long long), s));
  for (const auto& z : p.zero) BCK(cudaMemsetAsync(z.first, 0, z.second, s));
  kb_prep<<<p.k1_grid, 256, 0, s>>>(p.dev);
  kb_scan<<<nm, 1024, 0, s>>>(p.dev);
  // the renormalisation of each (dimensions, kernel shape) touches only its
  // own maps: the shapes after the first run on the side stream, so one
  // shape's tail overlaps another's work; the deposit waits for both
  const bool two = p.shapes.size() > 1;
  if (two) {
    BCK(cudaEventRecord(b->fork, s));
    BCK(cudaStreamWaitEvent(b->side, b->fork, 0));
  }
  for (size_t i = 0; i < p.shapes.size(); ++i) {  // dims * 8 + kernel shape
    const int shape = p.shapes[i];
    cudaStream_t t = (two && i > 0) ? b->side : s;
    if (shape >> 3 == 2) launch_norm_dims<2>(shape & 7, p.dev, b->num_sms, t);
    else launch_norm_dims<3>(shape & 7, p.dev, b->num_sms, t);
  }
  if (two) {
    BCK(cudaEventRecord(b->join, b->side));
    BCK(cudaStreamWaitEvent(s, b->join, 0));
  }
  if (!launch_kb_deposit(p.tile_x, p.tile_y, p.dev, p.det, b->num_sms * p.ctas_per_sm, p.smem, s))
    return bfail(b, SPHG_ERR_ARG, "tile shape must be 16x16, 32x16 or 32x32");
  BCK(cudaGetLastError());
  return SPHG_OK;
}

// Runs the batch eagerly until no list overflows (growing capacities).
int run_sized(sphg_batch* b) {
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (int st = enqueue(b, b->stream)) return st;
    BCK(cudaStreamSynchronize(b->stream));
    const int nm = (int)b->maps.size();
    BCK(cudaMemcpy(b->h_status.data(), b->plan.d_status, nm * sizeof(DevStatus), cudaMemcpyDeviceToHost));
    bool grow = false;
    for (int m = 0; m < nm; ++m) {
      if (b->h_status[m].flags & kFlagNonFinite) return bfail(b, SPHG_ERR_NONFINITE, "map " + std::to_string(m));
      if (b->h_status[m].flags & kFlagTimeout) return bfail(b, SPHG_ERR_TIMEOUT, "map " + std::to_string(m));
      if (!(b->h_status[m].flags & kFlagOverflow)) continue;
      const TiledArgs& A = b->plan.args[m];
      long long total = 0, chunks = 0;
      int nl = 0;
      BCK(cudaMemcpy(&total, A.tile_start + A.n_tiles, sizeof(long long), cudaMemcpyDeviceToHost));
      BCK(cudaMemcpy(&nl, A.n_large, sizeof(int), cudaMemcpyDeviceToHost));
      BCK(cudaMemcpy(&chunks, A.large_start + nl, sizeof(long long), cudaMemcpyDeviceToHost));
      BatchMapHost& M = b->maps[m];
      if (total > M.pair_cap) M.pair_cap = total + total / 4 + 1024;
      if (chunks > M.chunk_cap) M.chunk_cap = chunks + chunks / 4 + 1024;
      grow = true;
    }
    if (!grow) return SPHG_OK;
    if (int st = build_plan(b)) return st;
  }
  return bfail(b, SPHG_ERR_ALLOC, "batch lists kept overflowing");
}

int capture(sphg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int st = enqueue(b, b->stream);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (st) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  BCK(e);
  b->graph = g;
  BCK(cudaGraphInstantiate(&b->exec, g, 0));
  return SPHG_OK;
}

float time_runs(sphg_batch* b, int reps) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  for (int r = 0; r < reps; ++r) enqueue(b, b->stream);
  cudaEventRecord(e1, b->stream);
  cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

}  // namespace
}  // namespace sphg

extern "C" {

int sphg_batch_create(sphg_context* ctx, int32_t n_maps, const sphg_map_desc* descs,
                      const sphg_batch_tuning* tuning, sphg_batch** out) {
  using namespace sphg;
  if (!out) return SPHG_ERR_ARG;
  *out = nullptr;
  if (!ctx || n_maps < 1 || !descs) return SPHG_ERR_ARG;
  sphg_batch* b = new sphg_batch();
  b->ctx = ctx;
  b->device = context_device(ctx);
  b->num_sms = context_num_sms(ctx);
  b->maps.resize(n_maps);
  b->h_status.resize(n_maps);
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != b->device) cudaSetDevice(b->device);
  auto done = [&](int st) {
    if (prev >= 0 && prev != b->device) cudaSetDevice(prev);
    if (st) {
      set_context_error(ctx, b->err);
      sphg_batch_destroy(b);
      return st;
    }
    *out = b;
    return st;
  };
  for (int m = 0; m < n_maps; ++m) {
    const sphg_map_desc& D = descs[m];
    const std::string who = "map " + std::to_string(m) + ": ";
    if (D.opt.dimensions != 2 && D.opt.dimensions != 3) return done(bfail(b, SPHG_ERR_DIMS, who));
    if (D.opt.precision != SPHG_PREC_FP32C) return done(bfail(b, SPHG_ERR_UNSUPPORTED, who + "batches map in FP32C"));
    if (D.opt.memspace != SPHG_MEM_DEVICE) return done(bfail(b, SPHG_ERR_UNSUPPORTED, who + "batches take device memory"));
    if (D.opt.center == SPHG_CENTER_INPLACE)
      return done(bfail(b, SPHG_ERR_UNSUPPORTED, who + "a replayed batch cannot centre in place"));
    if (D.opt.kernel < 0 || D.opt.kernel > 4 || (D.opt.kernel_dim != 2 && D.opt.kernel_dim != 3))
      return done(bfail(b, SPHG_ERR_ARG, who + "kernel"));
    if (D.parts.n_q < 1 || D.parts.n_q > kMaxQ || (D.opt.dimensions == 3 && D.parts.n_q != 1))
      return done(bfail(b, SPHG_ERR_NQ, who));
    if (D.parts.n < 0 || D.parts.n > (int64_t)1 << 30) return done(bfail(b, SPHG_ERR_ARG, who + "particle count"));
    if (D.parts.n > 0 && (!D.parts.pos || !D.parts.hsml || !D.parts.mass || !D.parts.rho || !D.parts.weights ||
                          !D.parts.bin_q))
      return done(bfail(b, SPHG_ERR_ARG, who + "NULL particle array"));
    if (!D.out) return done(bfail(b, SPHG_ERR_ARG, who + "NULL output"));
    const int64_t P = D.par.Npixels[0];
    if (P < 1 || P > ((int64_t)1 << 16) || (D.opt.dimensions == 3 && P > 2048))
      return done(bfail(b, SPHG_ERR_ARG, who + "Npixels"));
    BatchMapHost& M = b->maps[m];
    M.desc = D;
    const double* cen = D.par.center;
    const double xl[2] = {D.par.x_lim[0] - cen[0], D.par.x_lim[1] - cen[0]};
    const double yl[2] = {D.par.y_lim[0] - cen[1], D.par.y_lim[1] - cen[1]};
    const double zl[2] = {D.par.z_lim[0] - cen[2], D.par.z_lim[1] - cen[2]};
    const double c0[3] = {0.0, 0.0, 0.0};
    int64_t Pm = std::max(D.par.Npixels[0], std::max(D.par.Npixels[1], D.par.Npixels[2]));
    if (int st = sphg_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, Pm, D.par.boxsize, &M.cpar))
      return done(bfail(b, st, who + "parameters"));
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess)
    return done(bfail(b, SPHG_ERR_CUDA, "stream"));
  // tuning candidates (tile shape, deposit CTAs per SM, large-footprint threshold)
  struct Cand {
    int tx, ty, cps, large;
  };
  std::vector<Cand> cands;
  if (tuning) {
    cands.push_back({tuning->tile_x, tuning->tile_y, tuning->ctas_per_sm, tuning->large_cells});
  } else {
    for (int sh = 0; sh < 3; ++sh)
      for (int cps : {2, 4, 8})
        cands.push_back({sh == 0 ? 16 : 32, sh == 2 ? 32 : 16, cps, (int)kLargeCells});
    cands.push_back({16, 16, 4, 2048});
    cands.push_back({16, 16, 4, 32768});
  }
  const bool det = descs[0].opt.deterministic != 0;
  float best = 3.0e38f;
  Cand pick = cands[0];
  for (const Cand& c : cands) {
    if (c.cps < 1 || c.cps > 32 || c.large < 256)
      return done(bfail(b, SPHG_ERR_ARG, "tuning values"));
    b->plan.tile_x = c.tx;
    b->plan.tile_y = c.ty;
    b->plan.ctas_per_sm = c.cps;
    b->plan.large_cells = c.large;
    b->plan.det = det;
    for (sphg::BatchMapHost& M : b->maps) {
      const int dims = M.desc.opt.dimensions;
      const int64_t P = M.desc.par.Npixels[0];
      const int tdx = dims == 2 ? c.tx : kTile3X, tdy = dims == 2 ? c.ty : kTile3Y, tdz = dims == 2 ? 1 : kTile3Z;
      M.n_tiles = ((P + tdx - 1) / tdx) * ((P + tdy - 1) / tdy) * (dims == 3 ? (P + tdz - 1) / tdz : 1);
      const int64_t n = M.desc.parts.n;
      const long long guess = (dims == 2 ? 3 : 8) * n + M.n_tiles;  // overlaps, re-sized by run_sized
      if (M.pair_cap < guess) M.pair_cap = guess;
      if (M.chunk_cap < 4096) M.chunk_cap = 4096;
    }
    if (int st = sphg::build_plan(b)) return done(st);
    if (int st = sphg::run_sized(b)) return done(st);
    if (cands.size() == 1) break;
    const float ms = sphg::time_runs(b, 3);
    if (ms < best) {
      best = ms;
      pick = c;
    }
  }
  if (cands.size() > 1) {
    b->plan.tile_x = pick.tx;
    b->plan.tile_y = pick.ty;
    b->plan.ctas_per_sm = pick.cps;
    b->plan.large_cells = pick.large;
    for (sphg::BatchMapHost& M : b->maps) {
      const int dims = M.desc.opt.dimensions;
      const int64_t P = M.desc.par.Npixels[0];
      const int tdx = dims == 2 ? pick.tx : kTile3X, tdy = dims == 2 ? pick.ty : kTile3Y;
      M.n_tiles = ((P + tdx - 1) / tdx) * ((P + tdy - 1) / tdy) * (dims == 3 ? (P + kTile3Z - 1) / kTile3Z : 1);
    }
    if (int st = sphg::build_plan(b)) return done(st);
    if (int st = sphg::run_sized(b)) return done(st);
    b->tuned_ms = best;
  }
  // headroom for replays with slightly different inputs, then capture
  for (sphg::BatchMapHost& M : b->maps) {
    M.pair_cap += M.pair_cap / 4;
    M.chunk_cap += M.chunk_cap / 4;
  }
  if (int st = sphg::build_plan(b)) return done(st);
  if (int st = sphg::capture(b)) return done(st);
  return done(SPHG_OK);
}

int sphg_batch_launch(sphg_batch* b, void* stream) {
  if (!b || !b->exec) return SPHG_ERR_ARG;
  cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
  cudaError_t e = cudaGraphLaunch(b->exec, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return sphg::bfail(b, SPHG_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
  }
  b->last = s;
  return SPHG_OK;
}

int sphg_batch_wait(sphg_batch* b, sphg_stats* stats) {
  using namespace sphg;
  if (!b) return SPHG_ERR_ARG;
  if (b->last) BCK(cudaStreamSynchronize(b->last));
  const int nm = (int)b->maps.size();
  BCK(cudaMemcpy(b->h_status.data(), b->plan.d_status, nm * sizeof(DevStatus), cudaMemcpyDeviceToHost));
  bool overflow = false;
  for (int m = 0; m < nm; ++m) {
    if (b->h_status[m].flags & kFlagNonFinite) return bfail(b, SPHG_ERR_NONFINITE, "map " + std::to_string(m));
    if (b->h_status[m].flags & kFlagTimeout) return bfail(b, SPHG_ERR_TIMEOUT, "map " + std::to_string(m));
    if (b->h_status[m].flags & kFlagOverflow) overflow = true;
  }
  if (overflow) {  // inputs outgrew the captured lists: grow, re-run, re-capture
    if (int st = run_sized(b)) return st;
    if (int st = capture(b)) return st;
    BCK(cudaMemcpy(b->h_status.data(), b->plan.d_status, nm * sizeof(DevStatus), cudaMemcpyDeviceToHost));
  }
  if (stats) {
    for (int m = 0; m < nm; ++m) {
      sphg_stats& s = stats[m];
      std::memset(&s, 0, sizeof(s));
      s.n_in = b->maps[m].desc.parts.n;
      s.n_mapped = (int64_t)b->h_status[m].n_mapped;
      s.deposits = (int64_t)b->h_status[m].deposits;
      s.grid_mass = b->h_status[m].grid_mass;
      s.particle_mass = b->h_status[m].particle_mass;
      s.centred = b->maps[m].cpar;
      s.n_launches = 6;
      s.n_reruns = overflow ? 1 : 0;
    }
  }
  return SPHG_OK;
}

int sphg_batch_get_tuning(const sphg_batch* b, sphg_batch_tuning* t) {
  if (!b || !t) return SPHG_ERR_ARG;
  std::memset(t, 0, sizeof(*t));
  t->tile_x = b->plan.tile_x;
  t->tile_y = b->plan.tile_y;
  t->ctas_per_sm = b->plan.ctas_per_sm;
  t->large_cells = b->plan.large_cells;
  t->tuned_ms = b->tuned_ms;
  return SPHG_OK;
}

const char* sphg_batch_last_error(const sphg_batch* b) { return b ? b->err.c_str() : "NULL batch"; }

int sphg_batch_destroy(sphg_batch* b) {
  if (!b) return SPHG_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  sphg::free_plan(b->plan);
  if (b->side) cudaStreamSynchronize(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  delete b;
  return SPHG_OK;
}

}  // extern "C"
