// noalloc.cu -- sphg_map_noalloc: the FP32-compensated tiled map for callers
// that cannot allocate device memory.
//
// Who needs it: code that runs inside a host application owning all device
// memory through its own pool, e.g. a simulation that maps images in situ
// under a fixed memory budget, or a plugin whose host forbids allocations
// once a time step has started.  cudaMalloc/cudaFree there either fail or
// synchronise the device in the middle of the step.  This entry point calls
// neither (nor any allocating library routine): its scratch -- particle
// records, tile lists, the (particle, tile) pair records and the status word
// -- is one file-scope static __device__ array of kNoAllocScratchBytes.  Every
// GPU that loads the library holds that array until the process exits.
//
// Compiled with --fmad=false (see tiled_fp32.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/sphgrid.h"
#include "internal.h"
#include "tiled.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = (size_t)SPHG_NOALLOC_SCRATCH_BYTES;

// The shared scratch of every sphg_map_noalloc call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Per-device device address of the scratch (a host-side name of a __device__
// array is not a device address) and SM count, set up once per device.
struct DeviceSlot {
  bool ready = false;
  unsigned char* scratch = nullptr;
  int num_sms = 0;
};
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSlot g_slots[kMaxDevices];

int setup_device(int dev, DeviceSlot* out, std::string* err) {
  if (dev < 0 || dev >= kMaxDevices) {
    *err = "device index out of range";
    return SPHG_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSlot& s = g_slots[dev];
  if (!s.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // with `dev` current
    if (e != cudaSuccess) {
      cudaGetLastError();
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return e == cudaErrorNoKernelImageForDevice ? SPHG_ERR_NO_DEVICE : SPHG_ERR_CUDA;
    }
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) {
      cudaGetLastError();
      *err = std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e);
      return SPHG_ERR_CUDA;
    }
    s.scratch = (unsigned char*)p;
    s.num_sms = sms;
    s.ready = true;
  }
  *out = s;
  return SPHG_OK;
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

int nfail(int st, const std::string& msg) {
  sphg::set_thread_error(std::string(sphg_status_string(st)) + (msg.empty() ? "" : ": " + msg));
  return st;
}

// center_particles (filter_shift.jl:6-21) written back into the caller's
// array, after a map that centred on the fly: the same arithmetic as the
// mapping's centring (prep_particle_fp64), so the map and the array agree.
__global__ void __launch_bounds__(256) k_center_inplace(sphg::DevParticles pt, sphg::DevMapParams mp) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < pt.n; p += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int64_t off = p * pt.sp + d * pt.sc;
      double v = sphg::round_to(pt.pos_dtype, sphg::ld_elem(pt.pos_dtype, pt.pos, off) - mp.cen[d]);
      if (mp.periodic && fabs(v) > mp.boxsize / 2)
        v = sphg::round_to(pt.pos_dtype, v > 0 ? v - mp.boxsize / 2 : v + mp.boxsize / 2);
      sphg::st_elem(pt.pos_dtype, pt.pos, off, v);
    }
  }
}

}  // namespace

extern "C" {

int sphg_map_noalloc(const sphg_params* par, const sphg_options* opt, const sphg_particles* pt,
                     double* out, void* stream, sphg_stats* stats) {
  using namespace sphg;
  if (!par || !opt || !pt || !out) return nfail(SPHG_ERR_ARG, "NULL argument");
  const int dims = opt->dimensions;
  if (dims != 2 && dims != 3) return nfail(SPHG_ERR_DIMS, "");
  if (opt->precision != SPHG_PREC_FP32C) return nfail(SPHG_ERR_UNSUPPORTED, "maps in FP32C only");
  if (opt->memspace != SPHG_MEM_DEVICE) return nfail(SPHG_ERR_UNSUPPORTED, "takes device memory only");
  if (opt->center < 0 || opt->center > 2) return nfail(SPHG_ERR_ARG, "unknown center mode");
  for (int r = 0; r < 3; ++r)
    if (opt->reserved[r]) return nfail(SPHG_ERR_ARG, "reserved option fields must be 0");
  if (opt->kernel < 0 || opt->kernel > 4 || (opt->kernel_dim != 2 && opt->kernel_dim != 3))
    return nfail(SPHG_ERR_ARG, "kernel");
  const int nq = pt->n_q;
  if (nq < 1 || nq > kMaxQ) return nfail(SPHG_ERR_ARG, "n_q must be in 1..16");
  if (dims == 3 && nq != 1) return nfail(SPHG_ERR_NQ, "");
  if (pt->pos_dtype != SPHG_F32 && pt->pos_dtype != SPHG_F64) return nfail(SPHG_ERR_ARG, "dtype");
  if (pt->attr_dtype != SPHG_F32 && pt->attr_dtype != SPHG_F64) return nfail(SPHG_ERR_ARG, "dtype");
  const int64_t n = pt->n;
  if (n < 0) return nfail(SPHG_ERR_ARG, "negative particle count");
  if (n > ((int64_t)1 << 30)) return nfail(SPHG_ERR_ARG, "particle count exceeds the no-allocation scratch");
  if (n > 0 && (!pt->pos || !pt->hsml || !pt->mass || !pt->rho || !pt->weights || !pt->bin_q))
    return nfail(SPHG_ERR_ARG, "NULL particle array");
  if (pt->pos_stride_p < 0 || pt->pos_stride_c < 0 || pt->q_stride_p < 0 || pt->q_stride_k < 0)
    return nfail(SPHG_ERR_ARG, "negative stride");
  const int64_t P = par->Npixels[0];
  if (P < 1 || P > (int64_t)1 << 20 || (dims == 3 && P > 4096)) return nfail(SPHG_ERR_ARG, "Npixels out of range");

  sphg_params cpar;
  {
    const double* cen = par->center;
    const double xl[2] = {par->x_lim[0] - cen[0], par->x_lim[1] - cen[0]};
    const double yl[2] = {par->y_lim[0] - cen[1], par->y_lim[1] - cen[1]};
    const double zl[2] = {par->z_lim[0] - cen[2], par->z_lim[1] - cen[2]};
    const double c0[3] = {0.0, 0.0, 0.0};
    int64_t Pmax = par->Npixels[0];
    if (par->Npixels[1] > Pmax) Pmax = par->Npixels[1];
    if (par->Npixels[2] > Pmax) Pmax = par->Npixels[2];
    if (int st = sphg_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, Pmax, par->boxsize, &cpar))
      return st;
  }

  // scratch layout: fixed parts first, the remainder is split between the
  // (particle, tile) pair list and the large-footprint chunk partials
  TiledArgs ta;
  std::memset(&ta, 0, sizeof(ta));
  tiled_geometry(dims, P, ta.tdim, ta.ntile, &ta.n_tiles);
  const int64_t cap = n > 0 ? n : 1;
  size_t off = 0;
  auto take = [&](size_t b) {
    size_t o = off;
    off += al(b);
    return o;
  };
  const size_t o_stat = take(sizeof(DevStatus));
  const size_t o_box = take(cap * sizeof(int4)), o_dim = take(cap * sizeof(int4));
  const size_t o_geo = take(cap * sizeof(float4)), o_cp = take(cap * sizeof(double));
  const size_t o_cpm = take(cap * sizeof(float)), o_cpe = take(cap * sizeof(int));
  const size_t o_aux = take(cap * sizeof(double)), o_qv = take(cap * nq * sizeof(float));
  const size_t o_cnt = take(tiled_counter_ints(ta.n_tiles) * sizeof(int));
  const size_t o_start = take((ta.n_tiles + 1) * sizeof(long long));
  const size_t o_exps = take((kMaxQ + 1) * sizeof(int));
  const size_t o_large = take(cap * sizeof(int)), o_lstart = take((cap + 1) * sizeof(long long));
  if (off + al(4096 * sizeof(float4)) + al((size_t)ta.n_tiles * kPairRecBytes) > kNoAllocScratchBytes)
    return nfail(SPHG_ERR_ARG, std::to_string(n) + " particles on a " + std::to_string(P) + "^" +
                                   std::to_string(dims) + " grid exceed the " +
                                   std::to_string(kNoAllocScratchBytes >> 20) +
                                   " MiB no-allocation scratch (use sphg_map)");
  // the rest: an eighth for the large-footprint chunk partials, the remainder
  // for the (particle, tile) pair records
  const size_t rest = kNoAllocScratchBytes - off;
  const size_t chunk_bytes = al(std::max<size_t>(4096 * sizeof(float4), rest / 8 / sizeof(float4) * sizeof(float4)));
  const size_t o_part = take(chunk_bytes);
  const size_t pair_bytes = (kNoAllocScratchBytes - off) / kPairRecBytes * kPairRecBytes;
  const size_t o_pairs = off;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return nfail(SPHG_ERR_NO_DEVICE, "no current CUDA device");
  }
  DeviceSlot slot;
  std::string err;
  if (int st = setup_device(dev, &slot, &err)) return nfail(st, err);
  unsigned char* ws = slot.scratch;
  cudaStream_t s = (cudaStream_t)stream;

  DevParticles d;
  d.n = n;
  d.pos_dtype = pt->pos_dtype;
  d.attr_dtype = pt->attr_dtype;
  d.pos = pt->pos;
  d.sp = pt->pos_stride_p;
  d.sc = pt->pos_stride_c;
  d.hsml = pt->hsml;
  d.mass = pt->mass;
  d.rho = pt->rho;
  d.w = pt->weights;
  d.q = pt->bin_q;
  d.nq = nq;
  d.qsp = pt->q_stride_p;
  d.qsk = pt->q_stride_k;
  DevMapParams mp;
  for (int k = 0; k < 3; ++k) {
    mp.cen[k] = par->center[k];
    mp.lo[k] = cpar.center[k] - cpar.halfsize[k];
    mp.hi[k] = cpar.center[k] + cpar.halfsize[k];
  }
  mp.boxsize = par->boxsize;
  mp.periodic = par->periodic;
  // in-place centring is applied on the fly and written back only after a
  // map that succeeded: a call that fails (a full scratch) leaves the
  // caller's positions as they were, so a retry with the same options
  // (through sphg_map) centres them once
  const bool inplace = opt->center == SPHG_CENTER_INPLACE;
  mp.center_mode = inplace ? SPHG_CENTER_READONLY : opt->center;
  mp.filter = opt->filter;
  mp.calc_mean = dims == 2 ? opt->calc_mean : 0;
  mp.kernel_dim = opt->kernel_dim;
  mp.dims = dims;
  mp.L = cpar.len2pix;
  mp.P = P;
  mp.sigma = kernel_sigma(opt->kernel, opt->kernel_dim);
  set_lite_params(mp);

  DevStatus* d_status = (DevStatus*)(ws + o_stat);
  ta.pt = d;
  ta.mp = mp;
  ta.mp_re = mp;
  ta.kern = opt->kernel;
  ta.large_cells = (int)kLargeCells;
  ta.cap = cap;
  ta.box = (int4*)(ws + o_box);
  ta.dimv = (int4*)(ws + o_dim);
  ta.geo = (float4*)(ws + o_geo);
  ta.cp = (double*)(ws + o_cp);
  ta.cpm = (float*)(ws + o_cpm);
  ta.cpe = (int*)(ws + o_cpe);
  ta.aux = (double*)(ws + o_aux);
  ta.qv = (float*)(ws + o_qv);
  bind_counters(ta, (int*)(ws + o_cnt));
  ta.tile_start = (long long*)(ws + o_start);
  ta.prec = (uint4*)(ws + o_pairs);
  ta.pair_cap = (long long)(pair_bytes / kPairRecBytes);
  ta.exps = (int*)(ws + o_exps);
  ta.det = opt->deterministic ? 1 : 0;
  ta.large = (int*)(ws + o_large);
  ta.large_start = (long long*)(ws + o_lstart);
  ta.partials = (float4*)(ws + o_part);
  ta.chunk_cap = (long long)(chunk_bytes / sizeof(float4));
  ta.large_grid = slot.num_sms * 4;
  ta.st = d_status;
  ta.out = out;
  const bool raw_out = opt->raw_accumulator || (dims == 2 && opt->return_both_maps);
  ta.mode = raw_out ? 1 : (dims == 3 ? 2 : 0);
  ta.reduce = opt->reduce_image;
  ta.w_is_one = opt->reduce_image ? 0 : 1;

  // everything that accumulates starts from zero (the scratch keeps the last
  // call's contents)
  cudaError_t e = cudaMemsetAsync(d_status, 0, sizeof(DevStatus), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ta.tile_count, 0, tiled_counter_ints(ta.n_tiles) * sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ta.exps, 0x80, (kMaxQ + 1) * sizeof(int), s);
  int n_launch = 0;
  if (e == cudaSuccess) e = launch_tiled_fp32(opt->kernel, ta, slot.num_sms, s, nullptr, &n_launch);
  DevStatus hs;
  std::memset(&hs, 0, sizeof(hs));
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, d_status, sizeof(DevStatus), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return nfail(SPHG_ERR_CUDA, cudaGetErrorString(e));
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->n_in = n;
    stats->n_mapped = (int64_t)hs.n_mapped;
    stats->deposits = (int64_t)hs.deposits;
    stats->grid_mass = hs.grid_mass;
    stats->particle_mass = hs.particle_mass;
    stats->centred = cpar;
    stats->n_launches = n_launch;
  }
  const bool full = (hs.flags & kFlagOverflow) && !(hs.flags & kFlagNonFinite);
  if (inplace && n > 0 && !full) {
    // the reference centres before it maps (and before it meets a
    // non-finite value), so a finished map or a non-finite input leaves
    // the caller's positions centred
    int grid = (int)std::min<int64_t>((n + 255) / 256, (int64_t)slot.num_sms * 8);
    k_center_inplace<<<grid, 256, 0, s>>>(d, mp);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return nfail(SPHG_ERR_CUDA, cudaGetErrorString(e));
    }
    if (stats) stats->n_launches += 1;
  }
  if (hs.flags & kFlagNonFinite) return nfail(SPHG_ERR_NONFINITE, "");
  if (hs.flags & kFlagTimeout) return nfail(SPHG_ERR_TIMEOUT, "");
  if (full)
    return nfail(SPHG_ERR_ALLOC,
                 "more (particle, tile) overlaps than the no-allocation scratch holds (use sphg_map; the "
                 "positions were left uncentred)");
  sphg::set_thread_error("");
  return SPHG_OK;
}

}  // extern "C"
