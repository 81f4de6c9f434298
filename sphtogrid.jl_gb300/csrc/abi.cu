// abi.cu -- host side of the C ABI declared in include/sphgrid.h: contexts,
// the mappingParameters constructor, argument checks, staging of host arrays
// and dispatch to the deposition kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/sphgrid.h"
#include "common.cuh"
#include "internal.h"

struct sphg_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  void* ws = nullptr;  // grow-only device workspace
  size_t ws_size = 0;
  sphg::DevStatus* d_status = nullptr;
  sphg::DevStatus* h_status = nullptr;  // pinned
  size_t pair_cap = 0;                  // FP32C tile-pair list capacity (grow-only)
  size_t chunk_cap = 0;                 // FP32C large-record chunk capacity (grow-only)
  cudaEvent_t ev[5] = {};               // phase timing events
  double* hp_centres = nullptr;         // HEALPix pixel-centre table of hp_nside
  int64_t hp_nside = 0;
  double* hp_dist = nullptr;            // HEALPix per-warp distance slices (pass 1 -> pass 2)
  int hp_dist_per_lane = 0;
};

namespace {

thread_local std::string g_error;  // errors raised before a context exists

const char* kStatusText[] = {
    "ok",
    "Giving a center position requires extent in x, y and z direction.",
    "Please specify pixelSideLength or number of pixels!",
    "dimensions must be 2 or 3",
    "non-finite pixel range of a mapped particle (InexactError in floor)",
    "3D mapping takes exactly one scalar quantity",
    "allocation failed",
    "invalid argument",
    "CUDA error",
    "device work queue timed out",
    "no usable CUDA device",
    "unsupported option combination",
};

int fail(sphg_context* ctx, int status, const std::string& msg) {
  std::string m = std::string(sphg_status_string(status)) + (msg.empty() ? "" : ": " + msg);
  if (ctx) ctx->last_error = m;
  else g_error = m;
  return status;
}

int cuda_fail(sphg_context* ctx, cudaError_t e, const char* where) {
  cudaGetLastError();
  return fail(ctx, e == cudaErrorNoKernelImageForDevice ? SPHG_ERR_NO_DEVICE : SPHG_ERR_CUDA,
              std::string(where) + ": " + cudaGetErrorString(e));
}

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call);  \
  } while (0)

// Keeps the caller's current device around a call.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

int ensure_ws(sphg_context* ctx, size_t bytes, cudaStream_t s) {
  if (bytes <= ctx->ws_size) return SPHG_OK;
  if (ctx->ws) {
    CK(cudaStreamSynchronize(s));
    CK(cudaFree(ctx->ws));
    ctx->ws = nullptr;
    ctx->ws_size = 0;
  }
  size_t want = bytes + bytes / 4 + (1u << 20);
  cudaError_t e = cudaMalloc(&ctx->ws, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&ctx->ws, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      ctx->ws = nullptr;
      return fail(ctx, SPHG_ERR_ALLOC, "device workspace of " + std::to_string(bytes) + " bytes");
    }
    want = bytes;
  }
  ctx->ws_size = want;
  return SPHG_OK;
}

// Bump allocator over the workspace (256-byte aligned slices).
struct Carve {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  }
};

size_t dtype_size(int dt) { return dt == SPHG_F32 ? 4 : 8; }

bool valid_dtype(int dt) { return dt == SPHG_F32 || dt == SPHG_F64; }

}  // namespace

namespace sphg {
int context_device(sphg_context* ctx) { return ctx->device; }
int context_num_sms(sphg_context* ctx) { return ctx->num_sms; }
void set_context_error(sphg_context* ctx, const std::string& msg) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  ctx->last_error = msg;
}
void set_thread_error(const std::string& msg) { g_error = msg; }
}  // namespace sphg

extern "C" {

int sphg_abi_version(void) { return SPHG_ABI_VERSION; }

const char* sphg_status_string(int status) {
  if (status < 0 || status > SPHG_ERR_UNSUPPORTED) return "unknown status";
  return kStatusText[status];
}

const char* sphg_last_error(const sphg_context* ctx) {
  if (!ctx) return g_error.c_str();
  return ctx->last_error.c_str();
}

int sphg_context_create(int device, sphg_context** out) {
  if (!out) return fail(nullptr, SPHG_ERR_ARG, "out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(nullptr, SPHG_ERR_NO_DEVICE, e != cudaSuccess ? cudaGetErrorString(e) : "no device");
  }
  if (device < 0 || device >= count) return fail(nullptr, SPHG_ERR_ARG, "device index out of range");
  DeviceGuard g(device);
  sphg_context* ctx = new sphg_context();
  ctx->device = device;
  auto bail = [&](cudaError_t err, const char* where) {
    int st = cuda_fail(nullptr, err, where);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    delete ctx;
    return st;
  };
  if ((e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
    return bail(e, "cudaDeviceGetAttribute");
  cudaFuncAttributes fa;
  if ((e = sphg::probe_kernel_image(&fa)) != cudaSuccess) return bail(e, "kernel image for this device");
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  if ((e = cudaMalloc(&ctx->d_status, sizeof(sphg::DevStatus))) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMallocHost(&ctx->h_status, sizeof(sphg::DevStatus))) != cudaSuccess)
    return bail(e, "cudaMallocHost");
  for (int k = 0; k < 5; ++k)
    if ((e = cudaEventCreate(&ctx->ev[k])) != cudaSuccess) return bail(e, "cudaEventCreate");
  *out = ctx;
  return SPHG_OK;
}

int sphg_context_destroy(sphg_context* ctx) {
  if (!ctx) return SPHG_OK;
  {
    DeviceGuard g(ctx->device);
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->ws) cudaFree(ctx->ws);
    if (ctx->hp_centres) cudaFree(ctx->hp_centres);
    if (ctx->hp_dist) cudaFree(ctx->hp_dist);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->h_status) cudaFreeHost(ctx->h_status);
    for (int k = 0; k < 5; ++k)
      if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
  return SPHG_OK;
}

// mappingParameters constructor, parameters.jl:44-125.
int sphg_mapping_parameters(const double x_lim_in[2], const double y_lim_in[2], const double z_lim_in[2],
                            const double center_in[3], double x_size, double y_size, double z_size,
                            double pixelSideLength, int64_t Npixels, double boxsize, sphg_params* out) {
  if (!x_lim_in || !y_lim_in || !z_lim_in || !center_in || !out)
    return fail(nullptr, SPHG_ERR_ARG, "NULL argument");
  double xl[2] = {x_lim_in[0], x_lim_in[1]}, yl[2] = {y_lim_in[0], y_lim_in[1]};
  double zl[2] = {z_lim_in[0], z_lim_in[1]};
  double c[3] = {center_in[0], center_in[1], center_in[2]};
  const bool xl_def = xl[0] == -1.0 && xl[1] == -1.0;
  const bool yl_def = yl[0] == -1.0 && yl[1] == -1.0;
  const bool zl_def = zl[0] == -1.0 && zl[1] == -1.0;
  const bool c_def = c[0] == -1.0 && c[1] == -1.0 && c[2] == -1.0;
  if (xl_def && yl_def && zl_def) {  // limits from centre and sizes (:58-69)
    if (!c_def && x_size != -1.0 && y_size != -1.0 && z_size != -1.0) {
      xl[0] = c[0] - 0.5 * x_size; xl[1] = c[0] + 0.5 * x_size;
      yl[0] = c[1] - 0.5 * y_size; yl[1] = c[1] + 0.5 * y_size;
      zl[0] = c[2] - 0.5 * z_size; zl[1] = c[2] + 0.5 * z_size;
    } else {
      return fail(nullptr, SPHG_ERR_CENTER_EXTENT, "");
    }
  }
  if (x_size == -1.0) x_size = xl[1] - xl[0];  // :72-80
  if (y_size == -1.0) y_size = yl[1] - yl[0];
  if (z_size == -1.0) z_size = zl[1] - zl[0];
  if (c_def) {  // :82-86
    c[0] = xl[0] + 0.5 * x_size;
    c[1] = yl[0] + 0.5 * y_size;
    c[2] = zl[0] + 0.5 * z_size;
  }
  double max_size = (std::isnan(x_size) || std::isnan(y_size)) ? NAN : (x_size > y_size ? x_size : y_size);
  if (pixelSideLength == -1.0 && Npixels != 0) {  // :91-99
    pixelSideLength = max_size / (double)Npixels;
  } else if (pixelSideLength != -1.0 && Npixels == 0) {
    double np = std::floor(max_size / pixelSideLength);
    if (!(std::fabs(np) < 9.2e18)) return fail(nullptr, SPHG_ERR_ARG, "Npixels not representable");
    Npixels = (int64_t)np;
    pixelSideLength = max_size / (double)Npixels;
  } else {
    return fail(nullptr, SPHG_ERR_PIXELS, "");
  }
  std::memset(out, 0, sizeof(*out));
  std::memcpy(out->x_lim, xl, sizeof(xl));
  std::memcpy(out->y_lim, yl, sizeof(yl));
  std::memcpy(out->z_lim, zl, sizeof(zl));
  std::memcpy(out->center, c, sizeof(c));
  out->halfsize[0] = 0.5 * x_size;  // :113
  out->halfsize[1] = 0.5 * y_size;
  out->halfsize[2] = 0.5 * z_size;
  out->len2pix = 1.0 / pixelSideLength;  // :115
  out->pixelSideLength = pixelSideLength;
  out->Npixels[0] = out->Npixels[1] = out->Npixels[2] = Npixels;
  out->boxsize = boxsize;
  out->periodic = boxsize != -1.0 ? 1 : 0;
  return SPHG_OK;
}

int64_t sphg_output_len(const sphg_params* par, const sphg_options* opt, int32_t n_q) {
  if (!par || !opt) return -1;
  const int64_t P = par->Npixels[0];
  const bool raw = opt->raw_accumulator || (opt->dimensions == 2 && opt->return_both_maps);
  if (opt->dimensions == 2) return raw ? P * P * (n_q + 1) : P * P * n_q;
  if (opt->dimensions == 3) return raw ? 2 * P * P * P : P * P * P;
  return -1;
}

namespace {
// Device address of page-locked (pinned) host memory, or NULL (pageable
// memory, or not host memory).
void* mapped_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// sphg_map with an optional position transform (xform: 0 none, 1 axis
// permutation `perm`, 2 FP64 matrix `rot`; see sphg::DevParticles).
int map_impl(sphg_context* ctx, const sphg_params* par, const sphg_options* opt, const sphg_particles* pt,
             int xform, const int* perm, const double* rot, double* out, void* stream, sphg_stats* stats) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!par || !opt || !pt || !out) return fail(ctx, SPHG_ERR_ARG, "NULL argument");
  const int dims = opt->dimensions;
  if (dims != 2 && dims != 3) return fail(ctx, SPHG_ERR_DIMS, "");
  const int nq = pt->n_q;
  if (nq < 1 || nq > sphg::kMaxQ) return fail(ctx, SPHG_ERR_ARG, "n_q must be in 1..16");
  if (dims == 3 && nq != 1) return fail(ctx, SPHG_ERR_NQ, "");
  if (opt->kernel < 0 || opt->kernel > 4) return fail(ctx, SPHG_ERR_ARG, "unknown kernel");
  if (opt->kernel_dim != 2 && opt->kernel_dim != 3) return fail(ctx, SPHG_ERR_ARG, "kernel_dim must be 2 or 3");
  if (opt->precision != SPHG_PREC_FP64 && opt->precision != SPHG_PREC_FP32C)
    return fail(ctx, SPHG_ERR_ARG, "unknown precision");
  if (opt->center < 0 || opt->center > 2) return fail(ctx, SPHG_ERR_ARG, "unknown center mode");
  if (opt->memspace != SPHG_MEM_DEVICE && opt->memspace != SPHG_MEM_HOST)
    return fail(ctx, SPHG_ERR_ARG, "unknown memspace");
  for (int r = 0; r < 3; ++r)
    if (opt->reserved[r]) return fail(ctx, SPHG_ERR_ARG, "reserved option fields must be 0");
  if (!valid_dtype(pt->pos_dtype) || !valid_dtype(pt->attr_dtype)) return fail(ctx, SPHG_ERR_ARG, "dtype");
  const int64_t n = pt->n;
  if (n < 0) return fail(ctx, SPHG_ERR_ARG, "negative particle count");
  if (n > 0 && (!pt->pos || !pt->hsml || !pt->mass || !pt->rho || !pt->weights || !pt->bin_q))
    return fail(ctx, SPHG_ERR_ARG, "NULL particle array");
  if (pt->pos_stride_p < 0 || pt->pos_stride_c < 0 || pt->q_stride_p < 0 || pt->q_stride_k < 0)
    return fail(ctx, SPHG_ERR_ARG, "negative stride");
  const int64_t P = par->Npixels[0];
  if (P < 1 || P > (int64_t)1 << 20 || (dims == 3 && P > 4096))
    return fail(ctx, SPHG_ERR_ARG, "Npixels out of range");
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  const int64_t out_len = sphg_output_len(par, opt, nq);

  // centred parameters, re-derived as center_particles does (filter_shift.jl:25-31)
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
    int st = sphg_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, Pmax, par->boxsize, &cpar);
    if (st) return fail(ctx, st, g_error);
  }

  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  const bool host = opt->memspace == SPHG_MEM_HOST;
  const bool fp32c = opt->precision == SPHG_PREC_FP32C;
  const bool raw_out = opt->raw_accumulator || (dims == 2 && opt->return_both_maps);
  const size_t psz = dtype_size(pt->pos_dtype), asz = dtype_size(pt->attr_dtype);
  const int64_t pos_span = n > 0 ? (n - 1) * pt->pos_stride_p + 2 * pt->pos_stride_c + 1 : 0;
  const int64_t q_span = n > 0 ? (n - 1) * pt->q_stride_p + (int64_t)(nq - 1) * pt->q_stride_k + 1 : 0;
  // Pinned host buffers on the FP32C path are used in place over the host
  // link: K1 reads each particle once (and writes the in-place centring
  // back), the deposit writes each output value once, so the transfers
  // overlap the kernels instead of preceding and following them.
  void* zc[7] = {};
  bool zero_copy = false;
  if (host && fp32c && n > 0) {
    const void* hp[7] = {pt->pos, pt->hsml, pt->mass, pt->rho, pt->weights, pt->bin_q, out};
    zero_copy = true;
    for (int k = 0; k < 7 && zero_copy; ++k) zero_copy = (zc[k] = mapped_ptr(hp[k])) != nullptr;
  }
  const bool staged = host && !zero_copy;  // inputs copied into the workspace, output copied back

  sphg::TiledArgs ta;
  std::memset(&ta, 0, sizeof(ta));
  if (fp32c) sphg::tiled_geometry(dims, P, ta.tdim, ta.ntile, &ta.n_tiles);
  int rerun = 0;
  long long pair_cap = (long long)ctx->pair_cap;
  // first guess of the (particle, tile) overlaps (64-byte pair records): a
  // 2D footprint meets about 1.5 tiles, a 3D one 3-7; more re-runs once
  // with the exact count, which the context keeps
  const long long guess = (dims == 2 ? 3 : 8) * n + ta.n_tiles;
  if (fp32c && pair_cap < guess) pair_cap = guess;
  long long chunk_cap = (long long)ctx->chunk_cap;
  if (fp32c && chunk_cap < 4096) chunk_cap = 4096;

again:
  // workspace layout
  Carve cv;
  size_t o_pos = 0, o_h = 0, o_m = 0, o_r = 0, o_w = 0, o_q = 0, o_out = 0;
  if (staged) {
    o_pos = cv.take(pos_span * psz);
    o_h = cv.take(n * asz);
    o_m = cv.take(n * asz);
    o_r = cv.take(n * asz);
    o_w = cv.take(n * asz);
    o_q = cv.take(q_span * asz);
    o_out = cv.take(out_len * sizeof(double));
  }
  // FP64 path accumulator: 2D raw maps accumulate straight into the output,
  // 3D keeps Q in the output and only the weight channel in the workspace.
  const bool acc_in_out = raw_out || dims == 3;
  size_t o_acc = 0;
  if (!fp32c) o_acc = cv.take((acc_in_out ? (dims == 3 && !raw_out ? PD : 0) : PD * (nq + 1)) * sizeof(double));
  size_t o_box = 0, o_dim = 0, o_geo = 0, o_cp = 0, o_aux = 0, o_qv = 0, o_cnt = 0, o_start = 0,
         o_pairs = 0, o_exps = 0, o_large = 0, o_lstart = 0, o_part = 0, o_cpm = 0, o_cpe = 0;
  const int64_t cap = n > 0 ? n : 1;
  if (fp32c) {
    o_box = cv.take(cap * sizeof(int4));
    o_dim = cv.take(cap * sizeof(int4));
    o_geo = cv.take(cap * sizeof(float4));
    o_cp = cv.take(cap * sizeof(double));
    o_cpm = cv.take(cap * sizeof(float));
    o_cpe = cv.take(cap * sizeof(int));
    o_aux = cv.take(cap * sizeof(double));
    o_qv = cv.take(cap * nq * sizeof(float));
    o_cnt = cv.take(sphg::tiled_counter_ints(ta.n_tiles) * sizeof(int));  // tile counts and fills, record counters
    o_start = cv.take((ta.n_tiles + 1) * sizeof(long long));
    o_pairs = cv.take(pair_cap * sphg::kPairRecBytes);
    o_exps = cv.take((sphg::kMaxQ + 1) * sizeof(int));
    o_large = cv.take(cap * sizeof(int));
    o_lstart = cv.take((cap + 1) * sizeof(long long));
    o_part = cv.take(chunk_cap * sizeof(float4));
  }
  if (int st = ensure_ws(ctx, cv.off, s)) return st;
  char* ws = (char*)ctx->ws;

  sphg::DevParticles d;
  d.n = n;
  d.pos_dtype = pt->pos_dtype;
  d.attr_dtype = pt->attr_dtype;
  d.sp = pt->pos_stride_p;
  d.sc = pt->pos_stride_c;
  d.nq = nq;
  d.qsp = pt->q_stride_p;
  d.qsk = pt->q_stride_k;
  d.xform = xform;
  for (int k = 0; k < 3; ++k) d.perm[k] = perm ? perm[k] : k;
  for (int k = 0; k < 9; ++k) d.rot[k] = rot ? rot[k] : 0.0;
  double* dout = out;
  if (zero_copy) {
    d.pos = zc[0];
    d.hsml = zc[1];
    d.mass = zc[2];
    d.rho = zc[3];
    d.w = zc[4];
    d.q = zc[5];
    dout = (double*)zc[6];
  } else if (host) {
    d.pos = ws + o_pos;
    d.hsml = ws + o_h;
    d.mass = ws + o_m;
    d.rho = ws + o_r;
    d.w = ws + o_w;
    d.q = ws + o_q;
    dout = (double*)(ws + o_out);
    if (n > 0) {  // every pass: a re-run may have reallocated the workspace
      CK(cudaMemcpyAsync(ws + o_pos, pt->pos, pos_span * psz, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(ws + o_h, pt->hsml, n * asz, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(ws + o_m, pt->mass, n * asz, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(ws + o_r, pt->rho, n * asz, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(ws + o_w, pt->weights, n * asz, cudaMemcpyHostToDevice, s));
      CK(cudaMemcpyAsync(ws + o_q, pt->bin_q, q_span * asz, cudaMemcpyHostToDevice, s));
    }
  } else {
    d.pos = pt->pos;
    d.hsml = pt->hsml;
    d.mass = pt->mass;
    d.rho = pt->rho;
    d.w = pt->weights;
    d.q = pt->bin_q;
  }

  sphg::DevMapParams mp;
  for (int k = 0; k < 3; ++k) {
    mp.cen[k] = par->center[k];
    mp.lo[k] = cpar.center[k] - cpar.halfsize[k];
    mp.hi[k] = cpar.center[k] + cpar.halfsize[k];
  }
  mp.boxsize = par->boxsize;
  mp.periodic = par->periodic;
  mp.center_mode = opt->center;
  // a re-run must not centre again: K1 already centred the caller's
  // positions in place (device inputs), or the first pass wrote the centred
  // positions back into the caller's host array, from which they are copied
  if (rerun && opt->center == SPHG_CENTER_INPLACE) mp.center_mode = SPHG_CENTER_NONE;
  mp.filter = opt->filter;
  mp.calc_mean = dims == 2 ? opt->calc_mean : 0;  // cic_mapping_3D gets no calc_mean (:219)
  mp.kernel_dim = opt->kernel_dim;
  mp.dims = dims;
  mp.L = cpar.len2pix;
  mp.P = P;
  mp.sigma = sphg::kernel_sigma(opt->kernel, opt->kernel_dim);
  sphg::set_lite_params(mp);

  cudaEvent_t* ev = opt->profile ? ctx->ev : nullptr;
  int n_launch = 0;
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(sphg::DevStatus), s));
  if (!fp32c) {
    double* acc;  // (nq+1) channels of PD doubles
    double* acc_w;
    if (raw_out) {
      acc = dout;
      acc_w = dout + (int64_t)nq * PD;
    } else if (dims == 3) {
      acc = dout;
      acc_w = (double*)(ws + o_acc);
    } else {
      acc = (double*)(ws + o_acc);
      acc_w = acc + (int64_t)nq * PD;
    }
    if (dims == 3 && !raw_out) {
      CK(cudaMemsetAsync(acc, 0, PD * sizeof(double), s));
      CK(cudaMemsetAsync(acc_w, 0, PD * sizeof(double), s));
    } else {
      CK(cudaMemsetAsync(acc, 0, PD * (nq + 1) * sizeof(double), s));
    }
    if (ev) {
      CK(cudaEventRecord(ev[0], s));
      CK(cudaEventRecord(ev[1], s));
      CK(cudaEventRecord(ev[2], s));
    }
    sphg::launch_plain_fp64(opt->kernel, d, mp, acc, acc_w, PD, ctx->d_status, ctx->num_sms, s);
    CK(cudaGetLastError());
    if (ev) CK(cudaEventRecord(ev[3], s));
    if (!raw_out) {
      if (dims == 2) sphg::launch_reduce_2d(acc, P, nq, opt->reduce_image, dout, s);
      else sphg::launch_reduce_3d(acc, acc_w, PD, opt->reduce_image ? 0 : 1, dout, ctx->num_sms, s);
    }
    CK(cudaGetLastError());
    if (ev) CK(cudaEventRecord(ev[4], s));
    n_launch = raw_out ? 1 : 2;
  } else {
    ta.pt = d;
    ta.mp = mp;
    ta.mp_re = mp;
    if (ta.mp_re.center_mode == SPHG_CENTER_INPLACE) ta.mp_re.center_mode = SPHG_CENTER_NONE;
    ta.cap = cap;
    ta.box = (int4*)(ws + o_box);
    ta.dimv = (int4*)(ws + o_dim);
    ta.geo = (float4*)(ws + o_geo);
    ta.cp = (double*)(ws + o_cp);
    ta.cpm = (float*)(ws + o_cpm);
    ta.cpe = (int*)(ws + o_cpe);
    ta.aux = (double*)(ws + o_aux);
    ta.qv = (float*)(ws + o_qv);
    sphg::bind_counters(ta, (int*)(ws + o_cnt));
    ta.tile_start = (long long*)(ws + o_start);
    ta.prec = (uint4*)(ws + o_pairs);
    ta.pair_cap = pair_cap;
    ta.exps = (int*)(ws + o_exps);
    ta.det = opt->deterministic ? 1 : 0;
    ta.large = (int*)(ws + o_large);
    ta.large_start = (long long*)(ws + o_lstart);
    ta.partials = (float4*)(ws + o_part);
    ta.chunk_cap = chunk_cap;
    ta.large_grid = ctx->num_sms * 4;
    ta.kern = opt->kernel;
    ta.large_cells = (int)sphg::kLargeCells;
    ta.st = ctx->d_status;
    ta.out = dout;
    ta.mode = raw_out ? 1 : (dims == 3 ? 2 : 0);
    ta.reduce = opt->reduce_image;
    ta.w_is_one = opt->reduce_image ? 0 : 1;
    CK(cudaMemsetAsync(ta.tile_count, 0, sphg::tiled_counter_ints(ta.n_tiles) * sizeof(int), s));
    CK(cudaMemsetAsync(ta.exps, 0x80, (sphg::kMaxQ + 1) * sizeof(int), s));
    CK(sphg::launch_tiled_fp32(opt->kernel, ta, ctx->num_sms, s, ev, &n_launch));
    if (ev) CK(cudaEventRecord(ev[4], s));
  }
  if (staged) {
    CK(cudaMemcpyAsync(out, dout, out_len * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (opt->center == SPHG_CENTER_INPLACE && n > 0)
      CK(cudaMemcpyAsync(pt->pos, d.pos, pos_span * psz, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(sphg::DevStatus), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const sphg::DevStatus hs = *ctx->h_status;
  if (fp32c && (hs.flags & sphg::kFlagOverflow) && !(hs.flags & sphg::kFlagNonFinite)) {
    // more (particle, tile) pairs or large-record chunks than the lists hold:
    // grow them and map again
    long long total = 0, chunks = 0;
    int nl = 0;
    CK(cudaMemcpy(&total, ta.tile_start + ta.n_tiles, sizeof(long long), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&nl, ta.n_large, sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(&chunks, ta.large_start + nl, sizeof(long long), cudaMemcpyDeviceToHost));
    if (total > pair_cap) pair_cap = total + total / 8 + 1024;
    if (chunks > chunk_cap) chunk_cap = chunks + chunks / 8 + 1024;
    ctx->pair_cap = (size_t)pair_cap;
    ctx->chunk_cap = (size_t)chunk_cap;
    if (++rerun > 2) return fail(ctx, SPHG_ERR_ALLOC, "tile-pair list kept overflowing");
    goto again;
  }
  if (fp32c && (size_t)pair_cap > ctx->pair_cap) ctx->pair_cap = (size_t)pair_cap;
  if (fp32c && (size_t)chunk_cap > ctx->chunk_cap) ctx->chunk_cap = (size_t)chunk_cap;
  if (stats) {
    stats->n_in = n;
    stats->n_mapped = (int64_t)hs.n_mapped;
    stats->deposits = (int64_t)hs.deposits;
    stats->grid_mass = hs.grid_mass;
    stats->particle_mass = hs.particle_mass;
    stats->centred = cpar;
    stats->n_launches = n_launch;
    stats->n_reruns = rerun;
    for (int k = 0; k < 4; ++k) stats->phase_ms[k] = 0.0f;
    if (ev)
      for (int k = 0; k < 4; ++k) cudaEventElapsedTime(&stats->phase_ms[k], ev[k], ev[k + 1]);
  }
  if (hs.flags & sphg::kFlagNonFinite) return fail(ctx, SPHG_ERR_NONFINITE, "");
  if (hs.flags & sphg::kFlagTimeout) return fail(ctx, SPHG_ERR_TIMEOUT, "");
  ctx->last_error.clear();
  return SPHG_OK;
}
}  // namespace

int sphg_map(sphg_context* ctx, const sphg_params* par, const sphg_options* opt, const sphg_particles* pt,
             double* out, void* stream, sphg_stats* stats) {
  return map_impl(ctx, par, opt, pt, 0, nullptr, nullptr, out, stream, stats);
}

int sphg_map_projected(sphg_context* ctx, const sphg_params* par, const sphg_options* opt,
                       const sphg_particles* pt, const sphg_projection* proj, double* out, void* stream,
                       sphg_stats* stats) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  if (!par || !opt || !proj) return fail(ctx, SPHG_ERR_ARG, "NULL argument");
  if (proj->reserved) return fail(ctx, SPHG_ERR_ARG, "reserved projection field must be 0");
  sphg_options o = *opt;  // map_it maps a copy: the caller's positions stay as they are
  if (o.center == SPHG_CENTER_INPLACE) o.center = SPHG_CENTER_READONLY;
  if (proj->kind == SPHG_PROJ_XY) return map_impl(ctx, par, &o, pt, 0, nullptr, nullptr, out, stream, stats);
  if (proj->kind == SPHG_PROJ_MATRIX) {
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(proj->matrix[k])) return fail(ctx, SPHG_ERR_ARG, "projection matrix not finite");
    return map_impl(ctx, par, &o, pt, 2, nullptr, proj->matrix, out, stream, stats);
  }
  if (proj->kind != SPHG_PROJ_XZ && proj->kind != SPHG_PROJ_YZ) return fail(ctx, SPHG_ERR_ARG, "projection kind");
  // rotate_to_xz_plane / rotate_to_yz_plane of the parameters
  // (rotate_parameters.jl:6-40): permuted centre and limits, the largest
  // Npixels, the same boxsize
  const int xz = proj->kind == SPHG_PROJ_XZ;
  const int perm[3] = {xz ? 0 : 1, 2, xz ? 1 : 0};
  const double* lims[3] = {par->x_lim, par->y_lim, par->z_lim};
  const double cen[3] = {par->center[perm[0]], par->center[perm[1]], par->center[perm[2]]};
  int64_t npix = par->Npixels[0];
  for (int k = 1; k < 3; ++k) npix = par->Npixels[k] > npix ? par->Npixels[k] : npix;
  sphg_params rp;
  const double m1 = -1.0;
  if (int st = sphg_mapping_parameters(lims[perm[0]], lims[perm[1]], lims[perm[2]], cen, m1, m1, m1, m1, npix,
                                       par->boxsize, &rp))
    return fail(ctx, st, "rotated parameters");
  return map_impl(ctx, &rp, &o, pt, 1, perm, nullptr, out, stream, stats);
}

int sphg_footprints(sphg_context* ctx, const sphg_params* par, const sphg_options* opt, const sphg_particles* pt,
                    int64_t* ranges, int8_t* state, void* stream) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!par || !opt || !pt || (pt->n > 0 && (!ranges || !state))) return fail(ctx, SPHG_ERR_ARG, "NULL argument");
  const int dims = opt->dimensions;
  if (dims != 2 && dims != 3) return fail(ctx, SPHG_ERR_DIMS, "");
  const int nq = pt->n_q;
  if (nq < 1 || nq > sphg::kMaxQ) return fail(ctx, SPHG_ERR_ARG, "n_q must be in 1..16");
  if (opt->center < 0 || opt->center > 2) return fail(ctx, SPHG_ERR_ARG, "unknown center mode");
  if (opt->memspace != SPHG_MEM_DEVICE) return fail(ctx, SPHG_ERR_UNSUPPORTED, "footprints take device memory");
  if (!valid_dtype(pt->pos_dtype) || !valid_dtype(pt->attr_dtype)) return fail(ctx, SPHG_ERR_ARG, "dtype");
  const int64_t n = pt->n;
  if (n < 0) return fail(ctx, SPHG_ERR_ARG, "negative particle count");
  if (n > 0 && (!pt->pos || !pt->hsml || !pt->bin_q)) return fail(ctx, SPHG_ERR_ARG, "NULL particle array");
  if (pt->pos_stride_p < 0 || pt->pos_stride_c < 0 || pt->q_stride_p < 0 || pt->q_stride_k < 0)
    return fail(ctx, SPHG_ERR_ARG, "negative stride");
  const int64_t P = par->Npixels[0];
  if (P < 1 || P > (int64_t)1 << 20 || (dims == 3 && P > 4096)) return fail(ctx, SPHG_ERR_ARG, "Npixels out of range");
  sphg_params cpar;  // centred parameters, as sphg_map derives them
  {
    const double* cen = par->center;
    const double xl[2] = {par->x_lim[0] - cen[0], par->x_lim[1] - cen[0]};
    const double yl[2] = {par->y_lim[0] - cen[1], par->y_lim[1] - cen[1]};
    const double zl[2] = {par->z_lim[0] - cen[2], par->z_lim[1] - cen[2]};
    const double c0[3] = {0.0, 0.0, 0.0};
    int64_t Pmax = par->Npixels[0];
    if (par->Npixels[1] > Pmax) Pmax = par->Npixels[1];
    if (par->Npixels[2] > Pmax) Pmax = par->Npixels[2];
    int st = sphg_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, Pmax, par->boxsize, &cpar);
    if (st) return fail(ctx, st, g_error);
  }
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  sphg::DevParticles d;
  d.n = n;
  d.pos_dtype = pt->pos_dtype;
  d.attr_dtype = pt->attr_dtype;
  d.pos = pt->pos;
  d.sp = pt->pos_stride_p;
  d.sc = pt->pos_stride_c;
  d.hsml = pt->hsml;
  // mass, rho and weights do not enter the state or the ranges, but the
  // preparation reads them for every particle: absent ones alias hsml
  d.mass = pt->mass ? pt->mass : pt->hsml;
  d.rho = pt->rho ? pt->rho : pt->hsml;
  d.w = pt->weights ? pt->weights : pt->hsml;
  d.q = pt->bin_q;
  d.nq = nq;
  d.qsp = pt->q_stride_p;
  d.qsk = pt->q_stride_k;
  sphg::DevMapParams mp;
  for (int k = 0; k < 3; ++k) {
    mp.cen[k] = par->center[k];
    mp.lo[k] = cpar.center[k] - cpar.halfsize[k];
    mp.hi[k] = cpar.center[k] + cpar.halfsize[k];
  }
  mp.boxsize = par->boxsize;
  mp.periodic = par->periodic;
  // the positions are read, never written
  mp.center_mode = opt->center == SPHG_CENTER_INPLACE ? SPHG_CENTER_READONLY : opt->center;
  mp.filter = opt->filter;
  mp.calc_mean = dims == 2 ? opt->calc_mean : 0;
  mp.kernel_dim = opt->kernel_dim;
  mp.dims = dims;
  mp.L = cpar.len2pix;
  mp.P = P;
  mp.sigma = sphg::kernel_sigma(opt->kernel, opt->kernel_dim);
  sphg::set_lite_params(mp);
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(sphg::DevStatus), s));
  if (n > 0) {
    sphg::launch_footprints(d, mp, (long long*)ranges, (signed char*)state, ctx->d_status, ctx->num_sms, s);
    CK(cudaGetLastError());
  }
  CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(sphg::DevStatus), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (ctx->h_status->flags & sphg::kFlagNonFinite) return fail(ctx, SPHG_ERR_NONFINITE, "");
  ctx->last_error.clear();
  return SPHG_OK;
}

int sphg_reduce(sphg_context* ctx, const sphg_params* par, const sphg_options* opt, int32_t n_q,
                const double* raw, double* out, void* stream) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!par || !opt || !raw || !out) return fail(ctx, SPHG_ERR_ARG, "NULL argument");
  const int dims = opt->dimensions;
  if (dims != 2 && dims != 3) return fail(ctx, SPHG_ERR_DIMS, "");
  if (n_q < 1 || n_q > sphg::kMaxQ || (dims == 3 && n_q != 1)) return fail(ctx, SPHG_ERR_NQ, "");
  const int64_t P = par->Npixels[0];
  const int64_t PD = dims == 2 ? P * P : P * P * P;
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  if (dims == 2) sphg::launch_reduce_2d(raw, P, n_q, opt->reduce_image, out, s);
  else sphg::launch_reduce_3d(raw, raw + PD, PD, opt->reduce_image ? 0 : 1, out, ctx->num_sms, s);
  CK(cudaGetLastError());
  if (!stream) CK(cudaStreamSynchronize(s));
  return SPHG_OK;
}

int sphg_accumulate(sphg_context* ctx, int64_t len, const double* part, double* sum, void* stream) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (len < 0 || (len > 0 && (!part || !sum))) return fail(ctx, SPHG_ERR_ARG, "NULL or negative size");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  sphg::launch_accumulate(part, sum, len, ctx->num_sms, s);
  CK(cudaGetLastError());
  if (!stream) CK(cudaStreamSynchronize(s));
  return SPHG_OK;
}

int sphg_healpix_map(sphg_context* ctx, const sphg_healpix_params* hp, int64_t n, const void* pos,
                     const void* hsml, const void* mass, const void* rho, const void* bin_q,
                     const void* weights, double* allsky, double* weight, void* stream, sphg_stats* stats) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!hp || !allsky || !weight || n < 0) return fail(ctx, SPHG_ERR_ARG, "NULL argument or negative count");
  if (n > 0 && (!pos || !hsml || !mass || !rho || !bin_q || !weights))
    return fail(ctx, SPHG_ERR_ARG, "NULL particle array");
  const int64_t ns = hp->nside;
  if (ns < 1 || ns > 8192 || (ns & (ns - 1))) return fail(ctx, SPHG_ERR_ARG, "nside must be a power of 2 up to 8192");
  if (hp->kernel < 0 || hp->kernel > 4 || (hp->kernel_dim != 2 && hp->kernel_dim != 3))
    return fail(ctx, SPHG_ERR_ARG, "kernel");
  if (!valid_dtype(hp->dtype)) return fail(ctx, SPHG_ERR_ARG, "dtype");
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(sphg::DevStatus), s));
  // the pixel-centre table (3 FP64 per pixel, kept for the next call of the
  // same Nside) up to Nside 4096 (4.8 GB); above that, or when it cannot be
  // allocated, the centres are computed per use
  bool fill = false;
  if (n > 0 && ns <= 4096 && ctx->hp_nside != ns) {
    if (ctx->hp_centres) {
      CK(cudaStreamSynchronize(s));
      CK(cudaFree(ctx->hp_centres));
      ctx->hp_centres = nullptr;
      ctx->hp_nside = 0;
    }
    if (cudaMalloc(&ctx->hp_centres, (size_t)12 * ns * ns * 3 * sizeof(double)) == cudaSuccess) {
      ctx->hp_nside = ns;
      fill = true;
    } else {
      cudaGetLastError();
      ctx->hp_centres = nullptr;
    }
  }
  double* centres = ctx->hp_nside == ns ? ctx->hp_centres : nullptr;
  // per-warp slices of pass-1 distances (16384 per warp, 2.5 GB on 152 SMs;
  // 2048 when that cannot be had): pass 2 reads them instead of
  // recomputing the dot product and acos
  if (n > 0 && !ctx->hp_dist) {
    const size_t warps = (size_t)ctx->num_sms * sphg::kHpCtasPerSm * 8;
    for (int per_lane : {512, 64}) {
      if (cudaMalloc(&ctx->hp_dist, warps * 32 * per_lane * sizeof(double)) == cudaSuccess) {
        ctx->hp_dist_per_lane = per_lane;
        break;
      }
      cudaGetLastError();
      ctx->hp_dist = nullptr;
    }
  }
  if (n > 0)
    sphg::launch_healpix(ns, hp->kernel, hp->kernel_dim, hp->calc_mean, hp->dtype, n, pos, hsml, mass, rho, bin_q,
                         weights, allsky, weight, centres, fill, ctx->hp_dist, ctx->hp_dist_per_lane,
                         ctx->d_status, ctx->num_sms, s);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(sphg::DevStatus), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const sphg::DevStatus hs = *ctx->h_status;
  if (hs.flags & sphg::kFlagNonFinite) return fail(ctx, SPHG_ERR_NONFINITE, "non-finite particle");
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->n_in = n;
    stats->n_mapped = (int64_t)hs.n_mapped;
    stats->deposits = (int64_t)hs.deposits;
    stats->grid_mass = hs.grid_mass;
    stats->particle_mass = hs.particle_mass;
    stats->n_launches = n > 0 ? 1 : 0;
  }
  ctx->last_error.clear();
  return SPHG_OK;
}

int sphg_probe_fixed_chunks(sphg_context* ctx, int32_t n, const float* v, int64_t* x) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (n < 1 || n > (1 << 24) || !v || !x) return fail(ctx, SPHG_ERR_ARG, "n must be in 1..2^24, arrays non-NULL");
  DeviceGuard g(ctx->device);
  CK(sphg::probe_fixed_chunks(n, v, (long long*)x, ctx->stream));
  return SPHG_OK;
}

int sphg_probe_wait_timeout(sphg_context* ctx, int32_t polls, int32_t* timed_out) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!timed_out || polls < 1 || polls > (1 << 20)) return fail(ctx, SPHG_ERR_ARG, "polls must be in 1..2^20");
  DeviceGuard g(ctx->device);
  int t = 0;
  CK(sphg::probe_wait_timeout(polls, ctx->stream, &t));
  *timed_out = t;
  return SPHG_OK;
}

int sphg_probe_smem_rate(sphg_context* ctx, int kind, double* ops_per_s) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!ops_per_s || kind < 0 || kind > 6) return fail(ctx, SPHG_ERR_ARG, "kind must be 0..6");
  DeviceGuard g(ctx->device);
  CK(sphg::probe_smem_rate(kind, ctx->num_sms, ctx->stream, ops_per_s));
  return SPHG_OK;
}

int sphg_adjoint(sphg_context* ctx, const sphg_params* par, const sphg_options* opt,
                 const sphg_particles* pt, const double* raw, const double* grad_out,
                 const sphg_grads* gr, void* stream) {
  if (!ctx) return fail(nullptr, SPHG_ERR_ARG, "context is NULL");
  std::lock_guard<std::mutex> lk(ctx->mu);
  if (!par || !opt || !pt || !raw || !grad_out || !gr) return fail(ctx, SPHG_ERR_ARG, "NULL argument");
  if (opt->memspace != SPHG_MEM_DEVICE) return fail(ctx, SPHG_ERR_UNSUPPORTED, "adjoint takes device memory");
  if (opt->precision != SPHG_PREC_FP64 && opt->precision != SPHG_PREC_FP32C)
    return fail(ctx, SPHG_ERR_ARG, "unknown precision");
  const int dims = opt->dimensions;
  if (dims != 2 && dims != 3) return fail(ctx, SPHG_ERR_DIMS, "");
  const int nq = pt->n_q;
  if (nq < 1 || nq > sphg::kMaxQ) return fail(ctx, SPHG_ERR_ARG, "n_q must be in 1..16");
  if (dims == 3 && nq != 1) return fail(ctx, SPHG_ERR_NQ, "");
  if (opt->kernel < 0 || opt->kernel > 4 || (opt->kernel_dim != 2 && opt->kernel_dim != 3))
    return fail(ctx, SPHG_ERR_ARG, "kernel");
  if (!valid_dtype(pt->pos_dtype) || !valid_dtype(pt->attr_dtype)) return fail(ctx, SPHG_ERR_ARG, "dtype");
  const int64_t n = pt->n;
  if (n < 0) return fail(ctx, SPHG_ERR_ARG, "negative particle count");
  if (n > 0 && (!pt->pos || !pt->hsml || !pt->mass || !pt->rho || !pt->weights || !pt->bin_q || !gr->pos ||
                !gr->hsml || !gr->mass || !gr->rho || !gr->weights || !gr->bin_q))
    return fail(ctx, SPHG_ERR_ARG, "NULL particle or gradient array");
  const int64_t P = par->Npixels[0];
  if (P < 1 || P > (int64_t)1 << 20 || (dims == 3 && P > 4096)) return fail(ctx, SPHG_ERR_ARG, "Npixels");
  const int64_t PD = dims == 2 ? P * P : P * P * P;
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
    int st = sphg_mapping_parameters(xl, yl, zl, c0, -1.0, -1.0, -1.0, -1.0, Pmax, par->boxsize, &cpar);
    if (st) return fail(ctx, st, g_error);
  }
  DeviceGuard g(ctx->device);
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  Carve cv;
  const size_t o_g = cv.take((size_t)PD * (nq + 1) * sizeof(double));
  // FP32C: the image gradients as FP32 (hi, lo) pairs too, for the FP32
  // per-cell path
  const bool f32 = opt->precision == SPHG_PREC_FP32C;
  const size_t o_g32 = f32 ? cv.take((size_t)PD * (nq + 1) * 2 * sizeof(float)) : 0;
  const size_t o_adj = f32 ? cv.take(sphg::adjoint_scratch_bytes(n)) : 0;
  if (int st = ensure_ws(ctx, cv.off, s)) return st;
  double* gq = (double*)((char*)ctx->ws + o_g);
  double* gw = gq + (int64_t)nq * PD;
  float* g32 = f32 ? (float*)((char*)ctx->ws + o_g32) : nullptr;
  sphg::DevParticles d;
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
  sphg::DevMapParams mp;
  for (int k = 0; k < 3; ++k) {
    mp.cen[k] = par->center[k];
    mp.lo[k] = cpar.center[k] - cpar.halfsize[k];
    mp.hi[k] = cpar.center[k] + cpar.halfsize[k];
  }
  mp.boxsize = par->boxsize;
  mp.periodic = par->periodic;
  mp.center_mode = opt->center == SPHG_CENTER_INPLACE ? SPHG_CENTER_READONLY : opt->center;
  mp.filter = opt->filter;
  mp.calc_mean = dims == 2 ? opt->calc_mean : 0;
  mp.kernel_dim = opt->kernel_dim;
  mp.dims = dims;
  mp.L = cpar.len2pix;
  mp.P = P;
  mp.sigma = sphg::kernel_sigma(opt->kernel, opt->kernel_dim);
  const bool raw_out = opt->raw_accumulator || (dims == 2 && opt->return_both_maps);
  CK(sphg::launch_adjoint(opt->kernel, d, mp, raw, grad_out, raw_out ? 1 : 0, opt->reduce_image, gq, gw,
                          gr->pos, gr->hsml, gr->mass, gr->rho, gr->weights, gr->bin_q, g32,
                          f32 ? (char*)ctx->ws + o_adj : nullptr, ctx->num_sms, s));
  if (!stream) CK(cudaStreamSynchronize(s));
  ctx->last_error.clear();
  return SPHG_OK;
}

}  // extern "C"
