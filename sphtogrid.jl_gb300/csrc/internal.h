// internal.h -- launchers shared between the translation units of
// libsphgrid.so (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/sphgrid.h"
#include "common.cuh"
#include "tiled.cuh"

namespace sphg {

// Fails with cudaErrorNoKernelImageForDevice when the library was built for
// another architecture than the current device.
cudaError_t probe_kernel_image(cudaFuncAttributes* fa);

void launch_plain_fp64(int kernel, const DevParticles& pt, const DevMapParams& mp, double* accq,
                       double* accw, int64_t PD, DevStatus* st, int num_sms, cudaStream_t s);
void launch_footprints(const DevParticles& pt, const DevMapParams& mp, long long* rng, signed char* state,
                       DevStatus* st, int num_sms, cudaStream_t s);
void launch_reduce_2d(const double* acc, int64_t P, int nq, int reduce, double* out, cudaStream_t s);
void launch_healpix(int64_t nside, int kernel, int kdim, int calc_mean, int dtype, int64_t n, const void* pos,
                    const void* hsml, const void* m, const void* rho, const void* q, const void* w,
                    double* allsky, double* weight, double* centres, bool fill_centres, double* dist,
                    int dist_per_lane, DevStatus* st, int num_sms, cudaStream_t s);
// CTAs (of 256 threads, a warp per particle) per SM of the HEALPix deposit.
constexpr int kHpCtasPerSm = 16;
cudaError_t probe_smem_rate(int kind, int num_sms, cudaStream_t s, double* ops_per_s);
cudaError_t probe_wait_timeout(int polls, cudaStream_t s, int* timed_out);
cudaError_t probe_fixed_chunks(int n, const float* v, long long* x, cudaStream_t s);
void launch_accumulate(const double* part, double* sum, int64_t len, int num_sms, cudaStream_t s);
void launch_reduce_3d(const double* q, const double* w, int64_t PD, int w_is_one, double* out,
                      int num_sms, cudaStream_t s);

// Context accessors for the other translation units (abi.cu).
int context_device(sphg_context* ctx);
int context_num_sms(sphg_context* ctx);
void set_context_error(sphg_context* ctx, const std::string& msg);
// Message returned by sphg_last_error(NULL) on this host thread.
void set_thread_error(const std::string& msg);

// Tile shape and tile counts of the FP32-compensated path.
void tiled_geometry(int dims, int64_t P, int tdim[3], int ntile[3], int64_t* n_tiles);
cudaError_t launch_adjoint(int kernel, const DevParticles& pt, const DevMapParams& mp, const double* raw,
                           const double* grad_out, int mode, int reduce, double* gq, double* gw,
                           double* d_pos, double* d_hsml, double* d_mass, double* d_rho, double* d_w,
                           double* d_q, float* g32, void* scratch, int num_sms, cudaStream_t s);
size_t adjoint_scratch_bytes(int64_t n);

// K3 + K4 for one kernel shape (tiled_k<K>.cu).
void launch_norm_deposit_0(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev);
void launch_norm_deposit_1(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev);
void launch_norm_deposit_2(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev);
void launch_norm_deposit_3(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev);
void launch_norm_deposit_4(const TiledArgs& A, int grid_rec, cudaStream_t s, cudaEvent_t* ev);
cudaError_t launch_tiled_fp32(int kernel, const TiledArgs& A, int num_sms, cudaStream_t s,
                              cudaEvent_t* ev, int* n_launch);

}  // namespace sphg
