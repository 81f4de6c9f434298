/*
 * sphgrid.h -- C ABI of the GB300 (sm_103a) sphMapping deposition library
 * (libsphgrid.so).
 *
 * It replaces the Julia deposition path of SPHtoGrid.jl v0.5.3:
 *   sphMapping(Pos, HSML, M, Rho, Bin_Quant, Weights=Rho; param, kernel,
 *              reduce_image, return_both_maps, dimensions, calc_mean, ...)
 *   src/cic_interpolation/cic_interpolation.jl:35-272
 * and below it center_particles / filter_particles_in_image
 * (filter_shift.jl:6-67), cic_mapping_2D (cic_2D.jl:103-244), cic_mapping_3D
 * (cic_3D.jl:110-208) and reduce_image_2D/3D (reduce_image.jl:8-55).
 * A Julia `ccall` shim keeping the sphMapping signature is in
 * sphtogrid.jl_gb300/julia/SPHtoGridGB300.jl; a Python ctypes mirror in
 * sphtogrid.jl_gb300/mapping.py.
 *
 * Conventions
 *  - Every entry point returns an int status (SPHG_OK = 0).  No exception
 *    crosses the ABI; sphg_last_error() gives the message of the last failed
 *    call on a context.
 *  - Arrays keep the Julia layouts: Pos is 3 x N column-major (element (c, p)
 *    at pos[p*pos_stride_p + c*pos_stride_c], strides in elements, so both the
 *    Julia layout (1 per component, 3 per particle) and a structure of arrays
 *    are accepted); Bin_Quant is N or Nq x N the same way.
 *  - Outputs are Float64 in Julia's column-major layouts:
 *      dimensions 2:                 (P, P, Nq) indexed [x, y, q]
 *      dimensions 2, return_both_maps: (P^2, Nq+1), row i*P + j (x slowest),
 *                                    columns Q_1..Q_Nq then the weight W
 *      dimensions 3:                 (P, P, P) indexed [z, y, x]
 *  - A context is bound to one CUDA device and is safe to share between host
 *    threads (calls on one context are serialised).
 */
#ifndef SPHGRID_H
#define SPHGRID_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHG_ABI_VERSION 1

typedef enum sphg_status {
  SPHG_OK = 0,
  SPHG_ERR_CENTER_EXTENT = 1, /* parameters.jl:67  error("Giving a center position ...") */
  SPHG_ERR_PIXELS = 2,        /* parameters.jl:98  error("Please specify pixelSideLength ...") */
  SPHG_ERR_DIMS = 3,          /* dimensions not 2 or 3 (the reference returns `nothing`) */
  SPHG_ERR_NONFINITE = 4,     /* non-finite pixel range of a mapped particle (the
                                 reference's floor(Integer, x) throws InexactError,
                                 cic_shared.jl:46-52) */
  SPHG_ERR_NQ = 5,            /* 3D maps a single scalar quantity (cic_3D.jl:140) */
  SPHG_ERR_ALLOC = 6,         /* device or host allocation failed */
  SPHG_ERR_ARG = 7,           /* null pointer, bad dtype, bad stride, bad size */
  SPHG_ERR_CUDA = 8,          /* CUDA runtime error (message in sphg_last_error) */
  SPHG_ERR_TIMEOUT = 9,       /* a device work queue gave up waiting (bounded spin) */
  SPHG_ERR_NO_DEVICE = 10,    /* no CUDA device / extension built for another arch */
  SPHG_ERR_UNSUPPORTED = 11   /* option combination not implemented */
} sphg_status;

enum { SPHG_F32 = 0, SPHG_F64 = 1 };

/* SPHKernels.jl kernel types (README.md:57-63 of the reference). */
enum {
  SPHG_KERNEL_CUBIC = 0,
  SPHG_KERNEL_QUINTIC = 1,
  SPHG_KERNEL_WENDLAND_C4 = 2,
  SPHG_KERNEL_WENDLAND_C6 = 3,
  SPHG_KERNEL_WENDLAND_C8 = 4
};

/* Arithmetic of the deposition. */
enum {
  SPHG_PREC_FP64 = 0, /* plain FP64: the reference's arithmetic, FP64 atomics */
  SPHG_PREC_FP32C = 1 /* FP32 weights + compensated FP32 tile sums, FP64 image */
};

enum { SPHG_MEM_DEVICE = 0, SPHG_MEM_HOST = 1 };

/* What sphg_map does with positions before mapping. */
enum {
  SPHG_CENTER_NONE = 0,      /* positions are already centred on 0 */
  SPHG_CENTER_INPLACE = 1,   /* Pos[d,i] -= center[d] written back into the caller's
                                array, as the reference does (filter_shift.jl:15) */
  SPHG_CENTER_READONLY = 2   /* centre on the fly, leave the caller's array intact */
};

/* Field-for-field image of `mappingParameters` (parameters.jl:14-27). */
typedef struct sphg_params {
  double x_lim[2], y_lim[2], z_lim[2];
  double center[3];
  double halfsize[3];
  double len2pix;
  double pixelSideLength;
  int64_t Npixels[3];
  double boxsize;
  int32_t periodic;
  int32_t pad_;
} sphg_params;

typedef struct sphg_particles {
  int64_t n;
  int32_t pos_dtype;  /* SPHG_F32 / SPHG_F64 */
  int32_t attr_dtype; /* dtype of hsml, mass, rho, weights and bin_q */
  void *pos;          /* 3 x n (see conventions); written when centering INPLACE */
  int64_t pos_stride_p, pos_stride_c;
  const void *hsml, *mass, *rho, *weights; /* length n, contiguous */
  const void *bin_q;                       /* n_q x n */
  int32_t n_q;
  int32_t pad_;
  int64_t q_stride_p, q_stride_k;
} sphg_particles;

typedef struct sphg_options {
  int32_t dimensions;       /* 2 or 3 */
  int32_t kernel;           /* SPHG_KERNEL_* */
  int32_t kernel_dim;       /* dimension of the SPHKernels object (2 or 3) */
  int32_t reduce_image;     /* sphMapping `reduce_image` */
  int32_t return_both_maps; /* sphMapping `return_both_maps` (2D) */
  int32_t calc_mean;        /* sphMapping `calc_mean` (2D; 3D always false) */
  int32_t precision;        /* SPHG_PREC_* */
  int32_t deterministic;    /* 1: bitwise reproducible sums (FP32C only) */
  int32_t center;           /* SPHG_CENTER_* */
  int32_t filter;           /* 1: keep particles whose centre is in the box (the
                               reference's filter); 0: map every particle */
  int32_t memspace;         /* SPHG_MEM_*: where pos/attrs/out live */
  int32_t profile;          /* 1: time the phases with CUDA events (sphg_stats.phase_ms) */
  int32_t raw_accumulator;  /* 1: write the raw (P^D, Nq+1) accumulator [Q_1..Q_Nq, W] in
                               2D and 3D (2D: same as return_both_maps); the reference's
                               3D path has no such output */
  int32_t reserved[3];      /* must be 0 */
} sphg_options;

/* Phases timed with sphg_options.profile (device time on the call's stream). */
enum {
  SPHG_PHASE_PREP = 0,    /* centring, filter, pixel ranges, tile counts */
  SPHG_PHASE_NORM = 1,    /* renormalisation sums, tile lists */
  SPHG_PHASE_DEPOSIT = 2, /* deposition (and, FP32C, the fused reduction) */
  SPHG_PHASE_REDUCE = 3   /* separate Q/W reduction (FP64 path) */
};

typedef struct sphg_stats {
  int64_t n_in;          /* particles passed in */
  int64_t n_mapped;      /* particles deposited (filtered and q != 0 or calc_mean) */
  int64_t deposits;      /* sum of integer footprints of mapped particles */
  double grid_mass;      /* 3D mass diagnostic (cic_3D.jl:186) */
  double particle_mass;  /* 3D: sum of mapped particle masses (cic_3D.jl:192) */
  sphg_params centred;   /* parameters re-derived around centre 0 (filter_shift.jl:25-31) */
  int32_t n_launches;    /* kernels this call launched */
  int32_t n_reruns;      /* FP32C: re-runs after growing the tile-pair list */
  float phase_ms[4];     /* with profile: device milliseconds per SPHG_PHASE_* */
} sphg_stats;

typedef struct sphg_context sphg_context;

/* ABI version compiled into the library (SPHG_ABI_VERSION). */
int sphg_abi_version(void);

/* Message of a status code. */
const char *sphg_status_string(int status);

/* Create / destroy a context on CUDA device `device`.  The context owns a
 * grow-only device workspace and pinned staging buffers. */
int sphg_context_create(int device, sphg_context **out);
int sphg_context_destroy(sphg_context *ctx);

/* Message of the last failed call on `ctx` (never NULL). */
const char *sphg_last_error(const sphg_context *ctx);

/* mappingParameters(T; x_lim, y_lim, z_lim, center, x_size, y_size, z_size,
 * pixelSideLength, Npixels, boxsize) -- parameters.jl:44-125.  Arguments take
 * the reference's sentinel defaults: -1 ("not given") for limits, centre,
 * sizes, pixelSideLength and boxsize; 0 for Npixels.  Host only. */
int sphg_mapping_parameters(const double x_lim[2], const double y_lim[2],
                            const double z_lim[2], const double center[3],
                            double x_size, double y_size, double z_size,
                            double pixelSideLength, int64_t Npixels, double boxsize,
                            sphg_params *out);

/* Number of doubles sphg_map writes to `out` for these options. */
int64_t sphg_output_len(const sphg_params *par, const sphg_options *opt, int32_t n_q);

/* Gradients of a map with respect to the particle inputs (FP64, device
 * memory).  pos and bin_q use the strides of the sphg_particles they belong to. */
typedef struct sphg_grads {
  double *pos;
  double *hsml, *mass, *rho, *weights;
  double *bin_q;
} sphg_grads;

/* sphMapping (cic_interpolation.jl:35-272): centre, filter, deposit, reduce.
 * `stream` is a cudaStream_t (NULL: the context's own stream).  The call
 * returns after the result is complete in `out`.  `stats` may be NULL. */
int sphg_map(sphg_context *ctx, const sphg_params *par, const sphg_options *opt,
             const sphg_particles *parts, double *out, void *stream, sphg_stats *stats);

/* map_it's projection (cic_interpolation.jl:314-345, rotate_particles.jl,
 * rotate_parameters.jl): the positions are read through it while mapping, and
 * the caller's arrays are left intact, as map_it maps a copy.
 * SPHG_PROJ_XZ / _YZ permute the axes (rotate_to_xz_plane! / _yz_plane!:
 * (x, z, y) and (y, z, x)) and the parameters with them (center and limits
 * permuted, Npixels = max(Npixels), the same boxsize).  SPHG_PROJ_MATRIX
 * applies the row-major 3 x 3 `matrix` in FP64 -- rotate_3D's RotXYZ(a, b, c)
 * = Rx(a) Ry(b) Rz(c) -- with the parameters unchanged, and maps the rotated
 * positions as Float64 (Julia promotes them).  SPHG_CENTER_INPLACE is taken
 * as SPHG_CENTER_READONLY. */
enum { SPHG_PROJ_XY = 0, SPHG_PROJ_XZ = 1, SPHG_PROJ_YZ = 2, SPHG_PROJ_MATRIX = 3 };
typedef struct sphg_projection {
  int32_t kind;
  int32_t reserved; /* 0 */
  double matrix[9];
} sphg_projection;
int sphg_map_projected(sphg_context *ctx, const sphg_params *par, const sphg_options *opt,
                       const sphg_particles *parts, const sphg_projection *proj, double *out,
                       void *stream, sphg_stats *stats);

/* healpix_map's particle loop (healpix_interpolation/main.jl:129-204) on
 * the GPU in FP64: the particles as filter_sort_particles leaves them
 * (centred on the observer and selected; their order does not matter),
 * positions 3 per particle, device memory.  Skips particles with q == 0
 * (unless calc_mean) and those closer than their hsml; adds into `allsky`
 * and `weight` (12 nside^2 doubles each, RING ordering, zeroed by the
 * caller).  stats: n_mapped, deposits (particle-pixel pairs), grid_mass and
 * particle_mass as the reference accumulates them. */
typedef struct sphg_healpix_params {
  int64_t nside;     /* power of 2, 1 .. 8192 */
  int32_t kernel;    /* SPHG_KERNEL_* */
  int32_t kernel_dim;
  int32_t calc_mean;
  int32_t dtype;     /* SPHG_F32 / SPHG_F64 of all particle arrays */
} sphg_healpix_params;
int sphg_healpix_map(sphg_context *ctx, const sphg_healpix_params *hp, int64_t n, const void *pos,
                     const void *hsml, const void *mass, const void *rho, const void *bin_q,
                     const void *weights, double *allsky, double *weight, void *stream,
                     sphg_stats *stats);

/* reduce_image_2D / reduce_image_3D (reduce_image.jl:8-55) of a raw
 * (P^D, Nq+1) accumulator into the output layout of `opt` (device memory). */
int sphg_reduce(sphg_context *ctx, const sphg_params *par, const sphg_options *opt, int32_t n_q,
                const double *raw, double *out, void *stream);

/* distributed_cic_map's summation of sub-file maps
 * (src/distributed_mapping/cic.jl:55-78): adds the finite entries of the raw
 * accumulator `part` into `sum` (both `len` doubles, device memory); NaN and
 * Inf entries are skipped as in the reference.  Reduce the sum with
 * sphg_reduce. */
int sphg_accumulate(sphg_context *ctx, int64_t len, const double *part, double *sum, void *stream);

/* Adjoint of sphg_map (no counterpart in the reference, which has no
 * derivatives): given the forward's raw accumulator `raw` ((P^D, Nq+1), from
 * raw_accumulator = 1) and dL/d(output) `grad_out` in the layout of the
 * output `opt` describes, writes dL/d(pos, hsml, mass, rho, weights, bin_q)
 * into `grads`.  Kernel weights are recomputed, not stored.  Particles the
 * forward skips (filtered out, or q == 0 without calc_mean) get zero
 * gradients.  Device memory only; positions must be centred the way the
 * forward saw them (use SPHG_CENTER_READONLY in both, or NONE after INPLACE).
 * opt->precision: SPHG_PREC_FP64 (FP64 throughout) or SPHG_PREC_FP32C (per-cell
 * weights and derivatives in FP32 with compensated sums, the per-particle
 * finish in FP64; particles the FP32C forward would redo in FP64 are done in
 * FP64 here too). */
int sphg_adjoint(sphg_context *ctx, const sphg_params *par, const sphg_options *opt,
                 const sphg_particles *parts, const double *raw, const double *grad_out,
                 const sphg_grads *grads, void *stream);

/* Measurement only (no counterpart in the reference): the rate, in additions
 * per second over the whole GPU, of the shared-memory accumulation step of
 * the tile deposit -- kind 0: FP32 atomic add with its old value used;
 * 1: FP32 atomic add without return; 2: int64 atomic add; 3: the FP32C
 * deposit's compensated add (atomic add, TwoSum, error term into a second
 * accumulator); 4: the same compensated add of an adjacent (hi, lo) pair by
 * one 64-bit compare-and-swap (an alternative, not used); 5: the
 * deterministic deposit's int64 fixed-point add as two native 32-bit atomics
 * with a carry (its tiles of more than 2047 pairs); 6: the same fixed point
 * as three 21-bit chunks added by three 32-bit reductions (its tiles of at
 * most 2047 pairs).
 * Conflict-free addresses: an upper bound, not a deposit rate.  Synchronous;
 * allocates a few bytes of device memory. */
int sphg_probe_smem_rate(sphg_context *ctx, int kind, double *ops_per_s);

/* Diagnostics only (no counterpart in the reference): the tile deposit's
 * bounded wait for a bulk copy, run on a barrier that no copy completes.
 * The wait gives up after `polls` polls (1..2^20) and *timed_out is set to 1
 * -- the path that turns a copy that never lands into SPHG_ERR_TIMEOUT
 * instead of a hang.  Synchronous; allocates a few bytes of device memory. */
int sphg_probe_wait_timeout(sphg_context *ctx, int32_t polls, int32_t *timed_out);

/* Diagnostics only (no counterpart in the reference): the deterministic
 * mode's rounding of n host floats v (|v| < 2^62) to integers as three
 * 21-bit chunks, recombined into x[2 i], beside the 64-bit conversion
 * (round to nearest, ties to even) in x[2 i + 1].  Synchronous. */
int sphg_probe_fixed_chunks(sphg_context *ctx, int32_t n, const float *v, int64_t *x);

/* Per-particle state and integer pixel ranges, from the device code every
 * map runs (center_particles and filter_particles_in_image,
 * filter_shift.jl:6-58; the quantity skip, cic_2D.jl:154-168;
 * get_xyz and pix_index_min_max, cic_shared.jl:46-52 and :85-99), for
 * checking them against a reference bit for bit.  state[p]: 0 filtered out,
 * 1 skipped (every quantity zero without calc_mean), 2 mapped, 3 non-finite
 * range (the call returns SPHG_ERR_NONFINITE).  ranges[6 p .. 6 p + 5] =
 * {iMin, iMax, jMin, jMax, kMin, kMax} of a mapped particle (zeros
 * otherwise; the third axis is 0 0 in 2D; an empty range has max = min - 1).
 * Device memory only; the positions are read, never written
 * (SPHG_CENTER_INPLACE is taken as READONLY).  mass, rho and weights may be
 * NULL: they do not enter the state or the ranges.  Synchronous. */
int sphg_footprints(sphg_context *ctx, const sphg_params *par, const sphg_options *opt,
                    const sphg_particles *parts, int64_t *ranges, int8_t *state, void *stream);

/* ------------------------------------------------------- no-allocation map
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory: code running inside a host application that owns all device memory
 * through its own pool (an in-situ map under a fixed memory budget, a plugin
 * whose host forbids allocations during a time step), where cudaMalloc and
 * cudaFree either fail or stall the device mid-step.
 *
 * sphg_map_noalloc maps like sphg_map with precision FP32C, but needs no
 * context and calls no cudaMalloc, cudaFree or allocating library routine.
 * Its scratch (particle records, tile lists, the (particle, tile) pair
 * records, the status word) is one static device array of
 * SPHG_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the library until
 * the process exits.  Limits: records take (84 + 4 n_q) bytes per input
 * particle; of what remains, about an eighth holds large-footprint chunk
 * sums and the rest the pair records, 64 bytes per (particle, tile) overlap,
 * so a few hundred thousand particles fit.  Larger calls return
 * SPHG_ERR_ARG (before any work) or SPHG_ERR_ALLOC (pair records full) --
 * use sphg_map for them.
 *
 * - Device memory only (opt->memspace = SPHG_MEM_DEVICE); runs on the
 *   caller's current device and `stream` (NULL: the legacy default stream),
 *   synchronises that stream and returns when the map is complete.
 * - SPHG_CENTER_INPLACE: the map centres on the fly and the centred
 *   positions are written back only when the map completes (or meets a
 *   non-finite value, as the reference does); a call that returns
 *   SPHG_ERR_ALLOC leaves the positions as they were, so a retry with the
 *   same options (through sphg_map) centres them once.
 * - The first call on a device looks up the array's device address
 *   (cudaGetSymbolAddress) and keeps it for the process.  The kept address
 *   is not valid after a cudaDeviceReset of that device.
 * - Every call on a device shares the one array and clears what it
 *   accumulates into; calls that overlap on the GPU (other streams or host
 *   threads without ordering between them) race and corrupt each other.
 * - opt->profile is ignored (no phase timings); opt->reserved must be 0.
 * - Errors: sphg_last_error(NULL) gives the message (per host thread). */
#define SPHG_NOALLOC_SCRATCH_BYTES (64ull << 20)

int sphg_map_noalloc(const sphg_params *par, const sphg_options *opt, const sphg_particles *parts,
                     double *out, void *stream, sphg_stats *stats);

/* ---------------------------------------------------------------- batches
 * Many maps (uneven particle counts, resolutions, quantities, kernel shapes)
 * mapped together: one launch per phase for all maps and one persistent
 * deposit launch over a work queue of every map's image tiles, captured once
 * in a CUDA graph and replayed.  No counterpart in the reference, which maps
 * one image per sphMapping call (cic_interpolation.jl:35).  Maps must use
 * precision FP32C, device memory and centering NONE or READONLY (a replay
 * reads the same input buffers again; refill them between launches). */
typedef struct sphg_map_desc {
  sphg_params par;
  sphg_options opt;
  sphg_particles parts;
  double *out; /* device, sphg_output_len(&par, &opt, parts.n_q) doubles */
} sphg_map_desc;

/* Tuned quantities: 2D tile shape (16x16, 32x16 or 32x32; 3D tiles are
 * 8x8x8), CTAs per SM of the persistent deposit, and the footprint size (in
 * cells) above which a particle's renormalisation is split across CTAs. */
typedef struct sphg_batch_tuning {
  int32_t tile_x, tile_y;
  int32_t ctas_per_sm;
  int32_t large_cells;
  float tuned_ms;      /* autotuned: time of one eager run of the chosen plan */
  int32_t reserved[3];
} sphg_batch_tuning;

typedef struct sphg_batch sphg_batch;

/* Plans a batch: sizes the intermediate lists by mapping once, autotunes when
 * `tuning` is NULL (trying tile shapes, CTAs per SM and large-footprint
 * thresholds), and captures the pipeline in a CUDA graph.  The outputs hold
 * valid maps on return. */
int sphg_batch_create(sphg_context *ctx, int32_t n_maps, const sphg_map_desc *maps,
                      const sphg_batch_tuning *tuning, sphg_batch **out);
/* Replays the captured graph on `stream` (NULL: the batch's own stream). */
int sphg_batch_launch(sphg_batch *batch, void *stream);
/* Waits for the last launch, checks every map's status (growing the lists and
 * re-capturing if the inputs outgrew them) and fills `stats[n_maps]` (may be
 * NULL). */
int sphg_batch_wait(sphg_batch *batch, sphg_stats *stats);
int sphg_batch_get_tuning(const sphg_batch *batch, sphg_batch_tuning *out);
const char *sphg_batch_last_error(const sphg_batch *batch);
int sphg_batch_destroy(sphg_batch *batch);

#ifdef __cplusplus
}
#endif

#endif /* SPHGRID_H */
