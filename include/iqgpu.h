/*
 * iqgpu.h -- C ABI of libiqgpu.so, the GB300 (sm_103a) image-quilting hot path.
 *
 * Drop-in boundary for ImageQuilting.jl v1.3.1. The reference has no FFI: its hot path is a
 * set of Julia functions. Each entry point below replaces one of them; a Julia host binds
 * them with `ccall` (imagequilting.jl_gb300/julia/IQGPU.jl), Python with ctypes.
 *
 * Conventions
 *   - Arrays are column-major (Julia order, dim 1 fastest); extents are given per dim.
 *   - Indices and coordinates are 0-based (Julia index minus one).
 *   - Buffers may be host memory (pageable or pinned) or device memory of the context's
 *     device: the library copies with cudaMemcpyDefault (unified addressing).
 *   - Every call returns IQ_OK (0) or an IQ_ERR_* code; iq_last_error() gives the message
 *     of the last failure on the calling thread. Calls on one context run in order on its
 *     stream and return after their results are written (synchronous for the caller).
 *   - One context per host thread; a context owns its device buffers.
 */
#ifndef IQGPU_H
#define IQGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IQ_OK 0
#define IQ_ERR_ARG 1       /* invalid argument (the reference's @assert failures) */
#define IQ_ERR_CUDA 2      /* CUDA runtime error */
#define IQ_ERR_ALLOC 3     /* device allocation failed */
#define IQ_ERR_NOPATTERN 4 /* every training-image pattern is disabled */
#define IQ_ERR_CUTCAP 5    /* graph cut hit its round limit */
#define IQ_ERR_STATE 6     /* no training image set on the context */
#define IQ_ERR_LIMIT 7     /* size beyond a stated maximum */
#define IQ_ERR_TIMEOUT 8   /* a device-side wait ran past its time limit (the kernel returned) */

#define IQ_F32 0
#define IQ_F64 1

#define IQ_PATH_RASTER 0
#define IQ_PATH_DILATION 1
#define IQ_PATH_RANDOM 2

typedef struct iq_ctx iq_ctx;

/* Keyword arguments of iqsim (src/iqsim.jl:50-63). */
typedef struct iq_sim_params {
  int32_t ndim;        /* 1, 2 or 3: dimension of the training image */
  int64_t tilesize[3]; /* tile size */
  int64_t simsize[3];  /* simulation grid size */
  double overlap[3];   /* overlap fraction per dim, in (0,1) */
  double tol;          /* relaxation tolerance in (0,1] */
  int32_t path;        /* IQ_PATH_RASTER / _DILATION / _RANDOM */
  int32_t nreal;       /* number of realizations */
  int32_t debug;       /* nonzero: also write boundary cuts and voxel reuse */
  uint64_t seed;       /* key of the Philox4x32-10 streams (path and draws) */
  int64_t real0;       /* global index of the first realization: realization r of this call
                          draws with counter (tile, real0 + r), so calls on several devices
                          with the same seed and disjoint [real0, real0 + nreal) ranges are
                          shards of one call (0 for a whole call) */
} iq_sim_params;

/* Hard data: the reference's Dict{CartesianIndex,Real} as a list of unique coordinates. */
typedef struct iq_hard_data {
  int64_t n;             /* number of data */
  const int64_t* coords; /* n x ndim, 0-based, one row per datum */
  const double* values;  /* n values; NaN marks an inactive voxel of the grid */
} iq_hard_data;

/* Soft data: one (aux, auxTI) pair of the reference's `soft` vector (src/iqsim.jl:77-82). */
typedef struct iq_soft_data {
  const float* aux;    /* auxiliary variable on the grid, extents auxsize (>= simsize) */
  int64_t auxsize[3];
  const float* auxti;  /* auxiliary variable on the training image, extents of the TI */
} iq_soft_data;

/* Version of this ABI (major * 10000 + minor * 100 + patch). */
int iq_version(void);

/* Message of the last failed call on this thread ("" if none). */
const char* iq_last_error(void);

/* Create a context on `device` with its own stream. */
int iq_ctx_create(int device, iq_ctx** out);
int iq_ctx_destroy(iq_ctx* ctx);

/* Stream (cudaStream_t) the context launches on, for callers that time it. */
void* iq_ctx_stream(iq_ctx* ctx);

/*
 * Near-ties of the last iq_simulate or iq_pick call on this context: the number of
 * (position, decision) pairs whose distance lies within 1e-6 (relative) of a decision value of
 * a pick, |D - t| <= 1e-6 t, summed over every pick of the call. The decisions are the
 * threshold (1 + tol) * min D (src/iqsim.jl:237; every position counts), and for the
 * relaxation the dbsize boundary of the primary distance and each auxiliary boundary of the
 * final round (src/relaxation.jl:11-12,22-27; the boundary position itself does not count).
 * No counterpart in the reference. Membership at those positions is decided on the exact
 * Float64 distance all the same; the count says how many decisions a 1e-6 change of the
 * distances could flip.
 */
int iq_ties(iq_ctx* ctx, int64_t* out);

/*
 * Upload the training image and keep it resident: prepare (src/utils.jl:96-102, NaN -> 0,
 * Float32 on the device like the reference's GPU path src/utils.jl:59), its NaN mask and the
 * Float64 integral image of its squares. dtype IQ_F32 or IQ_F64; NaN marks inactive voxels.
 */
int iq_set_ti(iq_ctx* ctx, const void* ti, int32_t dtype, int32_t ndim, const int64_t* size);

/*
 * The whole iqsim (src/iqsim.jl:50-315) on the resident training image.
 *   reals : nreal x prod(simsize) floats (realization r at offset r*prod(simsize))
 *   cuts  : nreal x prod(simsize) floats, or NULL (boundary cuts, needs p->debug)
 *   voxs  : nreal doubles, or NULL (voxel reuse, needs p->debug)
 * hard may be NULL; soft may be NULL when nsoft == 0.
 */
int iq_simulate(iq_ctx* ctx, const iq_sim_params* p, const iq_hard_data* hard, int32_t nsoft,
                const iq_soft_data* soft, float* reals, float* cuts, double* voxs);

/*
 * fastdistance (src/utils.jl:5-13) of `ntmpl` templates against the resident TI:
 *   out[t][p] = |sum_k w_k TI[p+k]^2 - 2 sum_k w_k tmpl_t[k] TI[p+k] + sum_k w_k tmpl_t[k]^2|
 * tmpl: ntmpl x prod(tilesize) floats; weights: prod(tilesize) bytes (0/1) or NULL for all
 * ones; out: ntmpl x prod(TIsize - tilesize + 1) floats. Windows that cover an inactive
 * TI voxel get +Inf (src/iqsim.jl:207).
 */
int iq_fastdistance(iq_ctx* ctx, const int64_t* tilesize, int32_t ntmpl, const float* tmpl,
                    const uint8_t* weights, float* out);

/*
 * Pattern pick of one tile (src/iqsim.jl:236-246): the threshold pick
 * findall(D .<= (1+tol)*minimum(D)) when naux == 0, else relaxation(D, Ds, tol)
 * (src/relaxation.jl:5-39); tau-model weights (src/taumodel.jl:5-45); the weighted draw with
 * u from Philox(seed; tile, real). D and Ds[i] hold P floats each.
 * out_index: drawn linear index; out_ncand: candidate count; out_cands (nullable, capacity
 * cap): candidate indices ascending; out_weights (nullable, capacity cap): their weights.
 */
int iq_pick(iq_ctx* ctx, const float* D, int64_t P, int32_t naux, const float* const* Ds,
            double tol, uint64_t seed, int64_t tile, int64_t real, int64_t* out_index,
            int64_t* out_ncand, int64_t* out_cands, double* out_weights, int64_t cap);

/*
 * iq_pick without any device allocation. No counterpart in the reference: for hosts that
 * cannot call cudaMalloc (device memory owned by their own pool allocator, or loops that
 * cannot afford its device-wide synchronization). Scratch lives in a file-scope __device__
 * array of the library (about 13 MB, held by every GPU that loads it until exit), so:
 *   - P <= 262144 positions and naux <= 3, else IQ_ERR_LIMIT;
 *   - the first call on a device looks up the array (cudaGetSymbolAddress): make it before
 *     any stream capture;
 *   - all calls share the array; calls that overlap on the GPU race and must be serialized.
 * D and Ds may be host or device memory; out_* are host memory. `stream` is a cudaStream_t
 * (NULL: the legacy default stream). Results equal iq_pick's.
 */
int iq_pick_noalloc(const float* D, int64_t P, int32_t naux, const float* const* Ds, double tol,
                    uint64_t seed, int64_t tile, int64_t real, int64_t* out_index,
                    int64_t* out_ncand, int64_t* out_cands, double* out_weights, int64_t cap,
                    void* stream);

/*
 * Minimum-error boundary cut (src/graphcut.jl:5-84) of two arrays of extents `size` along
 * `dim` (0-based). mask[v] = 1 when voxel v stays on the source side (keeps A).
 */
int iq_graphcut(iq_ctx* ctx, const float* A, const float* B, int32_t ndim, const int64_t* size,
                int32_t dim, uint8_t* mask);

/* Windows of the resident TI that cover an inactive voxel (src/utils.jl:115-129). */
int iq_finddisabled(iq_ctx* ctx, const int64_t* tilesize, uint8_t* out);

/*
 * Tile visiting order (src/utils.jl:158-204) over a grid of `extent` tiles: raster, random,
 * dilation or, when ndata > 0, data-first dilation from the shuffled `datainds`.
 * path_out receives prod(extent) 0-based linear tile indices.
 */
int iq_genpath(uint64_t seed, int32_t ndim, const int64_t* extent, int32_t kind, int64_t ndata,
               const int64_t* datainds, int64_t* path_out);

/*
 * Per-kernel timing with CUDA events on the context stream (enable = 1 clears the totals).
 * iq_profile_get reports, for kernel "corr", "pick", "graphcut" or "paste": the summed
 * event time, the launches, and the algorithmic work of those launches (corr: FLOPs of the
 * masked correlation, 2 * positions * offsets * templates; pick: bytes of the distance maps it
 * reads once; graphcut: lattice edges; paste: bytes written).
 */
int iq_profile(iq_ctx* ctx, int32_t enable);
int iq_profile_get(iq_ctx* ctx, const char* kernel, double* ms_total, int64_t* launches,
                   double* work);

/* Kernels this context has launched since it was created. */
int64_t iq_ctx_launches(iq_ctx* ctx);

/*
 * Tuning knobs of a context (launch shapes and heuristics; results do not depend on them):
 *   "graphcut.gr_period"  rounds between global relabels of the boundary cut (default 32)
 *   "graphcut.threads"    threads per cut CTA: 256, 512 or 1024 (default 512)
 *   "corr.variant"        launch shape of the 16-template correlation: 0 (4 positions per
 *                         thread), 1 (same, 3 CTAs per SM; default), 2 (8 positions),
 *                         3 (2 positions)
 *   "sim.level_chunk"     most tiles of one dependency level simulated together (default 64;
 *                         1 processes the tile path one tile at a time)
 *   "sim.max_steps"       simulate only the first n tiles of the path (< 0: all; default -1);
 *                         for bounded samples and for locating the first differing tile
 *   "corr.engine"         distance maps of "tile minus box" masks: 2 (default) tensor cores
 *                         (tcgen05) with FP16 halves after a power-of-two scaling when every
 *                         nonzero magnitude lies within 2^17 of the largest, else TF32 halves;
 *                         1 tensor cores with TF32 halves; 0 the SIMT FP32 kernel
 *   "sim.streams"         1 (default) or 2: with 2, the tensor-core engine and nreal >= 2,
 *                         iq_simulate runs two groups of realizations on two streams so that
 *                         one group's pick and cut overlap the other's correlation (each
 *                         correlation launch then holds half the columns, which costs more
 *                         than the overlap gains at 16 realizations)
 * Returns IQ_ERR_ARG for an unknown name or an out-of-range value.
 */
int iq_set_option(iq_ctx* ctx, const char* name, int64_t value);

/*
 * Learned proposal (no counterpart in the reference, which scans every training-image position
 * for every tile, src/iqsim.jl:206). A small 3-D convolutional encoder embeds a tile's masked
 * overlap and every training-image window under the same mask in 64 dimensions; iq_simulate
 * then evaluates the exact distance only at the ~lp.k positions whose embeddings lie nearest
 * the tile's, and picks among them. It applies to training images of integer codes in [0, 255]
 * (categorical facies; codes 0..3 are read as 2-bit planes)
 * without hard or soft data, for the tile shape the encoder was made for. Every lp.monitor-th
 * chunk compares one shortlist with the full exact scan; once the sampled recall of the true
 * candidate set, over at least 1000 sampled candidates, falls below 0.99 the shortlist length
 * doubles (and is judged afresh), and at lp.kmax the call continues with the full scan. Options:
 *   "lp.enable"   1: use the proposal where it applies (default 0)
 *   "lp.k"        shortlist length a call starts with (default 8192)
 *   "lp.kmax"     the recall monitor doubles the length while the sampled recall of the current
 *                 length is below 0.99, up to this (default 65536), then falls back
 *   "lp.monitor"  chunks between recall checks (default 16; 0: none)
 *   "lp.fallback" 1 (default): longer shortlists, then the full scan, below 0.99 sampled
 *                 recall; 0: keep the shortlists of lp.k (to measure the recall of an encoder)
 *   "lp.train_near" of the nneg negatives of iq_lp_train, how many are windows within 3 voxels
 *                 (x, y) and 1 (z) of the positive instead of random ones (default 16)
 *   "lp.capture"  capacity of training pairs recorded by iq_simulate's full-scan picks
 *                 (template features + 8 of its exact candidates); setting it clears them
 */
/* Fresh encoder parameters (Philox-seeded He initialization) for tiles of this shape. */
int iq_lp_init(iq_ctx* ctx, int32_t ndim, const int64_t* tilesize, uint64_t seed);
/* Copy the FP32 parameters out (n receives their count; out may be NULL to query it). */
int iq_lp_params(iq_ctx* ctx, float* out, int64_t cap, int64_t* n);
/* Set the parameters (trained elsewhere) for tiles of this shape. */
int iq_lp_set_params(iq_ctx* ctx, int32_t ndim, const int64_t* tilesize, const float* in,
                     int64_t n);
/* Window embeddings (n x 64 floats) of the resident TI at `positions` under the mask
 * "tile minus box" (box: lo[3], hi[3]). */
int iq_lp_embed(iq_ctx* ctx, int64_t n, const int64_t* positions, const int32_t* box,
                float* out);
/* Loss and parameter gradients of one InfoNCE batch (no update): nA anchors by their cell
 * features, one positive and nneg negatives per anchor by their positions, mask box `box`. */
int iq_lp_loss_grad(iq_ctx* ctx, int32_t nA, int32_t nneg, const float* anchor_feats,
                    const int64_t* pos_positions, const int64_t* neg_positions,
                    const int32_t* box, double temp, double* loss, float* grad);
/* Train on the captured pairs: `steps` Adam steps of `batch` anchors, `nneg` random negatives. */
int iq_lp_train(iq_ctx* ctx, int32_t steps, int32_t batch, int32_t nneg, double lr, double temp,
                uint64_t seed, double* loss_first, double* loss_last);
/* Statistics of the last iq_simulate (n >= 9): columns from shortlists, columns of the full
 * scan, monitored columns, their exact candidates, those shortlisted, sampled recall (-1: none),
 * fell back (1/0), mean shortlist length, captured training pairs; n >= 12 adds the shortlist
 * length the call ended with, the sampled recall at that length (-1: none) and its sampled
 * candidates. */
int iq_lp_stats(iq_ctx* ctx, double* out, int32_t n);

#ifdef __cplusplus
}
#endif

#endif /* IQGPU_H */
