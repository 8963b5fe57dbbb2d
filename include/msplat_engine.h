/*
 * msplat GB300 engine — device-level C ABI.
 *
 * This is the internal boundary of the training hot path: the CUDA
 * replacement of the reference's msplat_train_step and msplat_render
 * (core/metal/bindings.h:58-95, implemented at core/metal/msplat_metal.mm:
 * 1099-1117 and 1118-1740), plus the SGLD step (bindings.h:97-107,
 * msplat_metal.mm:1746-1812).  Everything takes plain device pointers and
 * sizes; the public trainer API (msplat_c_api.h) is built on top of it.
 *
 * Threading: one engine is driven from one host thread (the reference's
 * single-trainer rule, core/metal/msplat_metal.mm:411-417).  All work is
 * enqueued on the engine's own CUDA stream.
 *
 * Errors: functions return 0 on success and a negative code on failure;
 * msplat_engine_last_error() describes the last failure.
 */
#ifndef MSPLAT_ENGINE_H
#define MSPLAT_ENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct MsplatEngine MsplatEngine;

/* Gaussians in device memory, row-major, num_points rows, the reference's
 * layouts (core/include/model.hpp:65-70): means [N,3], scales [N,3] (log),
 * quats [N,4] (w,x,y,z), features_dc [N,3], features_rest [N,rest_bases,3],
 * opacities [N] (logit).  Pointers must be 16-byte aligned. */
typedef struct {
    int num_points;
    int rest_bases;
    float *means, *scales, *quats, *features_dc, *features_rest, *opacities;
} MsplatGaussians;

/* Adam moments in device memory, same shapes as the parameters, in the
 * reference's group order (model.cpp:223): means, scales, quats,
 * features_dc, features_rest, opacities. */
typedef struct {
    float *exp_avg[6];
    float *exp_avg_sq[6];
} MsplatAdamState;

/* The scalar arguments of msplat_train_step / msplat_render
 * (core/metal/bindings.h:58-95, model.cpp:901-969). */
typedef struct {
    float viewmat[16];      /* row-major world->camera (model.cpp:857-866) */
    float projmat[16];      /* row-major projection * view */
    float fx, fy, cx, cy;
    int width, height;
    float cam_pos[3];
    float background[3];
    float clip_thresh;      /* near-plane cull, 0.01 in the reference */
    int degrees_to_use;     /* active SH bands */
    float ssim_weight;      /* 0.2 */
    float loss_inv_n;       /* 1 / (3 * pixels), or 1 / (3 * unmasked pixels) */
    float step_size[6];     /* lr / (1 - beta1^t) per group */
    float bc2_sqrt[6];      /* sqrt(1 - beta2^t) per group */
    float beta1, beta2, eps;
    float op_reg, sc_reg;   /* MCMC regularizer weights (0 before step 500) */
    float invis_scale;      /* regularizer duty for rendered Gaussians (1 = reference) */
    int raster_mode;        /* 0: reference rule (chunked iff < 400 tiles), 1: monolithic, 2: chunked */
    int k_max;              /* chunk count of the chunked raster; 0 = reference rule */
    int do_optimizer;       /* 1: SH Adam, regularizer and Adam run in the step */
    int do_sgld;            /* 1: SGLD noise on the means after the optimizer */
    uint32_t seed;          /* SGLD noise seed (the training step) */
    float noise_lr, xyz_lr, max_disp;
} MsplatStepArgs;

/* Pipeline stages timed with CUDA events on the engine's stream. */
enum {
    MSPLAT_STAGE_PROJECT = 0, MSPLAT_STAGE_TILES, MSPLAT_STAGE_RASTER_FWD, MSPLAT_STAGE_LOSS,
    MSPLAT_STAGE_RASTER_BWD, MSPLAT_STAGE_PROJECT_BWD, MSPLAT_STAGE_ADAM, MSPLAT_STAGE_SGLD,
    MSPLAT_STAGE_COUNT
};

typedef struct {
    long long num_intersections;   /* M of the last step */
    int max_tile_count;
    int k_max;                     /* 1 = monolithic raster */
    int num_tiles;
    uint32_t nan_counts[16];       /* cumulative non-finite telemetry (reference slot numbering) */
    float stage_ms[MSPLAT_STAGE_COUNT];  /* summed over timed_steps steps since timing was enabled */
    long long timed_steps;         /* steps whose stage times are summed (at most the last 128) */
    long long launches;            /* engine kernel launches since creation */
    uint32_t check_record[3];      /* checked builds: first failed bound (code, index lo, index hi) */
    int isect_groups;              /* tile groups of the last step (fixed intersection budget; 1 otherwise) */
} MsplatEngineStats;

/* Creates an engine on CUDA device `device`.  max_points sizes the
 * per-Gaussian arena (0 = grow on demand). */
MsplatEngine *msplat_engine_create(int device, int max_points);
void msplat_engine_destroy(MsplatEngine *e);
const char *msplat_engine_last_error(const MsplatEngine *e);

/* One training step (msplat_train_step): projection, tile lists, raster,
 * SSIM+L1 loss, backward, fused SH Adam, regularizer + Adam, optional SGLD.
 * gt: device uint8 [H,W,3]; mask: device uint8 [H,W] or NULL.
 * Parameters and moments are updated in place.  Asynchronous. */
int msplat_engine_train_step(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                             const MsplatStepArgs *args, const uint8_t *gt, const uint8_t *mask);

/* The same step with the target image (and mask) in host memory, as the
 * reference reads the camera's image each step (core/src/msplat_api.mm:
 * 104-110): they are copied to the device on a copy stream into one of two
 * alternating engine buffers (asynchronously when the host buffers are
 * page-locked), so one step's upload overlaps the step before it; the step
 * itself waits for its copy.  The host buffer must stay valid until the
 * copy has run (msplat_engine_synchronize). */
int msplat_engine_train_step_host(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                                  const MsplatStepArgs *args, const uint8_t *gt_host, const uint8_t *mask_host);

/* Forward only (msplat_render); the image stays in the engine's "out_img"
 * buffer (device float [H,W,3]).  Asynchronous. */
int msplat_engine_render(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args);

/* Waits for the engine's stream. */
int msplat_engine_synchronize(MsplatEngine *e);

/* Loss of the last step (loss_sum / (H*W), msplat_metal.mm:1738); waits. */
int msplat_engine_loss(MsplatEngine *e, float *loss);

/* Without waiting: copies the last step's loss sums (one float per view of
 * the step; the loss is the sum divided by the view's pixel count) to dst on
 * the engine's stream.  With page-locked dst the values are there once the
 * stream has passed this point (msplat_engine_synchronize). */
int msplat_engine_loss_async(MsplatEngine *e, float *dst);

/* Stats of the last step; waits. */
int msplat_engine_stats(MsplatEngine *e, MsplatEngineStats *out);

/* Enables (and resets) per-stage CUDA-event timing: each step records
 * events between its stages on the engine's stream. */
int msplat_engine_set_timing(MsplatEngine *e, int enabled);

/* Named intermediate buffers ("rec", "depths", "radii", "aabb", "tiles_hit",
 * "tile_counts", "tile_offsets", "isect_ids", "out_img", "final_T",
 * "final_idx", "v_img", "grad", "v_mean", "v_scale", "v_quat", ...):
 * returns the size in bytes and the device pointer (or -1). */
long long msplat_engine_buffer(MsplatEngine *e, const char *name, void **dev_ptr);

/* Copies the first `bytes` of a named buffer to host or device memory (any
 * address CUDA can reach); waits. */
int msplat_engine_read(MsplatEngine *e, const char *name, void *dst, long long bytes);

/* MCMC relocation + growth (Model::mcmcAfterTrain, core/src/model.cpp:
 * 497-660), resident on the GPU.  g->num_points is the active count N; the
 * parameter and moment buffers must hold cap_max rows.  Dead Gaussians
 * (non-finite, sigmoid(opacity) <= 0.005, |mean| > cull_radius) are moved
 * onto living ones drawn in proportion to sigmoid(opacity), each source is
 * rescaled by Eq. 9 (model.cpp:311-332), and min(cap_max, 1.05 N) - N new
 * slots are filled the same way.  *relocation_count is the reference's
 * mcmc_relocation_count (seeds the draws); it is advanced in place.  The
 * chosen (dst, src) pairs stay readable in the "mcmc_moves" buffer
 * (relocation moves first, then growth).  Waits for the device. */
typedef struct {
    int num_dead, num_culled, num_nonfinite, num_relocated, num_grown, num_active;
} MsplatMcmcStats;

int msplat_engine_mcmc(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st, int cap_max,
                       float cull_radius, int *relocation_count, MsplatMcmcStats *out);

/* Parameter gradients for a caller-supplied image gradient (the autograd
 * binding's backward).  The forward of (g, args) is recomputed, then the
 * rasterizer and projection backward passes run without any optimizer and
 * write dL/d(parameter) for every Gaussian into the caller's device buffers
 * (shapes of the parameters; zero for culled Gaussians and for SH bands
 * above args->degrees_to_use).  v_img: device float [H,W,3].  Same VJPs as
 * the training step (rasterize_backward_kernel, project_and_sh_backward_kernel).
 * Under a fixed intersection budget (msplat_engine_set_isect_budget) the
 * view's lists must fit the budget in one tile group (error otherwise);
 * without one, the legacy 48-per-Gaussian buffer is used. */
typedef struct {
    float *v_means, *v_scales, *v_quats, *v_features_dc, *v_features_rest, *v_opacities;
} MsplatGradients;

int msplat_engine_backward(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args, const float *v_img,
                           const MsplatGradients *out);

/* Multi-view training step: num_views (1..16) views, each with its own
 * camera and size in args[v], target gt[v] and mask mask[v] (mask may be
 * NULL for none), rendered and back-propagated by the same launches as one
 * view: every stage (projection, tile mapping, raster, loss, raster
 * backward, projection backward) is one launch over all views.  Each view's
 * image gradient is scaled by 1/num_views, so the parameter gradients are the
 * views' mean; then one optimizer update: the 4-group Adam with the
 * regularizer, the SH Adam over the coefficients of Gaussians visible in at
 * least one view (bands below degrees_to_use), and SGLD; optimizer scalars
 * and raster mode from args[0].  The engine's record buffers (rec, depths,
 * radii, grad) are then [num_views, num_points] and its image buffers the
 * views' images one after another.  msplat_engine_loss returns the mean of
 * the views' losses.  With one view this is msplat_engine_train_step.  Graph
 * mode captures the batch. */
int msplat_engine_train_step_batch(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st,
                                   const MsplatStepArgs *args, int num_views, const uint8_t *const *gt,
                                   const uint8_t *const *mask);

/* Learned relocation proposal support.  `stats` (device float4 per
 * Gaussian, cap-sized, caller-owned, zeroed by the caller; NULL to stop)
 * accumulates per training step, for each view in which the Gaussian is
 * visible: x += |dL/d(pixel centre)| and y += 1; and z += 1 (age).  MCMC clears the entry of every
 * slot it fills with a copy. */
int msplat_engine_set_activity_stats(MsplatEngine *e, void *stats);

/* msplat_engine_mcmc with the sampling weight of each Gaussian taken from
 * `score` (device float [num_points]; non-positive or non-finite = never
 * drawn) instead of sigmoid(opacity).  The dead/culled classification is
 * unchanged. */
int msplat_engine_mcmc_scored(MsplatEngine *e, const MsplatGaussians *g, const MsplatAdamState *st, int cap_max,
                              float cull_radius, int *relocation_count, const float *score, MsplatMcmcStats *out);

/* Fixed intersection budget (the reference CLI's fixed buffers,
 * cli/msplat.mm:199-235 and msplat_metal.mm:1519-1596): `slots`
 * intersection slots (20 bytes each: key, sort scratch, id) allocated once
 * instead of the legacy 48 per Gaussian and view.  A step whose views need
 * more is rastered in groups of consecutive tiles that fit: after the
 * projection and the tile counts the host reads the counts, then each group's
 * lists are built and rastered forward, the loss runs on the whole image, and
 * each group's lists are rebuilt for its backward.  Monolithic raster only
 * (steps that choose the chunked raster keep the legacy buffers); such steps
 * run eagerly (no graph).  A tile with more intersections than `slots` is an
 * error.  0 restores the legacy buffers. */
int msplat_engine_set_isect_budget(MsplatEngine *e, long long slots);

/* Launch configuration of the tunable stages (no counterpart in the
 * reference).  None changes the tile lists; sort_width, raster_batch,
 * tile_order and tile_split leave the image bit-identical (tile_split and
 * bwd_pixels change how the backward's sums are grouped), bwd_pixels changes the gradients at float rounding (the
 * order of the sums), raster_mode and chunk change the image at float
 * rounding (as the reference's own monolithic / chunked choice does). */
typedef struct {
    int sort_width;    /* CTA width of the lightest shared-memory tile sort: 256 (tiles up to
                          2048 keys) or 512 (up to 4096); default 512 */
    int raster_batch;  /* splats staged per shared-memory round in the rasterizers: 128 or 256;
                          default 128 */
    int chunk;         /* splats per depth chunk of the chunked rasterizer: 256, 512 or 1024;
                          default 512 */
    int raster_mode;   /* used when args->raster_mode is 0: 0 the reference's rule (monolithic
                          from 400 tiles), 1 monolithic, 2 chunked; default 0 */
    int tile_order;    /* how the per-tile lists get their (depth, id) order: 0 a radix sort of
                          each tile's keys, 1 one depth sort per view before the scatter, then
                          each tile's per-CTA runs put in order (same lists; views of at most
                          20480 tiles, else 0); default 1 */
    int bwd_pixels;    /* pixels per thread of the raster backward: 1 (256 threads per tile,
                          8x4-pixel warps; default) or 2 (128 threads, 8x8-pixel warps: one
                          warp reduction per 64 pixels, more work per CTA) */
    int tile_split;    /* CTAs per tile of the monolithic rasterizers (the backward with one
                          pixel per thread): 1, or 2 (default; each CTA a 16x8 half with four
                          warps, so a barrier waits on four warps, not eight; each half stages
                          the whole tile list and flushes its own gradient sums) */
} MsplatTuning;

int msplat_engine_set_tuning(MsplatEngine *e, const MsplatTuning *t);
int msplat_engine_get_tuning(MsplatEngine *e, MsplatTuning *t);

/* Autotuner: times full training steps of the given views (forward, loss,
 * backward; no optimizer update and no SGLD, so the parameters do not
 * change) under candidate configurations, one coordinate at a time (tile
 * order, sort width, CTAs per tile, tile batch, backward pixels per thread, then raster
 * mode with chunk length when args[0].raster_mode is 0), keeps the fastest (the median of `reps` timed
 * steps, after ten untimed ones; a candidate must beat the best so far by more than 1 %) and leaves
 * it set.  gt[v] must be given for every view.  `out`
 * receives the chosen configuration and *ms (nullable) its step time. */
int msplat_engine_autotune(MsplatEngine *e, const MsplatGaussians *g, const MsplatStepArgs *args, int num_views,
                           const uint8_t *const *gt, const uint8_t *const *mask, int reps, MsplatTuning *out,
                           float *ms);

/* CUDA graph mode (off by default).  When on, the second training step with
 * the same shapes, flags and buffers (parameters, moments, target, mask) is
 * captured into a CUDA graph and later such steps replay it with one launch;
 * the step scalars are uploaded before each replay, outside the graph.
 * Per-stage timing and MSPLAT_SYNC_CHECK run steps eagerly.  Growing any
 * engine buffer drops the captured graphs. */
int msplat_engine_set_graphs(MsplatEngine *e, int enabled);

/* Two CUDA events on the engine's stream for timing a span of steps:
 * marker(0) before, marker(1) after, then marker_elapsed waits for the second
 * and returns the device time between them in ms. */
int msplat_engine_marker(MsplatEngine *e, int which);
int msplat_engine_marker_elapsed(MsplatEngine *e, float *ms);

/* The engine's CUDA stream (cudaStream_t). */
void *msplat_engine_stream(MsplatEngine *e);

#ifdef __cplusplus
}
#endif

#endif
