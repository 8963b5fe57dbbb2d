/*
 * msplat GB300 — host utilities and extensions of the public C API.
 *
 * The public trainer API is msplat_c_api.h (identical to the reference's
 * core/include/msplat_c_api.h); this header adds what the GB300 build needs
 * beyond it.  Each entry names the reference code it restates, or says that
 * it has no counterpart.
 */
#ifndef MSPLAT_GB300_H
#define MSPLAT_GB300_H

#include <stdbool.h>
#include <stdint.h>

#include "msplat_c_api.h"
#include "msplat_engine.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Camera matrices of Model::prepareCam (core/src/model.cpp:845-889): from a
 * row-major OpenGL camera-to-world pose to the row-major world->camera
 * matrix, projection*view (near 0.001, far 1000) and the camera centre. */
void msplat_prepare_camera(const float cam_to_world[16], int width, int height, float fx, float fy,
                           float viewmat[16], float projmat[16], float cam_pos[3]);

/* Evaluation metrics over float [H,W,3] images in [0,1]:
 * psnr / l1 (core/src/model.cpp:34-49), ssim with replicate padding
 * (core/src/ssim.cpp:61-123). */
float msplat_psnr(const float *img, const float *gt, long long n);
float msplat_l1(const float *img, const float *gt, long long n);
float msplat_ssim_eval(const float *img, const float *gt, int height, int width);

/* A dataset from host arrays — the InputData the reference's loaders build
 * (core/include/input_data.hpp:19-60): num_cameras camera-to-world poses
 * (row-major 4x4, OpenGL axes), intrinsics (fx, fy, cx, cy), sizes (width,
 * height), uint8 RGB images [H,W,3] and optional uint8 masks [H,W] (NULL),
 * plus the seed point cloud (xyz float, rgb uint8).  normalize applies the
 * reference's camera centring and scaling (input_data.cpp:115-169); with
 * eval_mode every test_every-th camera is a test camera
 * (input_data.cpp:199-208).  All inputs are copied.  NULL for negative
 * counts, missing pose, intrinsics, size or point arrays, or an empty image
 * size. */
MsplatDataset msplat_dataset_create_from_memory(int num_cameras, const float *cam_to_world, const float *intrinsics,
                                               const int *sizes, const uint8_t *const *images,
                                               const uint8_t *const *masks, int num_points, const float *xyz,
                                               const uint8_t *rgb, bool eval_mode, int test_every, bool normalize);

/* Trainer options the reference's CLI sets on its Model (cli/msplat.mm:
 * 90-131, 182-195) beyond MsplatConfig: the seed opacity and the seed scale
 * as a multiple of the mean distance to the 3 nearest seed points
 * (Model::Model, core/src/model.cpp:80-166), the subsampling of seeds above
 * 75 % of the cap to 50 % (setupOptimizers, :168-200), the length of the
 * means learning-rate decay (schedulersStep, :256-261) and the scale of the
 * opacity/scale regularizer for Gaussians not seen in a step (the step's
 * mcmc_reg_invis_scale).  msplat_default_trainer_options gives the
 * reference's defaults: 0.5, 0.1, 1, 30000, 1. */
typedef struct {
    float initOpacity;
    float initScaleMult;
    int seedDecimation;
    int positionLrMaxSteps;
    float regVisibilityDuty;
} MsplatTrainerOptions;
void msplat_default_trainer_options(MsplatTrainerOptions *options);

/* msplat_trainer_create with options (NULL: the defaults).  NULL when the
 * options are out of range (opacity in (0, 1), scale multiplier > 0,
 * decay length > 0, duty >= 0) or the trainer cannot be created. */
MsplatTrainer msplat_trainer_create_ex(MsplatDataset ds, MsplatConfig config, const MsplatTrainerOptions *options);

/* The trainer's seed initialisation on the host (Model::Model and
 * setupOptimizers, model.cpp:80-254): from num_points seed points (xyz
 * float [n,3], rgb uint8 [n,3]) at SH degree sh_degree and a cap of
 * cap_max, Gaussians in the layouts of msplat_trainer_set_gaussians written
 * to arrays of num_points rows; returns the rows in use (after seed
 * decimation or truncation to the cap), or -1 for invalid arguments. */
int msplat_seed_gaussians(int num_points, const float *xyz, const uint8_t *rgb, int sh_degree, int cap_max,
                          const MsplatTrainerOptions *options, float *means, float *scales, float *quats,
                          float *features_dc, float *features_rest, float *opacities);

/* Replaces the trainer's Gaussians (host arrays in the reference layouts, n
 * rows) and resets the optimizer, as loading a trained PLY does
 * (Model::loadPly, core/src/model.cpp:675-690).  rest_bases in [0, 15];
 * every array is required when n > 0 (features_rest only when rest_bases >
 * 0).  Returns 0, -1 for invalid arguments, -2 on a failure. */
int msplat_trainer_set_gaussians(MsplatTrainer t, int n, int rest_bases, const float *means, const float *scales,
                                 const float *quats, const float *features_dc, const float *features_rest,
                                 const float *opacities);

/* Copies the active Gaussians to host arrays (any pointer may be NULL). */
int msplat_trainer_get_gaussians(MsplatTrainer t, float *means, float *scales, float *quats, float *features_dc,
                                 float *features_rest, float *opacities);

/* Loss of the last training step (waits for the device); the reference
 * computes it in msplat_train_step but Trainer::step does not return it. */
float msplat_trainer_last_loss(MsplatTrainer t);

/* The trainer's engine (for stats, timing and buffer inspection). */
MsplatEngine *msplat_trainer_engine(MsplatTrainer t);

/* The counts of the trainer's last MCMC relocation round (dead, culled,
 * non-finite, relocated, grown, active; Model::mcmcAfterTrain's log line,
 * core/src/model.cpp:566-636).  Returns the number of rounds run so far. */
int msplat_trainer_mcmc_stats(MsplatTrainer t, MsplatMcmcStats *out);

/* Tensor-core self-test (the MMA path of the learned relocation proposal):
 * D[128 x N] = A[128 x K] * B[N x K]^T for row-major BF16 A, B (host, as
 * uint16 bit patterns) into row-major F32 D (host), N, K in {16, 32, 64}, on
 * the current device.  Returns 0, or -1 (bad size), -2 (CUDA error), -3 (the
 * MMA did not complete within the wait limit). */
int msplat_tc_gemm_check(const uint16_t *A, const uint16_t *B, float *D, int N, int K);

/* Host-side views of a dataset (no counterpart in the reference's C API):
 * camera i of the training (use_test = 0) or test list — intrinsics
 * (fx, fy, cx, cy), size (width, height), camera-to-world (OpenGL axes,
 * row-major) and the 8-bit RGB image [H,W,3]; any output may be NULL.
 * Returns 0, or -1 for a bad index. */
int msplat_dataset_camera(MsplatDataset ds, int i, int use_test, float intrinsics[4], int size[2], float c2w[16],
                          uint8_t *image);

/* msplat_dataset_create with the COLMAP image folder given explicitly (the
 * reference CLI's --colmap-image-path); NULL = images/ next to the model. */
MsplatDataset msplat_dataset_create_ex(const char *path, float downscaleFactor, bool evalMode, int testEvery,
                                       const char *colmapImagePath);

/* msplat_dataset_create_ex with training masks from maskDir (the reference
 * CLI's --mask-dir, Camera::loadMask, core/src/input_data.cpp:81-111): for
 * each camera "<maskDir>/<name>.png", else the name with its extension
 * replaced by .png (name: the image's path under the image folder), resized
 * to the camera's final size by area averaging; a pixel contributes where
 * the mask's first channel is above 0.5; an all-white mask, or none, leaves
 * the camera unmasked.  As in the reference, only COLMAP datasets name their
 * images for the lookup.  maskDir NULL or "": no masks. */
MsplatDataset msplat_dataset_create_masked(const char *path, float downscaleFactor, bool evalMode, int testEvery,
                                           const char *colmapImagePath, const char *maskDir);

/* Camera i's image file (disk datasets; "" for in-memory ones) written to
 * path (capacity bytes, NUL-terminated): returns its length, or -1 for a
 * bad index.  msplat_dataset_transform gives the centring and scaling the
 * loader applied (autoScaleAndCenter, core/src/input_data.cpp:115-169):
 * positions in the dataset's own frame are x / scale + translation. */
int msplat_dataset_camera_file(MsplatDataset ds, int i, int use_test, char *path, int capacity);
int msplat_dataset_transform(MsplatDataset ds, float *scale, float translation[3]);

/* The reference CLI's --val (InputData::getCameras, core/src/input_data.cpp:
 * 173-194): withholds one training camera as the dataset's only test camera
 * — val_image "random" (or NULL) picks mt19937(42)'s first draw modulo the
 * camera count, otherwise the first camera whose image path contains
 * val_image (the first camera when none does).  Returns the index it had
 * among the training cameras, or -1 when the dataset already has test
 * cameras (eval mode) or no cameras. */
int msplat_dataset_hold_out(MsplatDataset ds, const char *val_image);

/* Camera i's training mask (255 = contributes, 0 = ignored; [H,W], may be
 * NULL to ask only): returns the number of contributing pixels, -1 when the
 * camera has no mask, -2 for a bad index. */
long long msplat_dataset_mask(MsplatDataset ds, int i, int use_test, uint8_t *mask);

/* Learned relocation proposal (no counterpart in the reference; off by
 * default): per-Gaussian activity statistics are gathered during the steps,
 * a 22-64-64-2 MLP on the tensor cores is trained every 500 steps on the
 * run's own (state -> opacity and activity 500 steps later) pairs, and once
 * trained, at each relocation round, its predictions replace sigmoid(opacity)
 * as the weights of the MCMC source draws and the Gaussians it forecasts to
 * fade (opacity one window ahead at most the forecast-pruning threshold,
 * 0.02 unless set below) are relocated with the dead ones.  Returns 0 or a
 * negative code. */
int msplat_trainer_set_learned_relocation(MsplatTrainer t, int enabled);

/* The learned proposal's forecast-pruning threshold (no counterpart in the
 * reference): Gaussians whose forecast opacity one window ahead is at most
 * `forecast_opacity` are relocated with the dead ones (at most 5 % of them
 * per round); 0 turns forecast pruning off (source weighting only); default
 * 0.02.  Returns 0, or -1 for a bad handle or a threshold outside [0, 1). */
int msplat_trainer_set_learned_prune(MsplatTrainer t, float forecast_opacity);

/* Last training loss of the proposal MLP and its training rounds so far;
 * returns 1 when the proposal is enabled, 0 when not, -1 on a bad handle. */
int msplat_trainer_learned_stats(MsplatTrainer t, float *last_loss, int *rounds);

/* Held-out quality of the learned proposal's predictions (no counterpart in
 * the reference: it measures this build's MLP).  At each training round after
 * the first, before the MLP trains on the round's new labels, it predicts
 * them: mse[0] / mse[1] are the mean squared errors of its opacity forecast
 * and of the persistence forecast (the Gaussian's opacity at the snapshot),
 * mse[2] / mse[3] the same for the activity forecast (persistence: its mean
 * activity at the snapshot), averaged over rounds.  Returns the rounds
 * evaluated. */
int msplat_trainer_learned_eval(MsplatTrainer t, float mse[4]);

/* Views per optimizer step (no counterpart in the reference; default 1).
 * With num_views > 1 each msplat_trainer_step renders the next num_views
 * cameras of the shuffled order and applies one update from the mean of
 * their gradients (msplat_engine_train_step_batch), with the learning rates
 * multiplied by lr_scale (<= 0: num_views^0.75).  The iteration counter
 * counts views: a step advances it by num_views, and the schedules keyed on
 * it (learning-rate decay, SH degree, regularizer start, MCMC every 100
 * iterations, the learned proposal's window) fire when their boundary is
 * crossed.  Returns 0, or -1 on a bad handle or num_views outside 1..16. */
int msplat_trainer_set_batch_views(MsplatTrainer t, int num_views, float lr_scale);

/* Fixed intersection budget of the reference CLI (cli/msplat.mm:199-235):
 * bytes_per_gaussian x the Gaussian cap of intersection buffers, allocated
 * once (at least one slot per Gaussian of the cap); views that need more are
 * rastered in tile groups (msplat_engine_set_isect_budget).  0 = the legacy
 * buffers grown with the model.  Returns 0 or a negative code. */
int msplat_trainer_set_isect_budget(MsplatTrainer t, float bytes_per_gaussian);

/* Runs the engine's autotuner (msplat_engine_autotune) on the trainer's
 * next training cameras (as many as the views per step) and keeps the
 * fastest launch configuration for the rest of the run; `out` (nullable)
 * receives it.  The parameters are not changed.  Returns 0 or a negative
 * code. */
int msplat_trainer_autotune(MsplatTrainer t, MsplatTuning *out);

/* Replaces the trainer's Gaussians with a trained PLY (Model::loadPly, the
 * CLI's --resume); optimizer state starts fresh.  Returns the iteration
 * recorded in the file, or a negative code. */
int msplat_trainer_load_ply(MsplatTrainer t, const char *path);

/* Seed points (xyz [N,3] in training coordinates, rgb [N,3]); either output
 * may be NULL.  Returns N. */
int msplat_dataset_points(MsplatDataset ds, float *xyz, uint8_t *rgb);

/* Decodes an image file (PNG, baseline JPEG, binary PPM/PGM) to float RGB in
 * [0, 1]; with rgb == NULL only the size is returned.  Returns 0, or a
 * negative code with the reason on stderr. */
int msplat_image_read(const char *path, float *rgb, int *width, int *height);

/* Area-averaging resize of a float RGB image [height, width, 3] to
 * [out_height, out_width, 3] (resizeArea, core/src/loaders/image_io.cpp:
 * 115-161: the dataset's --downscale-factor and the masks' resize).
 * Returns 0, or -1 for invalid arguments. */
int msplat_image_resize(const float *rgb, int width, int height, int out_width, int out_height, float *out);

/* Reads and validates a checkpoint file (the reference's format,
 * core/src/model.cpp:698-843) on the host, without a trainer: every tensor
 * must hold N rows of its group's width and exactly N x width x 4 bytes.
 * Writes N, the SH degree and the iteration (any output may be NULL).
 * Returns 0, or -1 when the file is missing or malformed (reason on
 * stderr).  msplat_trainer_load_checkpoint applies the same checks. */
int msplat_checkpoint_info(const char *path, int *num_points, int *sh_degree, int *iteration);

/* Writes and reads a checkpoint (Model::saveCheckpoint / loadCheckpoint,
 * core/src/model.cpp:698-843) from host arrays, with the trainer's own code:
 * params, exp_avg and exp_avg_sq each point at the six groups (means [n,3],
 * log-scales [n,3], quaternions [n,4], features_dc [n,3], features_rest
 * [n,(sh_degree+1)^2-1,3], opacity logits [n]); adam_lr holds the six
 * groups' learning rates.  msplat_read_checkpoint fills arrays of the sizes
 * msplat_checkpoint_info gives (any output may be NULL) after the same
 * validation.  Return 0, -1 for invalid arguments, -2 when the file cannot
 * be written or is missing or malformed (reason on stderr). */
int msplat_write_checkpoint(const char *path, int iteration, int n, int sh_degree, int adam_steps,
                            const float adam_lr[6], float means_lr_init, float means_lr_final,
                            const float *const params[6], const float *const exp_avg[6],
                            const float *const exp_avg_sq[6]);
int msplat_read_checkpoint(const char *path, float adam_lr[6], float means_lr[2], int *adam_steps,
                           float *const params[6], float *const exp_avg[6], float *const exp_avg_sq[6]);

/* Host-side PLY and .splat files of Gaussians held by the caller (host
 * arrays in the reference layouts, n rows: means [n,3], log-scales [n,3],
 * quaternions [n,4], features_dc [n,3], features_rest [n,rest_bases,3],
 * opacity logits [n]), without a trainer — for models trained through the
 * differentiable renderer, say.  They are the trainer's own writers:
 * msplat_write_ply is saveGaussianPly (core/src/loaders/save_gaussians.cpp:
 * 10-88: non-finite Gaussians dropped, f_rest channel-major, the iteration
 * comment), msplat_write_splat is saveGaussianSplat (:90-139: 32 B per
 * Gaussian, largest first).  With keep_crs the positions and scales are
 * mapped back to the dataset's frame: x / scale + translation, log(e^s /
 * scale).  Return 0, -1 for invalid arguments, -2 when the file cannot be
 * written (reason on stderr). */
int msplat_write_ply(const char *path, int n, int rest_bases, const float *means, const float *scales,
                     const float *quats, const float *features_dc, const float *features_rest,
                     const float *opacities, int step, int keep_crs, float scale, const float translation[3]);
int msplat_write_splat(const char *path, int n, int rest_bases, const float *means, const float *scales,
                       const float *quats, const float *features_dc, const float *features_rest,
                       const float *opacities, int keep_crs, float scale, const float translation[3]);

/* A Gaussian PLY read as loadGaussianPly does (save_gaussians.cpp:141-231):
 * msplat_ply_info gives its rows, rest bases and iteration (any output may
 * be NULL); msplat_read_ply fills caller arrays of those sizes (the layouts
 * above), with keep_crs mapping the file's frame into the dataset's:
 * (x - translation) * scale, log(scale e^s).  Return 0, -1 for invalid
 * arguments, -2 for a missing or malformed file (reason on stderr). */
int msplat_ply_info(const char *path, int *num_points, int *rest_bases, int *iteration);
int msplat_read_ply(const char *path, int keep_crs, float scale, const float translation[3], float *means,
                    float *scales, float *quats, float *features_dc, float *features_rest, float *opacities);

/* SSIM + L1 training loss and dL/dimage without any device allocation.
 * No counterpart in the reference: it is for callers that cannot call
 * cudaMalloc (a host application or server that owns all device memory
 * through its own allocator, or a loop that cannot take cudaMalloc's
 * implicit synchronisation).  The same kernel as the training step, which
 * keeps its intermediates in shared memory; the three step scalars live in
 * the library's static device copy, so any image size works.  All calls on a
 * device share that copy: calls that overlap on the GPU race.  The first call
 * on a device looks up its address; make it before any stream capture.
 * img: device float [H,W,3]; gt: device uint8 [H,W,3]; mask: device uint8
 * [H,W] or NULL; v_img: device float [H,W,3] (out); loss_sum: device float
 * (out, loss_sum / (H*W) is the loss); stream: cudaStream_t or NULL.
 * Returns 0, or a negative code. */
int msplat_loss_ssim_l1_noalloc(const float *img, const uint8_t *gt, const uint8_t *mask, int width, int height,
                                float ssim_weight, float loss_inv_n, float *v_img, float *loss_sum, void *stream);

#ifdef __cplusplus
}
#endif

#endif
