/*
 * msplat CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * A scalar C++ restatement of the msplat (semhfe/msplat v1.1.3) training step:
 * the Metal kernels of core/metal/msplat_metal.metal and the host step logic of
 * core/src/model.cpp and core/metal/msplat_metal.mm.  It exists to check the
 * CUDA engine and to be timed as the CPU baseline.  Nothing in the product
 * (msplat_gb300/) may link, load or call it.
 *
 * Two precisions share one templated transcription:
 *   prec = 64 : every intermediate in double (the FP64 reference answer);
 *   prec = 32 : every intermediate in float, operations in the order the
 *               reference writes them, fused only where it writes fma(), with
 *               its own deterministic exp (Cody-Waite reduction + degree-7
 *               Taylor polynomial).  The CUDA engine follows the same sequence,
 *               so integer outputs (radii, tile rects, tile lists) and the
 *               forward image match bit for bit.
 *
 * Parity pin: the only known-answer test the reference ships for this path is
 * tests/test_relocation.cpp (Eq. 9 invariants), which or_compute_relocation
 * passes (tests/test_oracle.py).  Projection, tile lists, raster, SSIM, Adam
 * and SGLD have no reference golden vectors (the reference is Metal-only and
 * cannot run here), so for those stages the oracle is pinned only by being a
 * line-by-line restatement, by FP64 finite-difference checks of its gradients
 * and by the committed fixtures it generated (tests/golden/).
 */
#ifndef MSPLAT_ORACLE_H
#define MSPLAT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    /* sizes */
    int num_points;      /* N */
    int rest_bases;      /* features_rest second dim (15 at SH degree 3) */
    int width, height;
    /* camera (model.cpp:845-889 prepareCam outputs) */
    float viewmat[16], projmat[16];
    float fx, fy, cx, cy;
    float cam_pos[3];
    float background[3];
    float clip_thresh;   /* 0.01 in the reference */
    int degrees_to_use;
    /* parameters; updated in place when do_optimizer (cap-free: N rows) */
    float *means, *scales, *quats, *features_dc, *features_rest, *opacities;
    float *exp_avg[6], *exp_avg_sq[6];     /* groups: means scales quats dc rest opacity */
    float step_size[6], bc2_sqrt[6];
    float beta1, beta2, eps;
    float op_reg, sc_reg, invis_scale;
    /* loss */
    const uint8_t *gt;    /* H*W*3 */
    const uint8_t *mask;  /* H*W or NULL */
    float ssim_weight, loss_inv_n;
    /* raster: 0 = reference rule (chunked iff tiles < 400), 1 = monolithic, 2 = chunked */
    int raster_mode;
    int k_max;            /* chunk count for the chunked raster; 0 = reference rule */
    long long isect_capacity; /* 0 = 48 * N (reference legacy capacity) */
    /* SGLD (model.cpp:971-974) */
    int do_sgld;
    uint32_t seed;
    float noise_lr, xyz_lr, max_disp;
    int do_backward;      /* 0: forward (+ loss when gt != NULL) only */
    int do_optimizer;     /* SH Adam, reg, 4-group Adam */
    int no_cutoff;        /* test switch: drop the sigma >= 5.55 and alpha < 1/255
                             cutoffs (finite-difference checks of the VJPs) */
    const float *v_img_in; /* H*W*3 or NULL: backward from this dL/dimage instead
                             of the loss's (the autograd binding's contract) */
    int tile_row_lo, tile_row_hi; /* hi > lo: only tiles in rows [lo, hi) get
                             lists and are rasterized forward and backward
                             (heavy-view checks on a band; other tiles stay
                             empty) */
    const float *raster_grads_in; /* N*9 or NULL: per-Gaussian rasterizer
                             gradients (v_xy 2, v_conic 3, v_colors 3,
                             v_opacity 1) used instead of running the raster
                             backward (checks of the projection backward,
                             SH Adam, regularizer and Adam in isolation) */
} OrStepIn;

typedef struct {
    /* every pointer may be NULL */
    float *xys, *depths, *conics, *colors, *aabb;
    int *radii, *num_tiles_hit;
    int *tile_counts;      /* [T] */
    int *tile_bins;        /* [T,2] */
    int *gaussian_ids;     /* [min(M, ids_capacity)] sorted per tile */
    long long ids_capacity;
    long long num_isect;   /* M (out) */
    float *out_img, *final_Ts;
    int *final_idx;
    double loss;           /* loss_sum / (H*W), as msplat_train_step returns */
    float *v_rendered;
    float *v_xy, *v_conic, *v_colors, *v_opacity;   /* rasterizer gradients */
    float *v_mean3d, *v_scale, *v_quat;            /* projection gradients (pre-reg) */
    uint32_t nan_counts[16];
    int k_max_used;        /* 1 = monolithic */
    long long pairs_fwd, pairs_bwd;  /* (pixel, splat) evaluations executed */
    double img_dot_v;     /* sum of image * v_img_in at the step's precision (the linear
                             loss whose gradient the backward of v_img_in is) */
} OrStepOut;

/* One training step (prec = 32 or 64).  Returns 0 on success. */
int or_train_step(int prec, const OrStepIn *in, OrStepOut *out);

/* Deterministic float exp shared (by algorithm) with the CUDA engine. */
float or_det_expf(float x);
void or_gauss_1d(float out[11]);   /* the 11-tap SSIM window of the float path */

/* Eq. 9 relocation (model.cpp:311-332), exactly as the reference computes it. */
void or_compute_relocation(float opacity_old_sig, const float *scale_old_exp, int n,
                           float *opacity_new_sig, float *scale_new_exp);

/* prepareCam (model.cpp:845-889): camToWorld row-major 4x4 (OpenGL axes) ->
   viewmat, projview, cam_pos. */
void or_prepare_cam(const float cam_to_world[16], int width, int height, float fx, float fy,
                    float viewmat[16], float projmat[16], float cam_pos[3]);

/* Evaluation metrics (model.cpp:34-49, ssim.cpp:61-123). img, gt: H*W*3 float. */
double or_psnr(const float *img, const float *gt, long long n);
double or_l1(const float *img, const float *gt, long long n);
double or_ssim_eval(const float *img, const float *gt, int height, int width);

/* MCMC (model.cpp:497-566): dead flags for n Gaussians; returns the dead count. */
int or_mcmc_dead_mask(int n, int rest_stride, const float *means, const float *scales,
                      const float *quats, const float *features_dc, const float *features_rest,
                      const float *opacities, float cull_radius, uint8_t *dead_out);

/* Apply a relocation whose sources are already chosen (relocate + addNewGaussians,
   model.cpp:336-495).  dst[i] receives a copy of src[i]; each distinct source
   with c copies is first rescaled by Eq. 9 with n = c + 1; moments of every
   touched row are zeroed.  Arrays are full-capacity row-major buffers. */
void or_mcmc_apply(int n_moves, const int *dst, const int *src, int rest_stride,
                   float *means, float *scales, float *quats, float *features_dc,
                   float *features_rest, float *opacities,
                   float **exp_avg, float **exp_avg_sq, const int *group_stride);

int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
