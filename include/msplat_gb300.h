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

#include <stdint.h>

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

#ifdef __cplusplus
}
#endif

#endif
