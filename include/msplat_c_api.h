/*
 * msplat public C API, implemented by the GB300 engine.
 *
 * Every declaration keeps the name, argument list, struct layout and
 * ownership rule of the reference's core/include/msplat_c_api.h (v1.1.3), so
 * its Swift package (swift/Sources/Msplat) and other C callers link against
 * this library without source changes.  Differences of behaviour are limited
 * to error handling: where the reference throws or exits, these functions
 * log to stderr and return NULL / 0 / an empty buffer.
 */
#ifndef MSPLAT_C_API_H
#define MSPLAT_C_API_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Training configuration (reference: msplat_c_api.h:16-30). */
typedef struct {
    int iterations;
    int shDegree;
    int shDegreeInterval;
    float ssimWeight;
    int capMax;            /* Gaussian budget of MCMC densification */
    float noiseLr;         /* SGLD noise learning rate */
    float opacityReg;
    float scaleReg;
    float cullRadius;      /* relocate Gaussians with |mean| > cullRadius (0 = off) */
    bool keepCrs;          /* export in the dataset's original coordinates */
    float downscaleFactor;
    float bgColor[3];
} MsplatConfig;

/* Defaults of the reference (msplat_c_api.h:32-47). */
static inline MsplatConfig msplat_default_config(void) {
    MsplatConfig c;
    c.iterations = 30000;
    c.shDegree = 3;
    c.shDegreeInterval = 1000;
    c.ssimWeight = 0.2f;
    c.capMax = 1000000;
    c.noiseLr = 5e5f;
    c.opacityReg = 0.01f;
    c.scaleReg = 0.01f;
    c.cullRadius = 3.0f;
    c.keepCrs = false;
    c.downscaleFactor = 1.0f;
    c.bgColor[0] = 0.6130f;
    c.bgColor[1] = 0.0101f;
    c.bgColor[2] = 0.3984f;
    return c;
}

typedef struct {
    int iteration;
    int splatCount;
    float msPerStep;
} MsplatStats;

typedef struct {
    float psnr;
    float ssim;
    float l1;
    int numTest;
    int numGaussians;
} MsplatEvalMetrics;

/* RGB float32 image, [height, width, 3]; data is malloc()ed — the caller free()s it. */
typedef struct {
    float *data;
    int width;
    int height;
} MsplatPixelBuffer;

/* ---- Dataset ---- */

typedef void *MsplatDataset;

MsplatDataset msplat_dataset_create(const char *path, float downscaleFactor, bool evalMode, int testEvery);
void msplat_dataset_destroy(MsplatDataset ds);
int msplat_dataset_num_train(MsplatDataset ds);
int msplat_dataset_num_test(MsplatDataset ds);

/* ---- Trainer ---- (the dataset must outlive the trainer) */

typedef void *MsplatTrainer;

MsplatTrainer msplat_trainer_create(MsplatDataset ds, MsplatConfig config);
void msplat_trainer_destroy(MsplatTrainer t);

MsplatStats msplat_trainer_step(MsplatTrainer t);
void msplat_trainer_train(MsplatTrainer t);
MsplatEvalMetrics msplat_trainer_evaluate(MsplatTrainer t);
MsplatPixelBuffer msplat_trainer_render(MsplatTrainer t, int cameraIndex, bool useTest);
MsplatPixelBuffer msplat_trainer_render_pose(MsplatTrainer t, const float camToWorld[16], int refCameraIndex);

/* Renders into caller memory as RGBA8 (width*height*4 bytes); with
 * outRGBA == NULL only the dimensions are returned. */
void msplat_trainer_render_pose_to_buffer(MsplatTrainer t, const float camToWorld[16], int refCameraIndex,
                                          uint8_t *outRGBA, int *outWidth, int *outHeight);
void msplat_trainer_export_ply(MsplatTrainer t, const char *path);
void msplat_trainer_export_splat(MsplatTrainer t, const char *path);
void msplat_trainer_save_checkpoint(MsplatTrainer t, const char *path);
int msplat_trainer_load_checkpoint(MsplatTrainer t, const char *path);
int msplat_trainer_splat_count(MsplatTrainer t);
int msplat_trainer_iteration(MsplatTrainer t);
void msplat_dataset_camera_pose(MsplatDataset ds, int cameraIndex, float camToWorld[16]);

/* ---- Lifecycle ---- */

void msplat_set_metallib_path(const char *path);   /* no effect on GB300 */
void msplat_sync(void);
void msplat_cleanup(void);

/* ---- Viewer (render-only) ---- */

typedef void *MsplatViewer;

MsplatViewer msplat_viewer_create(const char *plyPath, int width, int height, float fovY);
void msplat_viewer_resize(MsplatViewer v, int width, int height);
void msplat_viewer_set_fov(MsplatViewer v, float fovY);
void msplat_viewer_set_background(MsplatViewer v, float r, float g, float b);
void msplat_viewer_render(MsplatViewer v, const float camToWorld[16], uint8_t *outRGBA);
int msplat_viewer_splat_count(MsplatViewer v);
void msplat_viewer_get_size(MsplatViewer v, int *outWidth, int *outHeight);
/* On GB300: a device pointer to float RGB [H*W*3], valid until the next render. */
void *msplat_viewer_render_buffer(MsplatViewer v, const float camToWorld[16], int *outWidth, int *outHeight);
void msplat_viewer_bounds(MsplatViewer v, float boundsMin[3], float boundsMax[3]);
void msplat_viewer_density_center(MsplatViewer v, float center[3]);
/* On GB300: the viewer's cudaStream_t. */
void *msplat_viewer_command_queue(MsplatViewer v);
void msplat_viewer_destroy(MsplatViewer v);

#ifdef __cplusplus
}
#endif

#endif
