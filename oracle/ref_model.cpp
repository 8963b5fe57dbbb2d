// The reference's host code on the path, compiled unchanged against
// oracle/model_shim.h — TEST INFRASTRUCTURE ONLY: from core/src/model.cpp
// the seed initialisation (Model::Model, setupOptimizers: 80-254, with the
// k-nearest adapter of core/include/kdtree_tensor.hpp), the MCMC pass
// (computeRelocation, relocate, addNewGaussians, mcmcAfterTrain: 311-660),
// checkpoint save and load (696-843), the camera setup (prepareCam:
// 845-889, getDownscaleFactor: 276-282) and the psnr / l1_loss metrics
// (33-49); from core/src/ssim.cpp ssim_eval (26-123); the COLMAP binary
// loader (loaders/load_colmap.cpp:7-165), the Nerfstudio and Polycam
// loaders (load_nerfstudio.cpp:7-72, load_polycam.cpp:7-95) with the point
// readers (loaders/load_ply.cpp:6-205) and autoScaleAndCenter
// (input_data.cpp:115-169), Camera::loadMask (81-111), getCameras and
// splitTrainTest (173-205); the
// Gaussian PLY / .splat files
// (loaders/save_gaussians.cpp:10-231); resizeArea (loaders/image_io.cpp:
// 115-161).  The code is copied into
// oracle/_ref/model_host.inc by oracle/ref_build.py (never committed); this
// file only wraps it for ctypes.
#include <cstdio>

#include "model_shim.h"

#include "model_host.inc"

namespace {
HostTensor host_image(const float *img, int h, int w) {
    HostTensor t;
    t.p = const_cast<float *>(img);
    t.dims = {h, w, 3};
    t.row = (int64_t)w * 3;
    return t;
}
}  // namespace

extern "C" {

// One Model::mcmcAfterTrain pass (model.cpp:497-660) over host arrays of cap
// rows whose first num_active are in use: means [cap,3], scales [cap,3],
// quats [cap,4], features_dc [cap,3], features_rest [cap,rest_floats],
// opacities [cap] and the six groups' Adam moments (row widths gstride[g]),
// all updated in place.  step, max_steps and cull_radius as the trainer
// passes them; *reloc_count is mcmc_relocation_count (the draws' seed), in
// and out.  Returns the new number of Gaussians in use.
int ref_mcmc_after_train(int cap, int num_active, int rest_floats, float *means, float *scales, float *quats,
                         float *features_dc, float *features_rest, float *opacities, float **exp_avg,
                         float **exp_avg_sq, const int *gstride, int step, int max_steps, float cull_radius,
                         int *reloc_count) {
    Model m;
    float *const arrays[6] = {means, scales, quats, features_dc, features_rest, opacities};
    const int64_t rows[6] = {3, 3, 4, 3, rest_floats, 1};
    HostTensor *bufs[6] = {&m.means_buf, &m.scales_buf, &m.quats_buf, &m.featuresDc_buf, &m.featuresRest_buf,
                           &m.opacities_buf};
    HostTensor *views[6] = {&m.means, &m.scales, &m.quats, &m.featuresDc, &m.featuresRest, &m.opacities};
    for (int g = 0; g < 6; g++) {
        bufs[g]->p = views[g]->p = arrays[g];
        bufs[g]->row = views[g]->row = rows[g];
        m.adam_exp_avg_buf[g].p = m.adam_exp_avg[g].p = exp_avg[g];
        m.adam_exp_avg_sq_buf[g].p = m.adam_exp_avg_sq[g].p = exp_avg_sq[g];
        m.adam_exp_avg_buf[g].row = m.adam_exp_avg[g].row = gstride[g];
        m.adam_exp_avg_sq_buf[g].row = m.adam_exp_avg_sq[g].row = gstride[g];
    }
    m.cap_max = cap;
    m.num_active = num_active;
    m.maxSteps = max_steps;
    m.cull_radius = cull_radius;
    m.mcmc_relocation_count = *reloc_count;
    m.mcmcAfterTrain(step);
    *reloc_count = m.mcmc_relocation_count;
    return m.num_active;
}

// Model::prepareCam (model.cpp:845-889) for a camera-to-world pose (row
// major 4x4), size and intrinsics at a step: the view and projection-view
// matrices, the camera centre, and (width, height, SH degree, degrees to
// use, tiles across, tiles down) in ints[6].
void ref_prepare_cam(const float c2w[16], int width, int height, float fx, float fy, float cx, float cy, int step,
                     int sh_degree, int sh_interval, int rest_bases, float viewmat[16], float projviewmat[16],
                     float cam_pos[3], int ints[6]) {
    Model m;
    m.shDegree = sh_degree;
    m.shDegreeInterval = sh_interval;
    m.featuresRest.dims = {1, rest_bases, 3};
    Camera cam;
    cam.width = width;
    cam.height = height;
    cam.fx = fx;
    cam.fy = fy;
    cam.cx = cx;
    cam.cy = cy;
    std::memcpy(cam.camToWorld, c2w, sizeof(cam.camToWorld));
    const Model::CamSetup s = m.prepareCam(cam, step);
    std::memcpy(viewmat, cam.cachedViewMat.data_ptr(), 64);
    std::memcpy(projviewmat, cam.cachedProjViewMat.data_ptr(), 64);
    for (int k = 0; k < 3; k++) cam_pos[k] = s.cam_pos[k];
    ints[0] = s.width;
    ints[1] = s.height;
    ints[2] = s.degree;
    ints[3] = s.degreesToUse;
    ints[4] = std::get<0>(s.tileBounds);
    ints[5] = std::get<1>(s.tileBounds);
}

// psnr, l1_loss (model.cpp:33-49) and ssim_eval with its defaults, window 11
// and sigma 1.5 (ssim.cpp:61-123, ssim.hpp:17-18), of two [h, w, 3] images.
float ref_psnr(const float *img, const float *gt, int h, int w) {
    return psnr(host_image(img, h, w), host_image(gt, h, w));
}
float ref_l1(const float *img, const float *gt, int h, int w) {
    return l1_loss(host_image(img, h, w), host_image(gt, h, w));
}
float ref_ssim_eval(const float *img, const float *gt, int h, int w) {
    return ssim_eval(host_image(img, h, w), host_image(gt, h, w), 11, 1.5f);
}

// loaders::loadColmap (load_colmap.cpp:122-165), loadNerfstudio
// (load_nerfstudio.cpp:18-72) or loadPolycam (load_polycam.cpp:18-95) of a
// dataset directory (format 0, 1, 2): its cameras in the reference's order
// with their poses after autoScaleAndCenter, and the point cloud.  Returns a
// handle, or NULL when the loader threw.
void *ref_dataset_load(const char *root, int format) {
    try {
        if (format == 1) return new InputData(loaders::loadNerfstudio(root));
        if (format == 2) return new InputData(loaders::loadPolycam(root));
        return new InputData(loaders::loadColmap(root));
    } catch (const std::exception &) {
        return nullptr;
    }
}
int ref_colmap_num_cameras(void *h) { return (int)static_cast<InputData *>(h)->cameras.size(); }
// Camera i: camera-to-world pose, (fx, fy, cx, cy), (width, height),
// (k1, k2, k3, p1, p2) and its file name relative to the image folder.
void ref_colmap_camera(void *h, int i, float c2w[16], float intr[4], int size[2], float dist[5], char *name,
                       int name_cap) {
    const Camera &c = static_cast<InputData *>(h)->cameras[(size_t)i];
    std::memcpy(c2w, c.camToWorld, 64);
    intr[0] = c.fx; intr[1] = c.fy; intr[2] = c.cx; intr[3] = c.cy;
    size[0] = c.width; size[1] = c.height;
    dist[0] = c.k1; dist[1] = c.k2; dist[2] = c.k3; dist[3] = c.p1; dist[4] = c.p2;
    std::snprintf(name, (size_t)name_cap, "%s", c.relativeName.c_str());
}
// The point cloud (xyz, rgb; either may be NULL): returns the point count.
long long ref_colmap_points(void *h, float *xyz, uint8_t *rgb) {
    const Points &p = static_cast<InputData *>(h)->points;
    if (xyz) std::memcpy(xyz, p.xyz.data(), p.xyz.size() * sizeof(float));
    if (rgb) std::memcpy(rgb, p.rgb.data(), p.rgb.size());
    return p.count;
}
void ref_colmap_transform(void *h, float *scale, float translation[3]) {
    const InputData *d = static_cast<InputData *>(h);
    *scale = d->scale;
    for (int k = 0; k < 3; k++) translation[k] = d->translation[k];
}
void ref_colmap_free(void *h) { delete static_cast<InputData *>(h); }

namespace {
HostTensor host_rows(const float *a, int64_t n, std::vector<int64_t> shape) {
    HostTensor t;
    t.p = const_cast<float *>(a);
    t.dims = std::move(shape);
    t.row = n ? t.numel() / n : 1;
    return t;
}
}  // namespace

// saveGaussianPly (save_gaussians.cpp:10-88) or, with splat, saveGaussianSplat
// (:90-139) of n Gaussians in host arrays (means [n,3], scales [n,3], quats
// [n,4], features_dc [n,3], features_rest [n,rest_bases,3], opacities [n]).
void ref_save_gaussians(const char *path, int splat, int n, int rest_bases, const float *means, const float *scales,
                        const float *quats, const float *features_dc, const float *features_rest,
                        const float *opacities, int step, int keep_crs, float scale, const float translation[3]) {
    HostTensor m = host_rows(means, n, {n, 3}), s = host_rows(scales, n, {n, 3}), q = host_rows(quats, n, {n, 4});
    HostTensor dc = host_rows(features_dc, n, {n, 3}), fr = host_rows(features_rest, n, {n, rest_bases, 3});
    HostTensor op = host_rows(opacities, n, {n, 1});
    GaussianParams p{m, s, q, dc, fr, op, scale, {translation[0], translation[1], translation[2]}, keep_crs != 0};
    if (splat)
        saveGaussianSplat(path, p);
    else
        saveGaussianPly(path, p, step);
}

// loadGaussianPly (save_gaussians.cpp:141-231): returns a handle (NULL when
// it threw); ref_loaded_info gives (rows, rest bases, iteration) and
// ref_loaded_arrays copies the arrays out in the layouts above.
void *ref_load_gaussians(const char *path, float scale, const float translation[3], int keep_crs) {
    try {
        return new LoadedGaussians(loadGaussianPly(path, scale, translation, keep_crs != 0));
    } catch (const std::exception &) {
        return nullptr;
    }
}
void ref_loaded_info(void *h, int info[3]) {
    const LoadedGaussians *g = static_cast<LoadedGaussians *>(h);
    info[0] = (int)g->means.size(0);
    info[1] = (int)g->featuresRest.size(1);
    info[2] = g->step;
}
void ref_loaded_arrays(void *h, float *means, float *scales, float *quats, float *features_dc, float *features_rest,
                       float *opacities) {
    LoadedGaussians *g = static_cast<LoadedGaussians *>(h);
    HostTensor *src[6] = {&g->means, &g->scales, &g->quats, &g->featuresDc, &g->featuresRest, &g->opacities};
    float *dst[6] = {means, scales, quats, features_dc, features_rest, opacities};
    for (int k = 0; k < 6; k++)
        if (dst[k]) std::memcpy(dst[k], src[k]->p, (size_t)src[k]->numel() * sizeof(float));
}
void ref_loaded_free(void *h) { delete static_cast<LoadedGaussians *>(h); }

namespace {
struct LoadedCheckpoint {
    Model m;
    int step = 0;
};
const int kCkptWidth[6] = {3, 3, 4, 3, 0, 1};   // group 4: 3 x rest bases
std::vector<int64_t> ckpt_shape(int g, int64_t n, int rest) {
    if (g == 4) return {n, rest, 3};
    if (g == 5) return {n, 1};
    return {n, kCkptWidth[g]};
}
}  // namespace

// Model::saveCheckpoint (model.cpp:725-764) of a model held in host arrays:
// n Gaussians at SH degree sh_degree, the six groups' parameters and Adam
// moments (layouts of the C API), learning rates and the Adam step.
void ref_save_checkpoint(const char *path, int step, int n, int sh_degree, int adam_steps, const float adam_lr[6],
                         float means_lr_init, float means_lr_final, const float *const params[6],
                         const float *const exp_avg[6], const float *const exp_avg_sq[6]) {
    Model m;
    const int rest = (sh_degree + 1) * (sh_degree + 1) - 1;
    m.shDegree = sh_degree;
    m.num_active = n;
    m.adam_step_count = adam_steps;
    for (int g = 0; g < 6; g++) m.adam_lr[g] = adam_lr[g];
    m.means_lr_init = means_lr_init;
    m.means_lr_final = means_lr_final;
    HostTensor *views[6] = {&m.means, &m.scales, &m.quats, &m.featuresDc, &m.featuresRest, &m.opacities};
    for (int g = 0; g < 6; g++) {
        *views[g] = host_rows(params[g], n, ckpt_shape(g, n, rest));
        m.adam_exp_avg[g] = host_rows(exp_avg[g], n, ckpt_shape(g, n, rest));
        m.adam_exp_avg_sq[g] = host_rows(exp_avg_sq[g], n, ckpt_shape(g, n, rest));
    }
    m.saveCheckpoint(path, step);
}

// Model::loadCheckpoint (model.cpp:766-843): a handle (NULL when it threw)
// whose ref_checkpoint_state gives (step, rows, Adam step, rest bases) and
// the eight learning rates, and ref_checkpoint_arrays the tensors.
void *ref_load_checkpoint(const char *path) {
    uint32_t head[4] = {0, 0, 0, 0};   // magic, version, step, rows: the rows size the model's buffers
    {
        std::ifstream f(path, std::ios::binary);
        f.read(reinterpret_cast<char *>(head), sizeof(head));
    }
    auto *c = new LoadedCheckpoint;
    c->m.cap_max = (int)head[3];
    try {
        c->step = c->m.loadCheckpoint(path);
        return c;
    } catch (const std::exception &) {
        delete c;
        return nullptr;
    }
}
void ref_checkpoint_state(void *h, int ints[4], float lr[8]) {
    const LoadedCheckpoint *c = static_cast<LoadedCheckpoint *>(h);
    const Model *m = &c->m;
    ints[0] = c->step;
    ints[1] = m->num_active;
    ints[2] = m->adam_step_count;
    ints[3] = (int)m->featuresRest.size(1);
    for (int g = 0; g < 6; g++) lr[g] = m->adam_lr[g];
    lr[6] = m->means_lr_init;
    lr[7] = m->means_lr_final;
}
void ref_checkpoint_arrays(void *h, float *const params[6], float *const exp_avg[6], float *const exp_avg_sq[6]) {
    Model *m = &static_cast<LoadedCheckpoint *>(h)->m;
    HostTensor *views[6] = {&m->means, &m->scales, &m->quats, &m->featuresDc, &m->featuresRest, &m->opacities};
    for (int g = 0; g < 6; g++) {
        std::memcpy(params[g], views[g]->p, views[g]->nbytes());
        std::memcpy(exp_avg[g], m->adam_exp_avg[g].p, m->adam_exp_avg[g].nbytes());
        std::memcpy(exp_avg_sq[g], m->adam_exp_avg_sq[g].p, m->adam_exp_avg_sq[g].nbytes());
    }
}
void ref_checkpoint_free(void *h) { delete static_cast<LoadedCheckpoint *>(h); }

// Model::Model and setupOptimizers (model.cpp:80-254) from n seed points:
// the Gaussians in use (the first rows of the model's cap-sized buffers)
// written to arrays of n rows in the C API's layouts; returns their count.
int ref_seed_model(int n, const float *xyz, const uint8_t *rgb, int sh_degree, int cap_max, float init_opacity,
                   float init_scale_mult, int decimate, float *means, float *scales, float *quats, float *features_dc,
                   float *features_rest, float *opacities) {
    InputData d;
    d.points.count = n;
    d.points.xyz.assign(xyz, xyz + 3 * (size_t)n);
    d.points.rgb.assign(rgb, rgb + 3 * (size_t)n);
    Model m(d, 1, sh_degree, 1000, cap_max, 5e5f, 0.01f, 0.01f, 30000, false, nullptr, 30000, decimate != 0,
            init_opacity, init_scale_mult);
    HostTensor *bufs[6] = {&m.means_buf, &m.scales_buf, &m.quats_buf, &m.featuresDc_buf, &m.featuresRest_buf,
                           &m.opacities_buf};
    float *dst[6] = {means, scales, quats, features_dc, features_rest, opacities};
    for (int g = 0; g < 6; g++) {
        const int64_t row = bufs[g]->numel() / bufs[g]->size(0);
        if (dst[g] && row) std::memcpy(dst[g], bufs[g]->p, (size_t)m.num_active * row * sizeof(float));
    }
    return m.num_active;
}

// InputData::getCameras (input_data.cpp:173-194) over cameras with the given
// image paths: the validation camera's index (or -1 without validation);
// and splitTrainTest (:196-205): test[i] = 1 for the test cameras.
int ref_val_camera(int n, const char *const *paths, int validate, const char *val_image) {
    InputData d;
    d.cameras.resize((size_t)n);
    for (int i = 0; i < n; i++) d.cameras[(size_t)i].filePath = paths[i];
    auto [train, val] = d.getCameras(validate != 0, val_image);
    (void)train;
    return val ? (int)(val - d.cameras.data()) : -1;
}
void ref_split_train_test(int n, int test_every, int *test) {
    InputData d;
    d.cameras.resize((size_t)n);
    for (int i = 0; i < n; i++) d.cameras[(size_t)i].filePath = std::to_string(i);
    auto [train, tst] = d.splitTrainTest(test_every);
    for (int i = 0; i < n; i++) test[i] = 0;
    for (const Camera &c : tst) test[std::stoi(c.filePath)] = 1;
    (void)train;
}

// Camera::loadMask (input_data.cpp:81-111) for a camera of the given size
// and image name: the mask (255 / 0, [height, width]) and the contributing
// pixel count, or -1 when the camera stays unmasked.
long long ref_load_mask(const char *mask_dir, const char *relative_name, int width, int height, uint8_t *out) {
    Camera c;
    c.width = width;
    c.height = height;
    c.relativeName = relative_name;
    c.loadMask(mask_dir);
    if (!c.gpuMask.defined()) return -1;
    std::memcpy(out, c.gpuMask.p, (size_t)width * height);
    return c.unmaskedPixels;
}

// resizeArea (loaders/image_io.cpp:115-161) of a float RGB image.
void ref_resize_area(const float *rgb, int w, int h, int dw, int dh, float *out) {
    Image src;
    src.width = w;
    src.height = h;
    src.data.assign(rgb, rgb + (size_t)w * h * 3);
    const Image r = resizeArea(src, dw, dh);
    std::memcpy(out, r.data.data(), r.data.size() * sizeof(float));
}

}  // extern "C"
