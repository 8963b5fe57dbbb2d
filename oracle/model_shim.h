// Host stand-ins for the reference's Model class (core/include/model.hpp:
// 17-130), its Camera, Points and InputData (core/include/input_data.hpp:
// 19-65), the loader and Gaussian-file declarations (core/include/
// loaders.hpp) and MTensor,
// with only the members the host code compiled by ref_model.cpp uses (the
// seed initialisation, MCMC pass, camera setup, evaluation metrics,
// checkpoints, the COLMAP, Nerfstudio and Polycam loaders, the Gaussian PLY
// / .splat files), so that
// code compiles unchanged — TEST INFRASTRUCTURE ONLY (it pins the oracle's
// and the library's restatements; nothing in the product uses it).
//
// The reference keeps each parameter group and Adam moment as an MTensor
// (core/include/metal_tensor.hpp) whose storage is shared with the GPU; here
// a HostTensor is a row-major float array with the accessors the code calls
// (data<T>(), stride0() = the floats per row, size(d), numel(), defined(),
// data_ptr()).  The `*_buf` tensors and their active views (means,
// opacities, ...) are the same arrays, as in the reference after
// refreshViews().
#pragma once

#include "json_shim.h"        // nlohmann::json, for the Nerfstudio and Polycam loaders
#include "nanoflann_shim.h"   // nanoflann, for the seed scales' k-nearest search

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <filesystem>
#include <fstream>
#include <limits>
#include <memory>
#include <numeric>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#define BLOCK_X 16
#define BLOCK_Y 16

struct HostTensor {
    float *p = nullptr;
    int64_t row = 1;
    std::vector<int64_t> dims;                   // for size(d), numel() and shape()
    std::shared_ptr<std::vector<float>> owned;   // storage of gpu_empty tensors
    template <class T> T *data() { return reinterpret_cast<T *>(p); }
    template <class T> const T *data() const { return reinterpret_cast<const T *>(p); }
    int64_t stride0() const { return row; }
    int64_t size(int d) const { return dims[d < 0 ? (int)dims.size() + d : d]; }
    int64_t numel() const {
        int64_t n = 1;
        for (int64_t s : dims) n *= s;
        return n;
    }
    std::vector<int64_t> shape() const { return dims; }
    bool defined() const { return p != nullptr; }
    void reset() { *this = HostTensor(); }
    void *data_ptr() { return p; }
    const void *data_ptr() const { return p; }
    uint32_t ndim() const { return (uint32_t)dims.size(); }
    uint64_t nbytes() const { return (uint64_t)numel() * sizeof(float); }
};
using MTensor = HostTensor;

enum class DType { Float32, UInt8 };
inline HostTensor gpu_empty(const std::vector<int64_t> &shape, DType) {
    HostTensor t;
    t.dims = shape;
    t.owned = std::make_shared<std::vector<float>>((size_t)t.numel());
    t.p = t.owned->data();
    t.row = t.dims.size() > 1 ? t.numel() / t.dims[0] : 1;
    return t;
}
inline HostTensor gpu_empty(std::initializer_list<int64_t> shape, DType d) {
    return gpu_empty(std::vector<int64_t>(shape), d);
}
inline HostTensor gpu_zeros(const std::vector<int64_t> &shape, DType d) { return gpu_empty(shape, d); }
inline HostTensor gpu_zeros(std::initializer_list<int64_t> shape, DType d) { return gpu_empty(shape, d); }

namespace fs = std::filesystem;

struct Camera {
    int width = 0, height = 0;
    float fx = 0, fy = 0, cx = 0, cy = 0;
    float k1 = 0, k2 = 0, k3 = 0, p1 = 0, p2 = 0;
    float camToWorld[16] = {};
    std::string filePath;
    std::string relativeName;
    MTensor gpuMask;
    int64_t unmaskedPixels = -1;
    void loadMask(const std::string &maskDir);
    MTensor cachedViewMat, cachedProjViewMat;
    float cachedCamPos[3] = {};
    float cachedFovX = 0, cachedFovY = 0;
};

struct Image {
    std::vector<float> data;
    int width = 0, height = 0;
    bool empty() const { return data.empty(); }
    float *ptr() { return data.data(); }
    const float *ptr() const { return data.data(); }
};

// The reference decodes images through CoreGraphics (loaders/image_io.cpp:
// 13-56), which is not here; this stand-in decodes 8-bit binary PGM / PPM
// (grey replicated to RGB, values / 255), enough for the masks the tests
// write.  An unreadable file decodes empty.
inline Image imreadRGB(const std::string &path) {
    Image im;
    std::ifstream f(path, std::ios::binary);
    std::string magic;
    int w = 0, h = 0, maxv = 0;
    if (!(f >> magic >> w >> h >> maxv) || (magic != "P5" && magic != "P6") || maxv != 255 || w <= 0 || h <= 0)
        return im;
    f.get();
    const int ch = magic == "P6" ? 3 : 1;
    std::vector<unsigned char> raw((size_t)w * h * ch);
    f.read(reinterpret_cast<char *>(raw.data()), (std::streamsize)raw.size());
    im.width = w;
    im.height = h;
    im.data.resize((size_t)w * h * 3);
    for (size_t i = 0; i < (size_t)w * h; i++)
        for (int c = 0; c < 3; c++) im.data[i * 3 + c] = raw[i * ch + (ch == 3 ? c : 0)] / 255.0f;
    return im;
}
Image resizeArea(const Image &src, int dstW, int dstH);

struct Points {
    std::vector<float> xyz;
    std::vector<uint8_t> rgb;
    int64_t count = 0;
};

struct InputData {
    std::vector<Camera> cameras;
    float scale = 1.0f;
    float translation[3] = {};
    Points points;
    std::tuple<std::vector<Camera>, Camera *> getCameras(bool validate, const std::string &valImage = "random");
    std::tuple<std::vector<Camera>, std::vector<Camera>> splitTrainTest(int testEvery);
};

namespace loaders {
InputData loadColmap(const std::string &projectRoot, const std::string &imageSourcePath = "");
InputData loadNerfstudio(const std::string &projectRoot);
InputData loadPolycam(const std::string &projectRoot);
}
Points readPly(const std::string &path);
Points readColmapPoints(const std::string &path);
void autoScaleAndCenter(InputData &data);

struct GaussianParams {
    MTensor &means, &scales, &quats, &featuresDc, &featuresRest, &opacities;
    float scale;
    float translation[3];
    bool keepCrs;
};
struct LoadedGaussians {
    MTensor means, scales, quats, featuresDc, featuresRest, opacities;
    int step;
};
void saveGaussianPly(const std::string &path, GaussianParams &p, int step);
void saveGaussianSplat(const std::string &path, GaussianParams &p);
LoadedGaussians loadGaussianPly(const std::string &path, float scale, const float translation[3], bool keepCrs);

// GPU hooks the MCMC pass calls (core/metal/bindings.h): nothing to wait for
// on the host, and no gradient NaN counters to report.
inline void msplat_gpu_sync() {}
inline void msplat_grad_nan_counts(uint32_t out[16]) {
    for (int k = 0; k < 16; k++) out[k] = 0;
}

class Model {
public:
    Model() = default;
    Model(const InputData &inputData, int numCameras, int shDegree, int shDegreeInterval, int capMax, float noiseLr,
          float opacityReg, float scaleReg, int maxSteps, bool keepCrs, const float *bgColor = nullptr,
          int positionLrMaxSteps = 30000, bool decimateSeeds = true, float initOpacity = 0.5f,
          float initScaleMult = 0.1f);
    void setupOptimizers(bool decimateSeeds);
    void releaseOptimizers();
    int numCameras = 0;
    bool keepCrs = false;
    float noise_lr = 0.f, opacity_reg = 0.f, scale_reg = 0.f;
    int position_lr_max_steps_ = 30000;
    float scale = 1.f;
    float translation[3] = {};
    HostTensor backgroundColor;
    static constexpr int N_ADAM_GROUPS = 6;
    HostTensor means_buf, scales_buf, quats_buf, featuresDc_buf, featuresRest_buf, opacities_buf;
    HostTensor means, scales, quats, featuresDc, featuresRest, opacities;
    HostTensor adam_exp_avg_buf[N_ADAM_GROUPS], adam_exp_avg_sq_buf[N_ADAM_GROUPS];
    HostTensor adam_exp_avg[N_ADAM_GROUPS], adam_exp_avg_sq[N_ADAM_GROUPS];
    int num_active = 0;
    int mcmc_relocation_count = 0;
    std::vector<float> scratch_probs_;
    std::vector<int> scratch_count_;
    int maxSteps = 0;
    int cap_max = 0;
    float cull_radius = 0.0f;
    int shDegree = 3;
    int shDegreeInterval = 1000;
    float adam_lr[N_ADAM_GROUPS] = {};
    float means_lr_init = 0.f, means_lr_final = 0.f;
    int adam_step_count = 0;
    int buf_capacity = 0;
    HostTensor sgld_noise_buf;
    void saveCheckpoint(const std::string &filename, int step);
    int loadCheckpoint(const std::string &filename);

    struct CamSetup {
        float fx, fy, cx, cy;
        int height, width, degree, degreesToUse;
        std::tuple<int, int, int> tileBounds;
        float cam_pos[3];
    };
    CamSetup prepareCam(Camera &cam, int step);
    int getDownscaleFactor(int step);

    void refreshViews() {}
    void computeRelocation(float opacity_old_sig, float *scale_old_exp, int N, float &opacity_new_sig,
                           float *scale_new_exp);
    void relocate(const std::vector<int> &dead, const std::vector<int> &alive);
    int addNewGaussians();
    void mcmcAfterTrain(int step);
};
