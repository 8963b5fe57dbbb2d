// The reference's public C API (include/msplat_c_api.h) over the GB300
// engine: dataset, trainer (Model + Trainer of core/src/model.cpp and
// core/src/msplat_api.mm), render-only viewer, PLY / .splat / checkpoint I/O.
// Parameters and Adam moments live in cap-sized device buffers with an
// N-row active prefix, as in the reference (model.cpp:168-254).
#include <algorithm>
#include <thread>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <memory>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "msplat_c_api.h"
#include "msplat_engine.h"
#include "dataset_io.h"
#include "mlp.h"
#include "msplat_gb300.h"

namespace msplat {

static const double kShC0 = 0.28209479177387814;

#define CKA(x)                                                                                 \
    do {                                                                                       \
        cudaError_t err_ = (x);                                                                \
        if (err_ != cudaSuccess)                                                               \
            throw std::runtime_error(std::string(#x) + ": " + cudaGetErrorString(err_));       \
    } while (0)

static int sh_bases_for_degree(int d) { return d <= 0 ? 1 : d == 1 ? 4 : d == 2 ? 9 : d == 3 ? 16 : 25; }
static int degree_for_rest(int rest) {
    const int b = rest + 1;
    return b <= 1 ? 0 : b <= 4 ? 1 : b <= 9 ? 2 : b <= 16 ? 3 : 4;
}

// ---------------------------------------------------------------------------
// Dataset
// ---------------------------------------------------------------------------

struct HostCamera {
    std::string path;             // image file (disk datasets; the validation pick matches it)
    float c2w[16];
    int width = 0, height = 0;
    float fx = 0, fy = 0, cx = 0, cy = 0;
    std::vector<uint8_t> image;   // [H,W,3]
    std::vector<uint8_t> mask;    // [H,W] 255 = use, empty = none
    long long unmasked = -1;
    uint8_t *d_image = nullptr, *d_mask = nullptr;
    bool cached = false;
    float viewmat[16], projmat[16], campos[3];

    void prepare() {
        if (cached) return;
        msplat_prepare_camera(c2w, width, height, fx, fy, viewmat, projmat, campos);
        cached = true;
    }
    void upload() {
        if (d_image || image.empty()) return;
        CKA(cudaMalloc(&d_image, image.size()));
        CKA(cudaMemcpy(d_image, image.data(), image.size(), cudaMemcpyHostToDevice));
        if (!mask.empty()) {
            CKA(cudaMalloc(&d_mask, mask.size()));
            CKA(cudaMemcpy(d_mask, mask.data(), mask.size(), cudaMemcpyHostToDevice));
        }
    }
    void release() {
        if (d_image) cudaFree(d_image);
        if (d_mask) cudaFree(d_mask);
        d_image = d_mask = nullptr;
    }
};

struct DatasetImpl {
    std::vector<HostCamera> train, test;
    std::vector<float> xyz;
    std::vector<uint8_t> rgb;
    float scale = 1.0f;
    float translation[3] = {0, 0, 0};
    ~DatasetImpl() {
        for (auto &c : train) c.release();
        for (auto &c : test) c.release();
    }
};

// Centre the cameras on their mean position and scale the largest |coordinate|
// to 1 (autoScaleAndCenter, core/src/input_data.cpp:115-169).
static void auto_scale_and_center(std::vector<HostCamera> &cams, std::vector<float> &xyz, float &scale, float t[3]) {
    if (cams.empty()) return;
    float m[3] = {0.f, 0.f, 0.f};   // float sums, as the reference accumulates
    for (auto &c : cams) { m[0] += c.c2w[3]; m[1] += c.c2w[7]; m[2] += c.c2w[11]; }
    for (int k = 0; k < 3; k++) m[k] /= (float)(int)cams.size();
    float mx = 0;
    for (auto &c : cams) {
        c.c2w[3] -= m[0]; c.c2w[7] -= m[1]; c.c2w[11] -= m[2];
        mx = std::max({mx, std::abs(c.c2w[3]), std::abs(c.c2w[7]), std::abs(c.c2w[11])});
    }
    scale = mx > 0 ? 1.0f / mx : 1.0f;
    for (auto &c : cams) { c.c2w[3] *= scale; c.c2w[7] *= scale; c.c2w[11] *= scale; }
    for (size_t i = 0; i + 2 < xyz.size(); i += 3)
        for (int k = 0; k < 3; k++) xyz[i + k] = (xyz[i + k] - m[k]) * scale;
    for (int k = 0; k < 3; k++) t[k] = m[k];
}

// ---------------------------------------------------------------------------
// Initial scales: mean distance to the 3 nearest other points (the
// reference's PointsTensor::scales, core/include/kdtree_tensor.hpp:26-40),
// found with a uniform grid instead of a k-d tree.
// ---------------------------------------------------------------------------
static std::vector<float> knn3_mean_distance(const std::vector<float> &xyz) {
    const int64_t n = (int64_t)xyz.size() / 3;
    std::vector<float> out(n, 1.0f);
    if (n < 2) return out;
    float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) { lo[k] = std::min(lo[k], xyz[3 * i + k]); hi[k] = std::max(hi[k], xyz[3 * i + k]); }
    double vol = 1;
    for (int k = 0; k < 3; k++) vol *= std::max(1e-6f, hi[k] - lo[k]);
    const float cell = (float)std::max(1e-6, std::cbrt(vol * 4.0 / (double)n));
    int dim[3];
    for (int k = 0; k < 3; k++) dim[k] = std::min(1024, std::max(1, (int)((hi[k] - lo[k]) / cell) + 1));
    auto cidx = [&](float v, int k) { return std::min(dim[k] - 1, std::max(0, (int)((v - lo[k]) / cell))); };
    std::unordered_map<int64_t, std::vector<int>> grid;
    auto key = [&](int x, int y, int z) { return ((int64_t)x * dim[1] + y) * dim[2] + z; };
    for (int64_t i = 0; i < n; i++)
        grid[key(cidx(xyz[3 * i], 0), cidx(xyz[3 * i + 1], 1), cidx(xyz[3 * i + 2], 2))].push_back((int)i);
    for (int64_t i = 0; i < n; i++) {
        const float *p = &xyz[3 * i];
        const int c[3] = {cidx(p[0], 0), cidx(p[1], 1), cidx(p[2], 2)};
        float best[3] = {1e30f, 1e30f, 1e30f};
        for (int r = 1; r < 1024; r++) {
            for (int dx = -r; dx <= r; dx++)
                for (int dy = -r; dy <= r; dy++)
                    for (int dz = -r; dz <= r; dz++) {
                        if (std::max({std::abs(dx), std::abs(dy), std::abs(dz)}) != r && r > 1) continue;
                        const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                        if (x < 0 || y < 0 || z < 0 || x >= dim[0] || y >= dim[1] || z >= dim[2]) continue;
                        auto it = grid.find(key(x, y, z));
                        if (it == grid.end()) continue;
                        for (int j : it->second) {
                            if (j == i) continue;
                            const float d0 = xyz[3 * j] - p[0], d1 = xyz[3 * j + 1] - p[1], d2 = xyz[3 * j + 2] - p[2];
                            const float d = d0 * d0 + d1 * d1 + d2 * d2;
                            if (d < best[2]) {
                                best[2] = d;
                                if (best[2] < best[1]) std::swap(best[1], best[2]);
                                if (best[1] < best[0]) std::swap(best[0], best[1]);
                            }
                        }
                    }
            // every point within r*cell of p has been seen; past the largest
            // grid dimension every cell has been visited
            const float reach = (float)r * cell;
            if (best[2] <= reach * reach || r > std::max({dim[0], dim[1], dim[2]})) break;
        }
        // with fewer than 3 neighbours the missing distances count as 0,
        // as in the reference's k = 4 search over a too-small cloud
        float s = 0;
        for (int k = 0; k < 3; k++)
            if (best[k] < 1e29f) s += std::sqrt(best[k]);
        out[i] = s / 3.0f;
    }
    return out;
}

// ---------------------------------------------------------------------------
// Gaussian state on the device (cap-sized buffers, N active rows)
// ---------------------------------------------------------------------------

struct DeviceModel {
    int cap = 0, n = 0, rest = 15;
    float *p[6] = {nullptr}, *m[6] = {nullptr}, *v[6] = {nullptr};

    int stride(int g) const {
        const int s[6] = {3, 3, 4, 3, 3 * rest, 1};
        return s[g];
    }
    void allocate(int capacity, int rest_bases) {
        free_all();
        cap = capacity;
        rest = rest_bases;
        for (int g = 0; g < 6; g++) {
            const size_t bytes = (size_t)std::max(cap, 1) * stride(g) * sizeof(float) + 16;
            CKA(cudaMalloc(&p[g], bytes));
            CKA(cudaMalloc(&m[g], bytes));
            CKA(cudaMalloc(&v[g], bytes));
            CKA(cudaMemset(p[g], 0, bytes));
            CKA(cudaMemset(m[g], 0, bytes));
            CKA(cudaMemset(v[g], 0, bytes));
        }
    }
    void free_all() {
        for (int g = 0; g < 6; g++) {
            if (p[g]) cudaFree(p[g]);
            if (m[g]) cudaFree(m[g]);
            if (v[g]) cudaFree(v[g]);
            p[g] = m[g] = v[g] = nullptr;
        }
    }
    ~DeviceModel() { free_all(); }

    MsplatGaussians gaussians() const {
        MsplatGaussians g;
        g.num_points = n;
        g.rest_bases = rest;
        g.means = p[0]; g.scales = p[1]; g.quats = p[2]; g.features_dc = p[3]; g.features_rest = p[4];
        g.opacities = p[5];
        return g;
    }
    MsplatAdamState adam() const {
        MsplatAdamState s;
        for (int g = 0; g < 6; g++) { s.exp_avg[g] = m[g]; s.exp_avg_sq[g] = v[g]; }
        return s;
    }
    // host copies of the N active rows
    std::vector<float> read(float *const *arr, int g) const {
        std::vector<float> out((size_t)n * stride(g));
        if (!out.empty()) CKA(cudaMemcpy(out.data(), arr[g], out.size() * 4, cudaMemcpyDeviceToHost));
        return out;
    }
    void write(float **arr, int g, const float *src, int rows) {
        if (rows > 0) CKA(cudaMemcpy(arr[g], src, (size_t)rows * stride(g) * 4, cudaMemcpyHostToDevice));
    }
};

// Checkpoint file (model.cpp:698-843): magic "MSPL", version 1, step, N,
// SH degree, Adam step; 6 learning rates, means lr init/final; 6 parameter
// tensors, then 6 first and 6 second moments, each as (ndim, int64 shape,
// uint64 bytes, float32 data).  Every tensor is checked against the header
// before any of it is used: N rows, the group's row width (features_rest
// [N, rest, 3] with rest = (degree+1)^2 - 1 fixes the width of groups 4, 10
// and 16), and exactly N x width x 4 bytes; anything else is a malformed
// checkpoint (the reader never reads past what it allocated).
struct CheckpointData {
    uint32_t step = 0, n = 0, deg = 0, adam_steps = 0;
    float adam_lr[6] = {0, 0, 0, 0, 0, 0};
    float means_lr_init = 0, means_lr_final = 0;
    int rest = 0;
    std::vector<float> t[18];
};

static CheckpointData read_checkpoint(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open checkpoint " + path);
    auto u32 = [&]() {
        uint32_t v = 0;
        f.read(reinterpret_cast<char *>(&v), 4);
        if (!f) throw std::runtime_error("malformed checkpoint: truncated header");
        return v;
    };
    if (u32() != 0x4C50534Du) throw std::runtime_error("not a msplat checkpoint");
    const uint32_t ver = u32();
    if (ver != 1) throw std::runtime_error("unsupported checkpoint version " + std::to_string(ver));
    CheckpointData ck;
    ck.step = u32();
    ck.n = u32();
    ck.deg = u32();
    ck.adam_steps = u32();
    f.read(reinterpret_cast<char *>(ck.adam_lr), sizeof(ck.adam_lr));
    f.read(reinterpret_cast<char *>(&ck.means_lr_init), 4);
    f.read(reinterpret_cast<char *>(&ck.means_lr_final), 4);
    if (!f) throw std::runtime_error("malformed checkpoint: truncated header");
    if (ck.n > 0x7fffffffu) throw std::runtime_error("malformed checkpoint: N out of range");
    if (ck.deg > 3) throw std::runtime_error("malformed checkpoint: SH degree " + std::to_string(ck.deg) + " > 3");
    ck.rest = (int)((ck.deg + 1) * (ck.deg + 1)) - 1;
    const int width[6] = {3, 3, 4, 3, 3 * ck.rest, 1};
    const char *names[6] = {"means", "scales", "quats", "features_dc", "features_rest", "opacities"};
    for (int k = 0; k < 18; k++) {
        const int g = k % 6;
        const std::string what = std::string("malformed checkpoint: ") + (k < 6 ? "" : k < 12 ? "exp_avg " : "exp_avg_sq ") +
                                 names[g];
        const uint32_t nd = u32();
        if (nd < 1 || nd > 4) throw std::runtime_error(what + ": " + std::to_string(nd) + " dimensions");
        int64_t shape[4] = {0, 0, 0, 0};
        for (uint32_t d = 0; d < nd; d++) {
            f.read(reinterpret_cast<char *>(&shape[d]), 8);
            if (!f) throw std::runtime_error(what + ": truncated shape");
            if (shape[d] < 0) throw std::runtime_error(what + ": negative extent");
        }
        int64_t row = 1;
        for (uint32_t d = 1; d < nd; d++) row *= shape[d];
        if (shape[0] != (int64_t)ck.n) throw std::runtime_error(what + ": " + std::to_string(shape[0]) +
                                                                " rows, header says " + std::to_string(ck.n));
        if (row != width[g] || (g == 4 && nd >= 3 && shape[1] != ck.rest))
            throw std::runtime_error(what + ": row width " + std::to_string(row) + ", expected " +
                                     std::to_string(width[g]));
        uint64_t bytes = 0;
        f.read(reinterpret_cast<char *>(&bytes), 8);
        if (!f) throw std::runtime_error(what + ": truncated size");
        const uint64_t want = (uint64_t)ck.n * (uint64_t)width[g] * 4u;
        if (bytes != want) throw std::runtime_error(what + ": " + std::to_string(bytes) + " bytes, expected " +
                                                    std::to_string(want));
        ck.t[k].resize((size_t)want / 4);
        f.read(reinterpret_cast<char *>(ck.t[k].data()), (std::streamsize)want);
        if (!f) throw std::runtime_error(what + ": truncated data");
    }
    return ck;
}

// Writes a checkpoint in the same format: the header, then the 18 tensors
// with the reference's shapes (means, scales [N,3], quats [N,4],
// features_dc [N,3], features_rest [N,rest,3], opacities [N,1]; each
// moment as its parameter).  ck.t[k] holds N rows of its group's width.
static void write_checkpoint(const std::string &path, const CheckpointData &ck) {
    const int rest = (int)((ck.deg + 1) * (ck.deg + 1)) - 1;
    const int width[6] = {3, 3, 4, 3, 3 * rest, 1};
    for (int k = 0; k < 18; k++)
        if (ck.t[k].size() != (size_t)ck.n * width[k % 6])
            throw std::runtime_error("checkpoint tensor " + std::to_string(k) + " has the wrong size");
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write checkpoint " + path);
    auto u32 = [&](uint32_t v) { f.write(reinterpret_cast<const char *>(&v), 4); };
    u32(0x4C50534Du);
    u32(1);
    u32(ck.step);
    u32(ck.n);
    u32(ck.deg);
    u32(ck.adam_steps);
    f.write(reinterpret_cast<const char *>(ck.adam_lr), sizeof(ck.adam_lr));
    f.write(reinterpret_cast<const char *>(&ck.means_lr_init), 4);
    f.write(reinterpret_cast<const char *>(&ck.means_lr_final), 4);
    for (int k = 0; k < 18; k++) {
        const int g = k % 6;
        const int64_t n = ck.n;
        std::vector<int64_t> shape;
        if (g == 4) shape = {n, rest, 3};
        else if (g == 5) shape = {n, 1};
        else shape = {n, g == 2 ? 4 : 3};
        u32((uint32_t)shape.size());
        for (int64_t e : shape) f.write(reinterpret_cast<const char *>(&e), 8);
        const uint64_t bytes = ck.t[k].size() * 4;
        f.write(reinterpret_cast<const char *>(&bytes), 8);
        f.write(reinterpret_cast<const char *>(ck.t[k].data()), (std::streamsize)bytes);
    }
    if (!f) throw std::runtime_error("cannot write checkpoint " + path);
}

// Reference-layout host copy of a model (means [N,3] ... opacities [N]).
struct HostGaussians {
    int n = 0, rest = 15;
    std::vector<float> a[6];
};

// PLY export (saveGaussianPly, core/src/loaders/save_gaussians.cpp:10-88):
// non-finite Gaussians dropped, f_rest written channel-major.
static void write_ply(const std::string &path, const HostGaussians &h, int step, bool keep_crs, float scale,
                      const float *t) {
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + path);
    const int rest = h.rest, nfr = 3 * rest;
    std::vector<int> keep;
    for (int i = 0; i < h.n; i++) {
        bool ok = std::isfinite(h.a[5][i]);
        for (int k = 0; ok && k < 3; k++) ok = std::isfinite(h.a[0][3 * i + k]) && std::isfinite(h.a[1][3 * i + k]);
        for (int k = 0; ok && k < 4; k++) ok = std::isfinite(h.a[2][4 * i + k]);
        for (int k = 0; ok && k < 3; k++) ok = std::isfinite(h.a[3][3 * i + k]);
        for (int k = 0; ok && k < nfr; k++) ok = std::isfinite(h.a[4][(size_t)nfr * i + k]);
        if (ok) keep.push_back(i);
    }
    if ((int)keep.size() < h.n) fprintf(stderr, "export ply: dropped %d non-finite Gaussian(s)\n", h.n - (int)keep.size());
    o << "ply\nformat binary_little_endian 1.0\n";
    o << "comment Generated by msplat at iteration " << step << "\n";
    o << "element vertex " << keep.size() << "\n";
    o << "property float x\nproperty float y\nproperty float z\n";
    o << "property float nx\nproperty float ny\nproperty float nz\n";
    for (int i = 0; i < 3; i++) o << "property float f_dc_" << i << "\n";
    for (int i = 0; i < nfr; i++) o << "property float f_rest_" << i << "\n";
    o << "property float opacity\n";
    o << "property float scale_0\nproperty float scale_1\nproperty float scale_2\n";
    o << "property float rot_0\nproperty float rot_1\nproperty float rot_2\nproperty float rot_3\n";
    o << "end_header\n";
    std::vector<float> row(3 + 3 + 3 + nfr + 1 + 3 + 4);
    for (int i : keep) {
        int c = 0;
        for (int k = 0; k < 3; k++) row[c++] = keep_crs ? h.a[0][3 * i + k] / scale + t[k] : h.a[0][3 * i + k];
        row[c++] = 0; row[c++] = 0; row[c++] = 0;
        for (int k = 0; k < 3; k++) row[c++] = h.a[3][3 * i + k];
        for (int ch = 0; ch < 3; ch++)
            for (int b = 0; b < rest; b++) row[c++] = h.a[4][(size_t)nfr * i + 3 * b + ch];
        row[c++] = h.a[5][i];
        for (int k = 0; k < 3; k++)
            row[c++] = keep_crs ? std::log(std::exp(h.a[1][3 * i + k]) / scale) : h.a[1][3 * i + k];
        for (int k = 0; k < 4; k++) row[c++] = h.a[2][4 * i + k];
        o.write(reinterpret_cast<const char *>(row.data()), row.size() * sizeof(float));
    }
}

// PLY import (loadGaussianPly, save_gaussians.cpp:141-231).
static HostGaussians read_ply(const std::string &path, int *step_out, bool keep_crs, float scale, const float *t) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open PLY " + path);
    std::string line;
    std::getline(f, line);
    if (line.find("ply") == std::string::npos) throw std::runtime_error("not a PLY file: " + path);
    int n = 0, ndc = 0, nfr = 0, step = 0;
    while (std::getline(f, line)) {
        if (line == "end_header") break;
        const std::string it = "comment Generated by msplat at iteration ", legacy = "comment msplat v",
                          vx = "element vertex ";
        if (line.rfind(it, 0) == 0) step = std::stoi(line.substr(it.size()));
        if (line.rfind(legacy, 0) == 0) step = std::stoi(line.substr(legacy.size()));
        if (line.rfind(vx, 0) == 0) n = std::stoi(line.substr(vx.size()));
        if (line.rfind("property float f_dc_", 0) == 0) ndc++;
        if (line.rfind("property float f_rest_", 0) == 0) nfr++;
    }
    if (n <= 0) throw std::runtime_error("PLY has no vertices");
    if (ndc != 3) throw std::runtime_error("PLY must have 3 f_dc properties");
    HostGaussians h;
    h.n = n;
    h.rest = nfr / 3;
    const size_t strides[6] = {3, 3, 4, 3, (size_t)nfr, 1};
    for (int g = 0; g < 6; g++) h.a[g].assign((size_t)n * strides[g], 0.f);
    std::vector<float> row(3 + 3 + ndc + nfr + 1 + 3 + 4);
    for (int i = 0; i < n; i++) {
        f.read(reinterpret_cast<char *>(row.data()), row.size() * 4);
        if (!f) throw std::runtime_error("truncated PLY " + path);
        int c = 0;
        for (int k = 0; k < 3; k++) h.a[0][3 * i + k] = row[c++];
        c += 3;
        for (int k = 0; k < 3; k++) h.a[3][3 * i + k] = row[c++];
        for (int ch = 0; ch < 3; ch++)
            for (int b = 0; b < h.rest; b++) h.a[4][(size_t)nfr * i + 3 * b + ch] = row[c++];
        h.a[5][i] = row[c++];
        for (int k = 0; k < 3; k++) h.a[1][3 * i + k] = row[c++];
        for (int k = 0; k < 4; k++) h.a[2][4 * i + k] = row[c++];
    }
    if (keep_crs) {
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) h.a[0][3 * i + k] = (h.a[0][3 * i + k] - t[k]) * scale;
        for (auto &s : h.a[1]) s = std::log(scale * std::exp(s));
    }
    if (step_out) *step_out = step;
    return h;
}

// .splat export (saveGaussianSplat, save_gaussians.cpp:90-139): 32 B per
// Gaussian, largest (sum of scales * opacity) first.
static void write_splat(const std::string &path, const HostGaussians &h, bool keep_crs, float scale, const float *t) {
    std::ofstream o(path, std::ios::binary);
    if (!o) throw std::runtime_error("cannot write " + path);
    std::vector<float> order(h.n, 0.f);
    std::vector<size_t> idx;
    for (int i = 0; i < h.n; i++) {
        bool ok = std::isfinite(h.a[5][i]);
        for (int k = 0; ok && k < 3; k++) ok = std::isfinite(h.a[0][3 * i + k]) && std::isfinite(h.a[1][3 * i + k]);
        for (int k = 0; ok && k < 4; k++) ok = std::isfinite(h.a[2][4 * i + k]);
        if (!ok) continue;
        float s = std::exp(h.a[1][3 * i]) + std::exp(h.a[1][3 * i + 1]) + std::exp(h.a[1][3 * i + 2]);
        if (keep_crs) s /= scale;
        order[i] = s / (1.0f + std::exp(-h.a[5][i]));
        idx.push_back(i);
    }
    std::sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return order[a] > order[b]; });
    for (size_t i : idx) {
        float m[3], sc[3];
        for (int k = 0; k < 3; k++) m[k] = keep_crs ? h.a[0][3 * i + k] / scale + t[k] : h.a[0][3 * i + k];
        for (int k = 0; k < 3; k++) sc[k] = keep_crs ? std::exp(h.a[1][3 * i + k]) / scale : std::exp(h.a[1][3 * i + k]);
        uint8_t rgb[3], a, q[4];
        for (int k = 0; k < 3; k++)
            rgb[k] = (uint8_t)std::clamp(((double)h.a[3][3 * i + k] * kShC0 + 0.5) * 255.0, 0.0, 255.0);
        const float sig = 1.0f / (1.0f + std::exp(-h.a[5][i]));
        a = (uint8_t)std::clamp(sig * 255.0f, 0.0f, 255.0f);
        for (int k = 0; k < 4; k++) q[k] = (uint8_t)std::clamp(h.a[2][4 * i + k] * 128.0f + 128.0f, 0.0f, 255.0f);
        o.write(reinterpret_cast<const char *>(m), 12);
        o.write(reinterpret_cast<const char *>(sc), 12);
        o.write(reinterpret_cast<const char *>(rgb), 3);
        o.write(reinterpret_cast<const char *>(&a), 1);
        o.write(reinterpret_cast<const char *>(q), 4);
    }
}

// ---------------------------------------------------------------------------
// Trainer (Model + Trainer)
// ---------------------------------------------------------------------------

static const float kLrInit[6] = {0.00016f, 0.005f, 0.001f, 0.0025f, 0.000125f, 0.05f};   // model.cpp:223

static MsplatTrainerOptions default_trainer_options() { return MsplatTrainerOptions{0.5f, 0.1f, 1, 30000, 1.0f}; }
static bool trainer_options_valid(const MsplatTrainerOptions &o) {
    return o.initOpacity > 0.f && o.initOpacity < 1.f && o.initScaleMult > 0.f && o.positionLrMaxSteps > 0 &&
           o.regVisibilityDuty >= 0.f;
}

// Model::Model (model.cpp:80-166): KNN scale x initScaleMult, random unit
// quaternions from mt19937(42), DC from the point colours, rest 0, opacity
// logit(initOpacity).
static HostGaussians seed_gaussians(const std::vector<float> &xyz, const std::vector<uint8_t> &rgb, int sh_degree,
                                    const MsplatTrainerOptions &o) {
    const int64_t n = (int64_t)xyz.size() / 3;
    const int rest = sh_bases_for_degree(sh_degree) - 1;
    HostGaussians h;
    h.n = (int)n;
    h.rest = rest;
    h.a[0] = xyz;
    auto sc = knn3_mean_distance(xyz);
    h.a[1].resize(3 * n);
    for (int64_t i = 0; i < n; i++) h.a[1][3 * i] = h.a[1][3 * i + 1] = h.a[1][3 * i + 2] = std::log(sc[i] * o.initScaleMult);
    std::mt19937 qr(42);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    h.a[2].resize(4 * n);
    for (int64_t i = 0; i < n; i++) {
        const float u = u01(qr), v = u01(qr), w = u01(qr);
        // float radius times a double-precision angle term, rounded once
        h.a[2][4 * i + 0] = (float)(std::sqrt(1 - u) * std::sin(2 * M_PI * v));
        h.a[2][4 * i + 1] = (float)(std::sqrt(1 - u) * std::cos(2 * M_PI * v));
        h.a[2][4 * i + 2] = (float)(std::sqrt(u) * std::sin(2 * M_PI * w));
        h.a[2][4 * i + 3] = (float)(std::sqrt(u) * std::cos(2 * M_PI * w));
    }
    h.a[3].resize(3 * n);
    for (int64_t i = 0; i < 3 * n; i++) h.a[3][i] = (float)((rgb[i] / 255.0 - 0.5) / kShC0);
    h.a[4].assign((size_t)3 * rest * n, 0.f);
    h.a[5].assign(n, std::log(o.initOpacity / (1.0f - o.initOpacity)));
    return h;
}

// setupOptimizers (model.cpp:168-200): the rows kept of n at a cap of cap:
// above 75 % of the cap (with decimation) a sorted random half of the cap
// (mt19937(42) shuffle), else the first min(n, cap).  Returns the count;
// keep is empty when the rows are the first ones.
static int seed_rows(int n, int cap, bool decimate, std::vector<int> &keep) {
    keep.clear();
    if (decimate && n > (int)(cap * 0.75)) {
        const int rows = (int)(cap * 0.5);
        keep.resize(n);
        std::iota(keep.begin(), keep.end(), 0);
        std::mt19937 r(42);
        std::shuffle(keep.begin(), keep.end(), r);
        keep.resize(rows);
        std::sort(keep.begin(), keep.end());
        return rows;
    }
    return std::min(n, cap);
}

struct TrainerImpl {
    MsplatConfig cfg;
    MsplatTrainerOptions opt = default_trainer_options();
    DatasetImpl *ds = nullptr;
    MsplatEngine *eng = nullptr;
    DeviceModel model;
    int current_step = 0, adam_step_count = 0, reloc_count = 0;
    float adam_lr[6];
    float means_lr_init = 0.00016f, means_lr_final = 0.0000016f;
    int position_lr_max_steps = 30000;
    std::vector<size_t> cam_order;
    size_t cam_pos = 0;
    std::mt19937 rng{42};
    float last_loss = 0.f;
    int batch_views = 1;          // views per optimizer step (1 = the reference's one-camera step)
    float batch_lr_scale = 1.0f;  // learning-rate factor of multi-view steps
    MsplatMcmcStats last_mcmc{};  // the last relocation round's counts
    int mcmc_rounds = 0;
    // MSPLAT_NAN_INJECT=<step>, read when the trainer is created (host-side
    // fault injection of model.cpp:638-659; -1: off)
    int nan_inject = -1;

    // a period boundary crossed between iterations prev (exclusive) and cur (inclusive)
    static bool crossed(int prev, int cur, int period) { return cur / period > prev / period; }

    // learned relocation proposal (off unless enabled): activity statistics
    // accumulated by the step, an MLP trained online every `window` steps on
    // (state -> opacity and activity `window` steps later) pairs the run
    // itself produces, whose predictions weight the MCMC source draws once it
    // has been trained; plain opacity weights before that and when disabled
    struct Learned {
        bool enabled = false;
        int window = 500, samples = 16384, epochs = 40;
        float lr = 1e-3f;
        float *P = nullptr, *G = nullptr, *M = nullptr, *V = nullptr, *loss = nullptr, *score = nullptr;
        float *eval = nullptr;          // device sums of the held-out check (mlp_eval)
        double eval_sum[4] = {0, 0, 0, 0};
        int eval_rounds = 0;
        uint8_t *img = nullptr;
        unsigned *err = nullptr, *pruned = nullptr;
        float4 *gstats = nullptr, *snap = nullptr;
        __nv_bfloat16 *X = nullptr, *Xs = nullptr;
        float2 *Y = nullptr, *T = nullptr;
        int *idx = nullptr;
        int pending = -1, rounds = 0, adam_steps = 0, cap = 0;
        float last_loss = NAN;
        float prune = 0.02f;            // forecast-opacity threshold of forecast pruning (0: off)
        std::mt19937 rng{7};
    } lrn;

    TrainerImpl(DatasetImpl *d, const MsplatConfig &c, const MsplatTrainerOptions &o) : cfg(c), opt(o), ds(d) {
        position_lr_max_steps = opt.positionLrMaxSteps;
        if (const char *e = std::getenv("MSPLAT_NAN_INJECT")) nan_inject = std::atoi(e);
        int dev = 0;
        CKA(cudaGetDevice(&dev));
        eng = msplat_engine_create(dev, std::max(1, cfg.capMax));
        if (!eng) throw std::runtime_error("engine creation failed");
        msplat_engine_set_graphs(eng, 1);   // a camera's repeated steps replay one graph
        init_from_points();
        cam_order.resize(ds->train.size());
        std::iota(cam_order.begin(), cam_order.end(), 0);
        shuffle_cameras();
    }
    ~TrainerImpl() {
        free_learned();
        if (eng) msplat_engine_destroy(eng);
    }

    void free_learned() {
        void *ptrs[] = {lrn.P, lrn.G, lrn.M, lrn.V, lrn.loss, lrn.score, lrn.img, lrn.err, lrn.gstats, lrn.snap,
                        lrn.X, lrn.Xs, lrn.Y, lrn.T, lrn.idx, lrn.eval, lrn.pruned};
        for (void *q : ptrs)
            if (q) cudaFree(q);
        lrn = Learned{};
    }

    void enable_learned(bool on) {
        if (!on) {
            if (eng) msplat_engine_set_activity_stats(eng, nullptr);
            free_learned();
            return;
        }
        if (lrn.enabled) return;
        const int cap = std::max(1, model.cap);
        lrn.cap = cap;
        CKA(cudaMalloc(&lrn.P, kMlpParams * 4));
        CKA(cudaMalloc(&lrn.G, kMlpParams * 4));
        CKA(cudaMalloc(&lrn.M, kMlpParams * 4));
        CKA(cudaMalloc(&lrn.V, kMlpParams * 4));
        CKA(cudaMalloc(&lrn.loss, 4));
        CKA(cudaMalloc(&lrn.err, 4));
        CKA(cudaMalloc(&lrn.pruned, 4));
        CKA(cudaMalloc(&lrn.eval, 5 * 4));
        CKA(cudaMalloc(&lrn.img, kImgBytes));
        CKA(cudaMalloc(&lrn.gstats, sizeof(float4) * (size_t)cap));
        CKA(cudaMalloc(&lrn.score, 4 * (size_t)cap));
        CKA(cudaMalloc(&lrn.X, 64 * (size_t)cap));
        CKA(cudaMalloc(&lrn.Y, 8 * (size_t)cap));
        CKA(cudaMalloc(&lrn.Xs, 64 * (size_t)lrn.samples));
        CKA(cudaMalloc(&lrn.T, 8 * (size_t)lrn.samples));
        CKA(cudaMalloc(&lrn.snap, sizeof(float4) * (size_t)lrn.samples));
        CKA(cudaMalloc(&lrn.idx, 4 * (size_t)lrn.samples));
        CKA(cudaMemset(lrn.gstats, 0, sizeof(float4) * (size_t)cap));
        CKA(cudaMemset(lrn.G, 0, kMlpParams * 4));
        CKA(cudaMemset(lrn.M, 0, kMlpParams * 4));
        CKA(cudaMemset(lrn.V, 0, kMlpParams * 4));
        CKA(cudaMemset(lrn.err, 0, 4));
        // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases
        std::vector<float> P(kMlpParams, 0.f);
        std::mt19937 r(1234);
        std::uniform_real_distribution<float> u(-1.f, 1.f);
        for (int i = 0; i < kMlpIn; i++)
            for (int o = 0; o < 64; o++) P[kMlpW1 + i * 64 + o] = u(r) / std::sqrt((float)kMlpIn);
        for (int i = 0; i < 64 * 64; i++) P[kMlpW2 + i] = u(r) / 8.f;
        for (int i = 0; i < 64; i++)
            for (int o = 0; o < 2; o++) P[kMlpW3 + i * 16 + o] = u(r) / 8.f;
        CKA(cudaMemcpy(lrn.P, P.data(), kMlpParams * 4, cudaMemcpyHostToDevice));
        lrn.enabled = true;
        msplat_engine_set_activity_stats(eng, lrn.gstats);
    }

    cudaStream_t stream() const { return static_cast<cudaStream_t>(msplat_engine_stream(eng)); }

    MlpFeatArgs feat_args(int rows, const int *idx, __nv_bfloat16 *X) {
        MlpFeatArgs fa{};
        fa.rows = rows;
        fa.idx = idx;
        fa.means = model.p[0]; fa.scales = model.p[1]; fa.quats = model.p[2];
        fa.features_dc = model.p[3]; fa.opacities = model.p[5];
        fa.gstats = lrn.gstats;
        void *radii = nullptr;
        const long long rb = msplat_engine_buffer(eng, "radii", &radii);
        fa.radii = (rb >= 4LL * model.n) ? static_cast<const int *>(radii) : nullptr;
        fa.X = X;
        return fa;
    }

    // every `window` steps: label the previous snapshot and train, then take a new one
    void learned_after_step(int prev, int step) {
        if (!lrn.enabled || step < lrn.window || !crossed(prev, step, lrn.window) || model.n <= 0) return;
        cudaStream_t s = stream();
        if (lrn.pending >= 0) {
            mlp_targets(lrn.idx, lrn.snap, lrn.samples, model.p[5], lrn.gstats, lrn.T, s);
            // held out: once trained, the MLP predicts this window's labels before it sees them
            float ev[5] = {0, 0, 0, 0, 0};
            const bool evaluate = lrn.rounds >= 1;
            if (evaluate) {
                mlp_pack(lrn.P, lrn.img, s);
                mlp_forward(lrn.Xs, lrn.samples, lrn.img, lrn.P, lrn.Y, lrn.err, s);
                CKA(cudaMemsetAsync(lrn.eval, 0, 5 * 4, s));
                mlp_eval(lrn.Y, lrn.T, lrn.snap, lrn.samples, lrn.eval, s);
                CKA(cudaMemcpyAsync(ev, lrn.eval, 5 * 4, cudaMemcpyDeviceToHost, s));
            }
            for (int e = 0; e < lrn.epochs; e++) {
                mlp_pack(lrn.P, lrn.img, s);
                CKA(cudaMemsetAsync(lrn.loss, 0, 4, s));
                mlp_train_batch(lrn.Xs, lrn.T, lrn.samples, lrn.img, lrn.P, lrn.G, lrn.loss, lrn.err, s);
                mlp_adam(lrn.P, lrn.G, lrn.M, lrn.V, lrn.lr, ++lrn.adam_steps, s);
            }
            CKA(cudaGetLastError());   // the launches above
            CKA(cudaMemcpyAsync(&lrn.last_loss, lrn.loss, 4, cudaMemcpyDeviceToHost, s));
            unsigned err = 0;
            CKA(cudaMemcpyAsync(&err, lrn.err, 4, cudaMemcpyDeviceToHost, s));
            CKA(cudaStreamSynchronize(s));
            if (err) throw std::runtime_error("learned relocation: tensor-core MMA did not complete");
            if (evaluate && ev[4] > 0.f) {
                for (int k = 0; k < 4; k++) lrn.eval_sum[k] += ev[k] / ev[4];
                lrn.eval_rounds++;
            }
            lrn.rounds++;
        }
        std::vector<int> idx(lrn.samples);
        std::uniform_int_distribution<int> pick(0, model.n - 1);
        for (auto &v : idx) v = pick(lrn.rng);
        CKA(cudaMemcpyAsync(lrn.idx, idx.data(), 4 * idx.size(), cudaMemcpyHostToDevice, s));
        mlp_features(feat_args(lrn.samples, lrn.idx, lrn.Xs), s);
        mlp_snapshot(lrn.idx, lrn.samples, lrn.gstats, model.p[5], lrn.snap, s);
        CKA(cudaGetLastError());
        CKA(cudaStreamSynchronize(s));   // idx is a host vector
        lrn.pending = step;
    }

    // MCMC source weights from the trained MLP, or null for the plain rule
    const float *learned_scores() {
        if (!lrn.enabled || lrn.rounds == 0 || model.n <= 0) return nullptr;
        cudaStream_t s = stream();
        mlp_pack(lrn.P, lrn.img, s);
        mlp_features(feat_args(model.n, nullptr, lrn.X), s);
        mlp_forward(lrn.X, model.n, lrn.img, lrn.P, lrn.Y, lrn.err, s);
        mlp_scores(lrn.Y, model.n, lrn.score, s);
        CKA(cudaGetLastError());
        return lrn.score;
    }

    void shuffle_cameras() {
        std::shuffle(cam_order.begin(), cam_order.end(), rng);
        cam_pos = 0;
    }
    size_t next_camera() {
        if (cam_pos >= cam_order.size()) shuffle_cameras();
        return cam_order[cam_pos++];
    }

    // Model::Model (model.cpp:81-166): KNN scale x 0.1, random unit
    // quaternions from mt19937(42), DC from the point colours, rest 0,
    // opacity 0.5; then setupOptimizers (model.cpp:168-254).
    void init_from_points() {
        HostGaussians h = seed_gaussians(ds->xyz, ds->rgb, cfg.shDegree, opt);
        set_model(h, opt.seedDecimation != 0);
    }

    // setupOptimizers: cap-sized buffers, seed decimation above 75 % of cap
    void set_model(HostGaussians &h, bool decimate) {
        const int cap = std::max(1, cfg.capMax);
        std::vector<int> keep;
        const int rows = seed_rows(h.n, cap, decimate, keep);
        model.allocate(cap, h.rest);
        model.n = rows;
        for (int g = 0; g < 6; g++) {
            const int s = model.stride(g);
            if (keep.empty()) {
                model.write(model.p, g, h.a[g].data(), rows);
            } else {
                std::vector<float> sel((size_t)rows * s);
                for (int i = 0; i < rows; i++) std::memcpy(&sel[(size_t)i * s], &h.a[g][(size_t)keep[i] * s], s * 4);
                model.write(model.p, g, sel.data(), rows);
            }
            adam_lr[g] = kLrInit[g];
        }
        adam_step_count = 0;
        means_lr_init = 0.00016f;
        means_lr_final = 0.0000016f;
    }

    void step_args(HostCamera &cam, int step, MsplatStepArgs &a, bool training) {
        cam.prepare();
        std::memset(&a, 0, sizeof(a));
        std::memcpy(a.viewmat, cam.viewmat, sizeof(a.viewmat));
        std::memcpy(a.projmat, cam.projmat, sizeof(a.projmat));
        a.fx = cam.fx; a.fy = cam.fy; a.cx = cam.cx; a.cy = cam.cy;
        a.width = cam.width; a.height = cam.height;
        std::memcpy(a.cam_pos, cam.campos, sizeof(a.cam_pos));
        std::memcpy(a.background, cfg.bgColor, sizeof(a.background));
        a.clip_thresh = 0.01f;
        a.degrees_to_use = std::min(step / std::max(1, cfg.shDegreeInterval), cfg.shDegree);
        a.degrees_to_use = std::min(a.degrees_to_use, degree_for_rest(model.rest));
        a.ssim_weight = cfg.ssimWeight;
        a.beta1 = 0.9f; a.beta2 = 0.999f; a.eps = 1e-8f;
        a.invis_scale = opt.regVisibilityDuty;
        if (!training) return;
        // float beta raised to an int power: evaluated in double, rounded once
        const float bc1 = (float)(1.0 - std::pow((double)0.9f, (double)adam_step_count));
        const float bc2 = (float)(1.0 - std::pow((double)0.999f, (double)adam_step_count));
        for (int g = 0; g < 6; g++) { a.step_size[g] = adam_lr[g] / bc1; a.bc2_sqrt[g] = std::sqrt(bc2); }
        const bool masked = !cam.mask.empty() && cam.unmasked > 0;
        a.loss_inv_n = masked ? 1.0f / (float)(cam.unmasked * 3) : 1.0f / (float)((long long)cam.width * cam.height * 3);
        a.op_reg = step >= 500 ? cfg.opacityReg : 0.f;
        a.sc_reg = step >= 500 ? cfg.scaleReg : 0.f;
        a.do_optimizer = 1;
        a.do_sgld = 1;
        a.seed = (uint32_t)step;
        a.noise_lr = cfg.noiseLr;
        a.xyz_lr = adam_lr[0];
        a.max_disp = cfg.cullRadius > 0.f ? cfg.cullRadius * 0.0167f : 0.05f;
    }

    void check(int rc, const char *what) {
        if (rc != 0) throw std::runtime_error(std::string(what) + ": " + msplat_engine_last_error(eng));
    }

    // Trainer::step (msplat_api.mm:104-127) + Model::fullIteration.  With
    // batch_views B > 1 one step renders the next B cameras and applies one
    // update from their mean gradient; the iteration counter advances by B
    // (it counts views), and every schedule keyed on it (learning-rate decay,
    // SH degree, regularizer start, MCMC every 100, the learned proposal's
    // window) fires when its boundary is crossed.
    MsplatStats step() {
        const auto t0 = std::chrono::high_resolution_clock::now();
        if (ds->train.empty()) throw std::runtime_error("dataset has no training cameras");
        const int B = std::max(1, batch_views);
        const int prev = current_step;
        current_step += B;
        adam_step_count++;
        MsplatGaussians g = model.gaussians();
        MsplatAdamState st = model.adam();
        if (B == 1) {
            HostCamera &cam = ds->train[next_camera()];
            cam.upload();
            MsplatStepArgs a;
            step_args(cam, current_step, a, true);
            check(msplat_engine_train_step(eng, &g, &st, &a, cam.d_image, cam.d_mask), "train step");
        } else {
            std::vector<MsplatStepArgs> a(B);
            std::vector<const uint8_t *> gt(B), mk(B);
            for (int v = 0; v < B; v++) {
                HostCamera &cam = ds->train[next_camera()];
                cam.upload();
                step_args(cam, current_step, a[v], true);
                for (int k = 0; k < 6; k++) a[v].step_size[k] *= batch_lr_scale;
                gt[v] = cam.d_image;
                mk[v] = cam.d_mask;
            }
            check(msplat_engine_train_step_batch(eng, &g, &st, a.data(), B, gt.data(), mk.data()), "batch step");
        }
        learned_after_step(prev, current_step);
        // schedulersStep (model.cpp:256-261)
        const float t = std::clamp((float)current_step / (float)position_lr_max_steps, 0.f, 1.f);
        adam_lr[0] = std::exp(std::log(means_lr_init) * (1.f - t) + std::log(means_lr_final) * t);
        mcmc_after_train(prev, current_step);
        const auto t1 = std::chrono::high_resolution_clock::now();
        MsplatStats s;
        s.iteration = current_step;
        s.splatCount = model.n;
        s.msPerStep = std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count() / 1000.0f;
        return s;
    }

    // Model::mcmcAfterTrain (model.cpp:497-660), on the GPU
    void mcmc_after_train(int prev, int step) {
        if (step < 500 || !crossed(prev, step, 100)) return;
        if (step >= (int)(cfg.iterations * 0.833f)) return;
        MsplatGaussians g = model.gaussians();
        MsplatAdamState st = model.adam();
        MsplatMcmcStats ms;
        const float *score = learned_scores();
        if (score && lrn.prune > 0.f) CKA(mlp_forecast_prune(lrn.Y, model.n, model.p[5], lrn.prune, lrn.pruned, stream()));
        check(msplat_engine_mcmc_scored(eng, &g, &st, model.cap, cfg.cullRadius, &reloc_count, score, &ms), "mcmc");
        model.n = ms.num_active;
        if (crossed(prev, step, 1000))
            fprintf(stderr, "MCMC step=%d active=%d dead=%d culled=%d nonfinite=%d grown=%d\n", step, ms.num_active,
                   ms.num_dead, ms.num_culled, ms.num_nonfinite, ms.num_grown);
        if (ms.num_nonfinite > 0) fprintf(stderr, "MCMC nonfinite step=%d count=%d\n", step, ms.num_nonfinite);
        last_mcmc = ms;
        mcmc_rounds++;
        // MSPLAT_NAN_INJECT=<step>: poison features_dc of 100 Gaussians (host-side fault injection,
        // model.cpp:638-659)
        if (nan_inject > prev && nan_inject <= step && model.n > 0) {
            std::mt19937 r(1234);
            std::uniform_int_distribution<int> pick(0, model.n - 1);
            const float nan3[3] = {NAN, NAN, NAN};
            for (int k = 0; k < 100; k++)
                CKA(cudaMemcpy(model.p[3] + 3 * (size_t)pick(r), nan3, 12, cudaMemcpyHostToDevice));
            fprintf(stderr, "MCMC nan-inject step=%d poisoned=100 (featuresDc)\n", step);
        }
    }

    // forward only; returns host float [H,W,3]
    std::vector<float> render_cam(HostCamera &cam, int step) {
        MsplatStepArgs a;
        step_args(cam, step, a, false);
        MsplatGaussians g = model.gaussians();
        check(msplat_engine_render(eng, &g, &a), "render");
        std::vector<float> img((size_t)cam.width * cam.height * 3);
        check(msplat_engine_read(eng, "out_img", img.data(), (long long)img.size() * 4), "read image");
        return img;
    }

    MsplatEvalMetrics evaluate() {
        MsplatEvalMetrics m{};
        if (ds->test.empty()) return m;
        double sp = 0, ss = 0, sl = 0;
        for (auto &cam : ds->test) {
            auto img = render_cam(cam, cfg.iterations);
            std::vector<float> gt(cam.image.size());
            for (size_t i = 0; i < gt.size(); i++) gt[i] = (float)cam.image[i] * (1.0f / 255.0f);
            sp += msplat_psnr(img.data(), gt.data(), (long long)img.size());
            ss += msplat_ssim_eval(img.data(), gt.data(), cam.height, cam.width);
            sl += msplat_l1(img.data(), gt.data(), (long long)img.size());
        }
        const int n = (int)ds->test.size();
        m.psnr = (float)(sp / n); m.ssim = (float)(ss / n); m.l1 = (float)(sl / n);
        m.numTest = n;
        m.numGaussians = model.n;
        return m;
    }

    HostGaussians host_model() {
        HostGaussians h;
        h.n = model.n;
        h.rest = model.rest;
        CKA(cudaDeviceSynchronize());
        for (int g = 0; g < 6; g++) h.a[g] = model.read(model.p, g);
        return h;
    }

    // checkpoint (model.cpp:698-843): magic "MSPL", version 1, step, N, degree,
    // Adam step; 6 learning rates, means lr init/final; 6 parameter tensors,
    // then 6 first and 6 second moments as (ndim, shape, bytes, data)
    void save_checkpoint(const std::string &path) {
        CKA(cudaDeviceSynchronize());
        // the degree recorded is the one the stored rest bases belong to
        int deg = 0;
        while (deg < 3 && (deg + 1) * (deg + 1) - 1 < model.rest) deg++;
        if ((deg + 1) * (deg + 1) - 1 != model.rest)
            throw std::runtime_error("cannot save a checkpoint of " + std::to_string(model.rest) +
                                     " rest SH bases (not those of degree 0-3)");
        CheckpointData ck;
        ck.step = (uint32_t)current_step;
        ck.n = (uint32_t)model.n;
        ck.deg = (uint32_t)deg;
        ck.adam_steps = (uint32_t)adam_step_count;
        std::memcpy(ck.adam_lr, adam_lr, sizeof(ck.adam_lr));
        ck.means_lr_init = means_lr_init;
        ck.means_lr_final = means_lr_final;
        ck.rest = model.rest;
        for (int g = 0; g < 6; g++) {
            ck.t[g] = model.read(model.p, g);
            ck.t[6 + g] = model.read(model.m, g);
            ck.t[12 + g] = model.read(model.v, g);
        }
        write_checkpoint(path, ck);
    }

    // Model::loadPly (model.cpp:683-694): trained Gaussians, fresh optimizer
    int load_ply(const std::string &path) {
        int step = 0;
        HostGaussians h = read_ply(path, &step, cfg.keepCrs, ds->scale, ds->translation);
        set_model(h, false);
        current_step = step;
        shuffle_cameras();
        return step;
    }

    int load_checkpoint(const std::string &path) {
        CheckpointData ck = read_checkpoint(path);
        const uint32_t n = ck.n;
        std::memcpy(adam_lr, ck.adam_lr, sizeof(adam_lr));
        means_lr_init = ck.means_lr_init;
        means_lr_final = ck.means_lr_final;
        const uint32_t step = ck.step, adam_steps = ck.adam_steps;
        const int rest = ck.rest;
        std::vector<float> *t = ck.t;
        const int cap = std::max((int)n, std::max(1, cfg.capMax));
        model.allocate(cap, rest);
        model.n = (int)n;
        for (int g = 0; g < 6; g++) {
            model.write(model.p, g, t[g].data(), (int)n);
            model.write(model.m, g, t[6 + g].data(), (int)n);
            model.write(model.v, g, t[12 + g].data(), (int)n);
        }
        adam_step_count = (int)adam_steps;
        current_step = (int)step;
        shuffle_cameras();
        return current_step;
    }
};

// ---------------------------------------------------------------------------
// Viewer
// ---------------------------------------------------------------------------

struct ViewerImpl {
    MsplatEngine *eng = nullptr;
    DeviceModel model;
    int width = 0, height = 0;
    float fovY = 1.0f;
    float bg[3] = {0, 0, 0};
    float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0}, dcenter[3] = {0, 0, 0};

    ~ViewerImpl() {
        if (eng) msplat_engine_destroy(eng);
    }

    void load(const std::string &ply) {
        int step = 0;
        const float zero[3] = {0, 0, 0};
        HostGaussians h = read_ply(ply, &step, false, 1.0f, zero);
        model.allocate(h.n, h.rest);
        model.n = h.n;
        for (int g = 0; g < 6; g++) model.write(model.p, g, h.a[g].data(), h.n);
        // bounds and the centre of the densest cell of an 8x8x8 grid
        // (msplat_api.mm:436-486)
        for (int k = 0; k < 3; k++) bmin[k] = bmax[k] = h.a[0][k];
        for (int i = 1; i < h.n; i++)
            for (int k = 0; k < 3; k++) {
                bmin[k] = std::min(bmin[k], h.a[0][3 * i + k]);
                bmax[k] = std::max(bmax[k], h.a[0][3 * i + k]);
            }
        constexpr int G = 8;
        std::vector<int> grid(G * G * G, 0);
        float ext[3];
        for (int k = 0; k < 3; k++) ext[k] = std::max(bmax[k] - bmin[k], 1e-6f);
        for (int i = 0; i < h.n; i++) {
            int c[3];
            for (int k = 0; k < 3; k++) c[k] = std::min((int)((h.a[0][3 * i + k] - bmin[k]) / ext[k] * G), G - 1);
            grid[c[0] * G * G + c[1] * G + c[2]]++;
        }
        const int best = (int)(std::max_element(grid.begin(), grid.end()) - grid.begin());
        const int c[3] = {best / (G * G), (best / G) % G, best % G};
        for (int k = 0; k < 3; k++) dcenter[k] = bmin[k] + (c[k] + 0.5f) / G * ext[k];
    }

    // intrinsics from the vertical field of view (msplat_api.mm:488-553)
    void render(const float c2w[16]) {
        const float fy = (float)height / (2.0f * std::tan(fovY * 0.5f));
        const float aspect = (float)width / (float)height;
        const float fovX = 2.0f * std::atan(std::tan(fovY * 0.5f) * aspect);
        const float fx = (float)width / (2.0f * std::tan(fovX * 0.5f));
        MsplatStepArgs a;
        std::memset(&a, 0, sizeof(a));
        msplat_prepare_camera(c2w, width, height, fx, fy, a.viewmat, a.projmat, a.cam_pos);
        a.fx = fx; a.fy = fy; a.cx = width * 0.5f; a.cy = height * 0.5f;
        a.width = width; a.height = height;
        std::memcpy(a.background, bg, sizeof(bg));
        a.clip_thresh = 0.01f;
        a.degrees_to_use = degree_for_rest(model.rest);
        MsplatGaussians g = model.gaussians();
        if (msplat_engine_render(eng, &g, &a) != 0) throw std::runtime_error(msplat_engine_last_error(eng));
    }
};

static void to_rgba(const float *src, uint8_t *dst, int n) {
    for (int i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) dst[4 * i + c] = (uint8_t)(std::fmin(std::fmax(src[3 * i + c], 0.f), 1.f) * 255.f);
        dst[4 * i + 3] = 255;
    }
}

template <class F> static auto guard(const char *what, F &&f, decltype(f()) fallback) -> decltype(f()) {
    try {
        return f();
    } catch (const std::exception &e) {
        fprintf(stderr, "msplat %s: %s\n", what, e.what());
        return fallback;
    }
}

}  // namespace msplat

using namespace msplat;

// A dataset directory (Camera::loadImage + inputDataFromX,
// core/src/input_data.cpp:22-73 and 244-261): cameras and seed points from
// the layout, poses centred and scaled, then every image decoded, its
// intrinsics rescaled to the decoded size, area-downscaled by the factor,
// undistorted when the camera has distortion, and quantised to 8 bits.
// Images decode on all host threads.
// Camera::loadMask (core/src/input_data.cpp:81-111): "<dir>/<name>.png",
// else the name with its extension replaced by .png; resized to the
// camera's final size by area averaging; kept where the first channel is
// above 0.5; all-white leaves the camera unmasked.
static void load_mask(HostCamera &c, const std::string &dir, const std::string &name) {
    if (dir.empty() || name.empty() || c.width <= 0 || c.height <= 0) return;
    namespace fs = std::filesystem;
    const fs::path appended = fs::path(dir) / (name + ".png");
    const fs::path swapped = (fs::path(dir) / name).replace_extension(".png");
    std::string file;
    if (fs::exists(appended)) file = appended.string();
    else if (fs::exists(swapped)) file = swapped.string();
    else return;
    io::Image m = io::read_image(file);
    if (m.width <= 0 || m.height <= 0) return;
    if (m.width != c.width || m.height != c.height) m = io::resize_area(m, c.width, c.height);
    const size_t n = (size_t)c.width * (size_t)c.height;
    std::vector<uint8_t> keep(n);
    long long kept = 0;
    for (size_t i = 0; i < n; i++) {
        const bool k = m.rgb[i * 3] > 0.5f;
        keep[i] = k ? 255 : 0;
        kept += k ? 1 : 0;
    }
    if (kept == (long long)n) return;
    c.mask = std::move(keep);
    c.unmasked = kept;
}

static MsplatDataset msplat_dataset_load(const char *path, float downscale, bool eval_mode, int test_every,
                                         const char *colmap_image_dir = nullptr, const char *mask_dir = nullptr) {
    if (!path) throw std::runtime_error("dataset path is null");
    io::LoadedScene sc = io::load_scene(path, colmap_image_dir ? colmap_image_dir : "");
    auto d = std::make_unique<DatasetImpl>();
    std::vector<HostCamera> cams(sc.cameras.size());
    for (size_t i = 0; i < cams.size(); i++) std::memcpy(cams[i].c2w, sc.cameras[i].c2w, 64);
    d->xyz = std::move(sc.xyz);
    d->rgb = std::move(sc.rgb);
    if (d->xyz.empty()) throw std::runtime_error(std::string("dataset has no seed points: ") + path);
    auto_scale_and_center(cams, d->xyz, d->scale, d->translation);
    std::vector<std::string> errors(cams.size());
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i = next++; i < cams.size(); i = next++) {
            try {
                const io::LoadedCamera &lc = sc.cameras[i];
                HostCamera &c = cams[i];
                c.path = lc.path;
                io::Image img = io::read_image(lc.path);
                c.width = lc.width; c.height = lc.height;
                c.fx = lc.fx; c.fy = lc.fy; c.cx = lc.cx; c.cy = lc.cy;
                if (c.width > 0 && c.height > 0 && (img.width != c.width || img.height != c.height)) {
                    const float sx = (float)img.width / (float)c.width, sy = (float)img.height / (float)c.height;
                    c.fx *= sx; c.fy *= sy; c.cx *= sx; c.cy *= sy;
                }
                c.width = img.width;
                c.height = img.height;
                if (downscale > 1.0f) {
                    const int nw = (int)(c.width / downscale), nh = (int)(c.height / downscale);
                    img = io::resize_area(img, nw, nh);
                    const float sx = (float)nw / (float)c.width, sy = (float)nh / (float)c.height;
                    c.fx *= sx; c.fy *= sy; c.cx *= sx; c.cy *= sy;
                    c.width = nw;
                    c.height = nh;
                }
                if (lc.k1 != 0.f || lc.k2 != 0.f || lc.k3 != 0.f || lc.p1 != 0.f || lc.p2 != 0.f)
                    img = io::undistort(img, c.fx, c.fy, c.cx, c.cy, lc.k1, lc.k2, lc.p1, lc.p2, lc.k3);
                c.image.resize(img.rgb.size());
                for (size_t k = 0; k < img.rgb.size(); k++)
                    c.image[k] = (uint8_t)std::min(std::max(std::round(img.rgb[k] * 255.0f), 0.0f), 255.0f);
                if (mask_dir) load_mask(c, mask_dir, lc.relative_name);
            } catch (const std::exception &e) {
                errors[i] = e.what();
            }
        }
    };
    const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 32u));
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; t++) pool.emplace_back(work);
    for (auto &t : pool) t.join();
    for (size_t i = 0; i < cams.size(); i++)
        if (!errors[i].empty()) throw std::runtime_error(sc.cameras[i].path + ": " + errors[i]);
    if (eval_mode) {
        const int every = std::max(1, test_every);
        for (size_t i = 0; i < cams.size(); i++) (i % every == 0 ? d->test : d->train).push_back(std::move(cams[i]));
    } else {
        d->train = std::move(cams);
    }
    return d.release();
}

static DatasetImpl *DS(MsplatDataset d) { return static_cast<DatasetImpl *>(d); }
static TrainerImpl *TR(MsplatTrainer t) { return static_cast<TrainerImpl *>(t); }
static ViewerImpl *VW(MsplatViewer v) { return static_cast<ViewerImpl *>(v); }

extern "C" {

MsplatDataset msplat_dataset_create(const char *path, float downscaleFactor, bool evalMode, int testEvery) {
    return guard("dataset", [&]() -> MsplatDataset {
        return msplat_dataset_load(path, downscaleFactor, evalMode, testEvery);
    }, (MsplatDataset) nullptr);
}

MsplatDataset msplat_dataset_create_ex(const char *path, float downscaleFactor, bool evalMode, int testEvery,
                                       const char *colmapImagePath) {
    return guard("dataset", [&]() -> MsplatDataset {
        return msplat_dataset_load(path, downscaleFactor, evalMode, testEvery, colmapImagePath);
    }, (MsplatDataset) nullptr);
}

MsplatDataset msplat_dataset_create_masked(const char *path, float downscaleFactor, bool evalMode, int testEvery,
                                           const char *colmapImagePath, const char *maskDir) {
    return guard("dataset", [&]() -> MsplatDataset {
        return msplat_dataset_load(path, downscaleFactor, evalMode, testEvery, colmapImagePath,
                                   maskDir && maskDir[0] ? maskDir : nullptr);
    }, (MsplatDataset) nullptr);
}

int msplat_dataset_camera_file(MsplatDataset ds, int i, int use_test, char *path, int capacity) {
    if (!ds) return -1;
    auto &cams = use_test ? DS(ds)->test : DS(ds)->train;
    if (i < 0 || i >= (int)cams.size()) return -1;
    const std::string &p = cams[i].path;
    if (path && capacity > 0) std::snprintf(path, (size_t)capacity, "%s", p.c_str());
    return (int)p.size();
}

int msplat_dataset_transform(MsplatDataset ds, float *scale, float translation[3]) {
    if (!ds) return -1;
    if (scale) *scale = DS(ds)->scale;
    if (translation)
        for (int k = 0; k < 3; k++) translation[k] = DS(ds)->translation[k];
    return 0;
}

int msplat_dataset_hold_out(MsplatDataset ds, const char *val_image) {
    if (!ds) return -1;
    DatasetImpl *d = DS(ds);
    if (d->train.empty() || !d->test.empty()) return -1;
    // InputData::getCameras (core/src/input_data.cpp:173-194)
    int idx = -1;
    const std::string want = val_image ? val_image : "random";
    if (want == "random") {
        std::mt19937 rng(42);
        idx = (int)(rng() % d->train.size());
    } else {
        for (int i = 0; i < (int)d->train.size(); i++)
            if (d->train[i].path.find(want) != std::string::npos) { idx = i; break; }
    }
    if (idx < 0) idx = 0;
    d->test.push_back(std::move(d->train[idx]));
    d->train.erase(d->train.begin() + idx);
    return idx;
}

long long msplat_dataset_mask(MsplatDataset ds, int i, int use_test, uint8_t *mask) {
    if (!ds) return -2;
    auto &cams = use_test ? DS(ds)->test : DS(ds)->train;
    if (i < 0 || i >= (int)cams.size()) return -2;
    const HostCamera &c = cams[i];
    if (c.mask.empty()) return -1;
    if (mask) std::memcpy(mask, c.mask.data(), c.mask.size());
    return c.unmasked;
}

MsplatDataset msplat_dataset_create_from_memory(int num_cameras, const float *cam_to_world, const float *intrinsics,
                                               const int *sizes, const uint8_t *const *images,
                                               const uint8_t *const *masks, int num_points, const float *xyz,
                                               const uint8_t *rgb, bool eval_mode, int test_every, bool normalize) {
    if (num_cameras < 0 || num_points < 0) return nullptr;
    if (num_cameras > 0 && (!cam_to_world || !intrinsics || !sizes)) return nullptr;
    if (num_points > 0 && (!xyz || !rgb)) return nullptr;
    for (int i = 0; i < num_cameras; i++)
        if (sizes[2 * i] <= 0 || sizes[2 * i + 1] <= 0) return nullptr;
    return guard("dataset", [&]() -> MsplatDataset {
        auto d = std::make_unique<DatasetImpl>();
        std::vector<HostCamera> cams(num_cameras);
        for (int i = 0; i < num_cameras; i++) {
            HostCamera &c = cams[i];
            std::memcpy(c.c2w, cam_to_world + 16 * i, 64);
            c.fx = intrinsics[4 * i]; c.fy = intrinsics[4 * i + 1];
            c.cx = intrinsics[4 * i + 2]; c.cy = intrinsics[4 * i + 3];
            c.width = sizes[2 * i]; c.height = sizes[2 * i + 1];
            const size_t P = (size_t)c.width * c.height;
            if (images && images[i]) c.image.assign(images[i], images[i] + 3 * P);
            if (masks && masks[i]) {
                long long keep = 0;
                c.mask.resize(P);
                for (size_t p = 0; p < P; p++) { c.mask[p] = masks[i][p] >= 128 ? 255 : 0; keep += c.mask[p] ? 1 : 0; }
                if (keep == (long long)P) c.mask.clear();
                else c.unmasked = keep;
            }
        }
        d->xyz.assign(xyz, xyz + 3 * (size_t)num_points);
        d->rgb.assign(rgb, rgb + 3 * (size_t)num_points);
        if (normalize) auto_scale_and_center(cams, d->xyz, d->scale, d->translation);
        if (eval_mode) {
            const int every = std::max(1, test_every);
            for (int i = 0; i < num_cameras; i++) (i % every == 0 ? d->test : d->train).push_back(cams[i]);
        } else {
            d->train = cams;
        }
        return d.release();
    }, (MsplatDataset) nullptr);
}

void msplat_dataset_destroy(MsplatDataset ds) { delete DS(ds); }

int msplat_dataset_camera(MsplatDataset ds, int i, int use_test, float intrinsics[4], int size[2], float c2w[16],
                          uint8_t *image) {
    if (!ds) return -1;
    auto &cams = use_test ? DS(ds)->test : DS(ds)->train;
    if (i < 0 || i >= (int)cams.size()) return -1;
    const HostCamera &c = cams[i];
    if (intrinsics) { intrinsics[0] = c.fx; intrinsics[1] = c.fy; intrinsics[2] = c.cx; intrinsics[3] = c.cy; }
    if (size) { size[0] = c.width; size[1] = c.height; }
    if (c2w) std::memcpy(c2w, c.c2w, 64);
    if (image) std::memcpy(image, c.image.data(), c.image.size());
    return 0;
}

int msplat_dataset_points(MsplatDataset ds, float *xyz, uint8_t *rgb) {
    if (!ds) return -1;
    const DatasetImpl *d = DS(ds);
    if (xyz) std::memcpy(xyz, d->xyz.data(), d->xyz.size() * sizeof(float));
    if (rgb) std::memcpy(rgb, d->rgb.data(), d->rgb.size());
    return (int)(d->xyz.size() / 3);
}

int msplat_image_read(const char *path, float *rgb, int *width, int *height) {
    if (!path) return -1;
    return guard("image", [&]() {
        io::Image im = io::read_image(path);
        if (width) *width = im.width;
        if (height) *height = im.height;
        if (rgb) std::memcpy(rgb, im.rgb.data(), im.rgb.size() * sizeof(float));
        return 0;
    }, -2);
}
int msplat_image_resize(const float *rgb, int width, int height, int out_width, int out_height, float *out) {
    if (!rgb || !out || width <= 0 || height <= 0 || out_width <= 0 || out_height <= 0) return -1;
    return guard("image_resize", [&]() {
        io::Image im;
        im.width = width;
        im.height = height;
        im.rgb.assign(rgb, rgb + (size_t)width * height * 3);
        const io::Image r = io::resize_area(im, out_width, out_height);
        std::memcpy(out, r.rgb.data(), r.rgb.size() * sizeof(float));
        return 0;
    }, -2);
}
int msplat_checkpoint_info(const char *path, int *num_points, int *sh_degree, int *iteration) {
    if (!path) return -1;
    return guard("checkpoint", [&]() {
        const CheckpointData ck = read_checkpoint(path);
        if (num_points) *num_points = (int)ck.n;
        if (sh_degree) *sh_degree = (int)ck.deg;
        if (iteration) *iteration = (int)ck.step;
        return 0;
    }, -1);
}
int msplat_write_checkpoint(const char *path, int iteration, int n, int sh_degree, int adam_steps,
                            const float adam_lr[6], float means_lr_init, float means_lr_final,
                            const float *const params[6], const float *const exp_avg[6],
                            const float *const exp_avg_sq[6]) {
    if (!path || n < 0 || sh_degree < 0 || sh_degree > 3 || iteration < 0 || adam_steps < 0 || !adam_lr ||
        !params || !exp_avg || !exp_avg_sq)
        return -1;
    const int rest = (sh_degree + 1) * (sh_degree + 1) - 1;
    const int width[6] = {3, 3, 4, 3, 3 * rest, 1};
    const float *const *src[3] = {params, exp_avg, exp_avg_sq};
    for (int k = 0; k < 18; k++)
        if (n > 0 && width[k % 6] > 0 && !src[k / 6][k % 6]) return -1;
    return guard("write_checkpoint", [&]() {
        CheckpointData ck;
        ck.step = (uint32_t)iteration;
        ck.n = (uint32_t)n;
        ck.deg = (uint32_t)sh_degree;
        ck.adam_steps = (uint32_t)adam_steps;
        std::memcpy(ck.adam_lr, adam_lr, sizeof(ck.adam_lr));
        ck.means_lr_init = means_lr_init;
        ck.means_lr_final = means_lr_final;
        ck.rest = rest;
        for (int k = 0; k < 18; k++) {
            const float *a = src[k / 6][k % 6];
            const size_t cnt = (size_t)n * width[k % 6];
            if (cnt) ck.t[k].assign(a, a + cnt);
        }
        write_checkpoint(path, ck);
        return 0;
    }, -2);
}
int msplat_read_checkpoint(const char *path, float adam_lr[6], float means_lr[2], int *adam_steps,
                           float *const params[6], float *const exp_avg[6], float *const exp_avg_sq[6]) {
    if (!path) return -1;
    return guard("read_checkpoint", [&]() {
        const CheckpointData ck = read_checkpoint(path);
        if (adam_lr) std::memcpy(adam_lr, ck.adam_lr, sizeof(ck.adam_lr));
        if (means_lr) { means_lr[0] = ck.means_lr_init; means_lr[1] = ck.means_lr_final; }
        if (adam_steps) *adam_steps = (int)ck.adam_steps;
        float *const *dst[3] = {params, exp_avg, exp_avg_sq};
        for (int k = 0; k < 18; k++)
            if (dst[k / 6] && dst[k / 6][k % 6] && !ck.t[k].empty())
                std::memcpy(dst[k / 6][k % 6], ck.t[k].data(), ck.t[k].size() * sizeof(float));
        return 0;
    }, -2);
}
static bool host_gaussians_args(int n, int rest_bases, const float *means, const float *scales, const float *quats,
                                const float *features_dc, const float *features_rest, const float *opacities) {
    if (n < 0 || rest_bases < 0 || rest_bases > 24) return false;
    return n == 0 || (means && scales && quats && features_dc && opacities && (rest_bases == 0 || features_rest));
}
static HostGaussians host_gaussians(int n, int rest_bases, const float *means, const float *scales,
                                    const float *quats, const float *features_dc, const float *features_rest,
                                    const float *opacities) {
    HostGaussians h;
    h.n = n;
    h.rest = rest_bases;
    const float *src[6] = {means, scales, quats, features_dc, features_rest, opacities};
    const size_t w[6] = {3, 3, 4, 3, (size_t)3 * rest_bases, 1};
    for (int g = 0; g < 6; g++)
        if (src[g]) h.a[g].assign(src[g], src[g] + (size_t)n * w[g]);
    return h;
}
int msplat_write_ply(const char *path, int n, int rest_bases, const float *means, const float *scales,
                     const float *quats, const float *features_dc, const float *features_rest,
                     const float *opacities, int step, int keep_crs, float scale, const float translation[3]) {
    if (!path || !host_gaussians_args(n, rest_bases, means, scales, quats, features_dc, features_rest, opacities) ||
        (keep_crs && (!translation || !(scale > 0.f))))
        return -1;
    return guard("write_ply", [&]() {
        const float zero[3] = {0.f, 0.f, 0.f};
        write_ply(path, host_gaussians(n, rest_bases, means, scales, quats, features_dc, features_rest, opacities),
                  step, keep_crs != 0, scale, translation ? translation : zero);
        return 0;
    }, -2);
}
int msplat_write_splat(const char *path, int n, int rest_bases, const float *means, const float *scales,
                       const float *quats, const float *features_dc, const float *features_rest,
                       const float *opacities, int keep_crs, float scale, const float translation[3]) {
    if (!path || !host_gaussians_args(n, rest_bases, means, scales, quats, features_dc, features_rest, opacities) ||
        (keep_crs && (!translation || !(scale > 0.f))))
        return -1;
    return guard("write_splat", [&]() {
        const float zero[3] = {0.f, 0.f, 0.f};
        write_splat(path, host_gaussians(n, rest_bases, means, scales, quats, features_dc, features_rest, opacities),
                    keep_crs != 0, scale, translation ? translation : zero);
        return 0;
    }, -2);
}
int msplat_ply_info(const char *path, int *num_points, int *rest_bases, int *iteration) {
    if (!path) return -1;
    return guard("ply_info", [&]() {
        int step = 0;
        const HostGaussians h = read_ply(path, &step, false, 1.f, nullptr);
        if (num_points) *num_points = h.n;
        if (rest_bases) *rest_bases = h.rest;
        if (iteration) *iteration = step;
        return 0;
    }, -2);
}
int msplat_read_ply(const char *path, int keep_crs, float scale, const float translation[3], float *means,
                    float *scales, float *quats, float *features_dc, float *features_rest, float *opacities) {
    if (!path || !means || !scales || !quats || !features_dc || !opacities ||
        (keep_crs && (!translation || !(scale > 0.f))))
        return -1;
    return guard("read_ply", [&]() {
        const HostGaussians h = read_ply(path, nullptr, keep_crs != 0, scale, translation);
        float *dst[6] = {means, scales, quats, features_dc, features_rest, opacities};
        for (int g = 0; g < 6; g++)
            if (dst[g] && !h.a[g].empty()) std::memcpy(dst[g], h.a[g].data(), h.a[g].size() * sizeof(float));
        return 0;
    }, -2);
}
int msplat_dataset_num_train(MsplatDataset ds) { return ds ? (int)DS(ds)->train.size() : 0; }
int msplat_dataset_num_test(MsplatDataset ds) { return ds ? (int)DS(ds)->test.size() : 0; }

void msplat_dataset_camera_pose(MsplatDataset ds, int i, float c2w[16]) {
    if (ds && c2w && i >= 0 && i < (int)DS(ds)->train.size()) std::memcpy(c2w, DS(ds)->train[i].c2w, 64);
}

MsplatTrainer msplat_trainer_create(MsplatDataset ds, MsplatConfig config) {
    return msplat_trainer_create_ex(ds, config, nullptr);
}

void msplat_default_trainer_options(MsplatTrainerOptions *options) {
    if (options) *options = default_trainer_options();
}

MsplatTrainer msplat_trainer_create_ex(MsplatDataset ds, MsplatConfig config, const MsplatTrainerOptions *options) {
    const MsplatTrainerOptions o = options ? *options : default_trainer_options();
    if (!ds || !trainer_options_valid(o)) return nullptr;
    return guard("trainer", [&]() -> MsplatTrainer { return new TrainerImpl(DS(ds), config, o); },
                 (MsplatTrainer) nullptr);
}

int msplat_seed_gaussians(int num_points, const float *xyz, const uint8_t *rgb, int sh_degree, int cap_max,
                          const MsplatTrainerOptions *options, float *means, float *scales, float *quats,
                          float *features_dc, float *features_rest, float *opacities) {
    const MsplatTrainerOptions o = options ? *options : default_trainer_options();
    if (num_points < 0 || sh_degree < 0 || sh_degree > 3 || cap_max < 1 || !trainer_options_valid(o)) return -1;
    if (num_points > 0 && (!xyz || !rgb || !means || !scales || !quats || !features_dc || !opacities ||
                           (sh_degree > 0 && !features_rest)))
        return -1;
    return guard("seed_gaussians", [&]() {
        const std::vector<float> p(xyz, xyz + 3 * (size_t)num_points);
        const std::vector<uint8_t> c(rgb, rgb + 3 * (size_t)num_points);
        const HostGaussians h = seed_gaussians(p, c, sh_degree, o);
        std::vector<int> keep;
        const int rows = seed_rows(h.n, cap_max, o.seedDecimation != 0, keep);
        float *dst[6] = {means, scales, quats, features_dc, features_rest, opacities};
        const size_t w[6] = {3, 3, 4, 3, (size_t)3 * h.rest, 1};
        for (int g = 0; g < 6; g++) {
            if (!dst[g] || !w[g]) continue;
            for (int i = 0; i < rows; i++)
                std::memcpy(dst[g] + (size_t)i * w[g], &h.a[g][(size_t)(keep.empty() ? i : keep[i]) * w[g]],
                            w[g] * sizeof(float));
        }
        return rows;
    }, -1);
}

void msplat_trainer_destroy(MsplatTrainer t) { delete TR(t); }

MsplatStats msplat_trainer_step(MsplatTrainer t) {
    MsplatStats empty{0, 0, 0.f};
    if (!t) return empty;
    return guard("step", [&]() { return TR(t)->step(); }, empty);
}

void msplat_trainer_train(MsplatTrainer t) {
    if (!t) return;
    guard("train", [&]() {
        while (TR(t)->current_step < TR(t)->cfg.iterations) TR(t)->step();
        return 0;
    }, 0);
}

MsplatEvalMetrics msplat_trainer_evaluate(MsplatTrainer t) {
    MsplatEvalMetrics empty{};
    if (!t) return empty;
    return guard("evaluate", [&]() { return TR(t)->evaluate(); }, empty);
}

static MsplatPixelBuffer pixel_buffer(std::vector<float> &&img, int w, int h) {
    MsplatPixelBuffer b{nullptr, 0, 0};
    b.data = static_cast<float *>(std::malloc(img.size() * sizeof(float)));
    if (!b.data) return b;
    std::memcpy(b.data, img.data(), img.size() * sizeof(float));
    b.width = w;
    b.height = h;
    return b;
}

MsplatPixelBuffer msplat_trainer_render(MsplatTrainer t, int i, bool useTest) {
    MsplatPixelBuffer empty{nullptr, 0, 0};
    if (!t) return empty;
    return guard("render", [&]() {
        auto &cams = useTest ? TR(t)->ds->test : TR(t)->ds->train;
        if (i < 0 || i >= (int)cams.size()) return empty;
        HostCamera &c = cams[i];
        return pixel_buffer(TR(t)->render_cam(c, TR(t)->current_step), c.width, c.height);
    }, empty);
}

MsplatPixelBuffer msplat_trainer_render_pose(MsplatTrainer t, const float c2w[16], int ref) {
    MsplatPixelBuffer empty{nullptr, 0, 0};
    if (!t || !c2w) return empty;
    return guard("render_pose", [&]() {
        auto &cams = TR(t)->ds->train;
        if (ref < 0 || ref >= (int)cams.size()) return empty;
        HostCamera c;
        const HostCamera &r = cams[ref];
        c.width = r.width; c.height = r.height; c.fx = r.fx; c.fy = r.fy; c.cx = r.cx; c.cy = r.cy;
        std::memcpy(c.c2w, c2w, 64);
        return pixel_buffer(TR(t)->render_cam(c, TR(t)->current_step), c.width, c.height);
    }, empty);
}

void msplat_trainer_render_pose_to_buffer(MsplatTrainer t, const float c2w[16], int ref, uint8_t *out, int *ow,
                                          int *oh) {
    if (ow) *ow = 0;
    if (oh) *oh = 0;
    if (!t || !c2w) return;
    guard("render_pose_to_buffer", [&]() {
        auto &cams = TR(t)->ds->train;
        if (ref < 0 || ref >= (int)cams.size()) return 0;
        HostCamera c;
        const HostCamera &r = cams[ref];
        c.width = r.width; c.height = r.height; c.fx = r.fx; c.fy = r.fy; c.cx = r.cx; c.cy = r.cy;
        std::memcpy(c.c2w, c2w, 64);
        if (ow) *ow = c.width;
        if (oh) *oh = c.height;
        if (!out) return 0;
        auto img = TR(t)->render_cam(c, TR(t)->current_step);
        to_rgba(img.data(), out, c.width * c.height);
        return 0;
    }, 0);
}

void msplat_trainer_export_ply(MsplatTrainer t, const char *path) {
    if (!t || !path) return;
    guard("export_ply", [&]() {
        auto h = TR(t)->host_model();
        write_ply(path, h, TR(t)->current_step, TR(t)->cfg.keepCrs, TR(t)->ds->scale, TR(t)->ds->translation);
        return 0;
    }, 0);
}

void msplat_trainer_export_splat(MsplatTrainer t, const char *path) {
    if (!t || !path) return;
    guard("export_splat", [&]() {
        auto h = TR(t)->host_model();
        write_splat(path, h, TR(t)->cfg.keepCrs, TR(t)->ds->scale, TR(t)->ds->translation);
        return 0;
    }, 0);
}

void msplat_trainer_save_checkpoint(MsplatTrainer t, const char *path) {
    if (!t || !path) return;
    guard("save_checkpoint", [&]() { TR(t)->save_checkpoint(path); return 0; }, 0);
}

int msplat_trainer_load_checkpoint(MsplatTrainer t, const char *path) {
    if (!t || !path) return 0;
    return guard("load_checkpoint", [&]() { return TR(t)->load_checkpoint(path); }, 0);
}

int msplat_trainer_splat_count(MsplatTrainer t) { return t ? TR(t)->model.n : 0; }
int msplat_trainer_iteration(MsplatTrainer t) { return t ? TR(t)->current_step : 0; }

void msplat_set_metallib_path(const char *path) { (void)path; }
void msplat_sync(void) { cudaDeviceSynchronize(); }
void msplat_cleanup(void) {}

// ---- GB300 extensions (msplat_gb300.h) ----

int msplat_trainer_set_gaussians(MsplatTrainer t, int n, int rest_bases, const float *means, const float *scales,
                                 const float *quats, const float *features_dc, const float *features_rest,
                                 const float *opacities) {
    // the engine takes up to 15 rest bases (SH degree 3); every array must be
    // given when there are rows (features_rest only with rest bases)
    if (!t || n < 0 || rest_bases < 0 || rest_bases > 15) return -1;
    if (n > 0 && (!means || !scales || !quats || !features_dc || !opacities || (rest_bases > 0 && !features_rest)))
        return -1;
    return guard("set_gaussians", [&]() {
        HostGaussians h;
        h.n = n;
        h.rest = rest_bases;
        const float *src[6] = {means, scales, quats, features_dc, features_rest, opacities};
        const size_t s[6] = {3, 3, 4, 3, (size_t)3 * rest_bases, 1};
        for (int g = 0; g < 6; g++)
            if (src[g]) h.a[g].assign(src[g], src[g] + (size_t)n * s[g]);
        TR(t)->set_model(h, false);
        return 0;
    }, -2);
}

int msplat_trainer_get_gaussians(MsplatTrainer t, float *means, float *scales, float *quats, float *features_dc,
                                 float *features_rest, float *opacities) {
    if (!t) return -1;
    return guard("get_gaussians", [&]() {
        auto h = TR(t)->host_model();
        float *dst[6] = {means, scales, quats, features_dc, features_rest, opacities};
        for (int g = 0; g < 6; g++)
            if (dst[g]) std::memcpy(dst[g], h.a[g].data(), h.a[g].size() * 4);
        return 0;
    }, -2);
}

int msplat_trainer_set_learned_relocation(MsplatTrainer t, int enabled) {
    if (!t) return -1;
    return guard("learned_relocation", [&]() { TR(t)->enable_learned(enabled != 0); return 0; }, -2);
}

int msplat_trainer_set_learned_prune(MsplatTrainer t, float forecast_opacity) {
    if (!t || !(forecast_opacity >= 0.f && forecast_opacity < 1.f)) return -1;
    TR(t)->lrn.prune = forecast_opacity;
    return 0;
}

int msplat_trainer_set_batch_views(MsplatTrainer t, int num_views, float lr_scale) {
    if (!t || num_views < 1 || num_views > 16) return -1;
    TR(t)->batch_views = num_views;
    TR(t)->batch_lr_scale = lr_scale > 0.f ? lr_scale : std::pow((float)num_views, 0.75f);
    return 0;
}

int msplat_trainer_set_isect_budget(MsplatTrainer t, float bytes_per_gaussian) {
    if (!t || !(bytes_per_gaussian >= 0.f)) return -1;
    return guard("isect_budget", [&]() {
        TrainerImpl *tr = TR(t);
        long long slots = 0;
        if (bytes_per_gaussian > 0.f) {
            // 20 bytes per slot (key, sort scratch, id); at least one view's worth
            // of one Gaussian per tile slot count, so that any single tile fits
            const long long cap = std::max(1, tr->model.cap);
            slots = std::max<long long>(cap, (long long)((double)bytes_per_gaussian * (double)cap / 20.0));
        }
        return msplat_engine_set_isect_budget(tr->eng, slots);
    }, -2);
}

int msplat_trainer_autotune(MsplatTrainer t, MsplatTuning *out) {
    if (!t) return -1;
    return guard("autotune", [&]() {
        TrainerImpl *tr = TR(t);
        if (tr->ds->train.empty()) throw std::runtime_error("dataset has no training cameras");
        // the next batch of cameras of the shuffled order (without advancing it)
        const int B = std::max(1, tr->batch_views);
        std::vector<MsplatStepArgs> a(B);
        std::vector<const uint8_t *> gt(B), mk(B);
        for (int v = 0; v < B; v++) {
            HostCamera &cam = tr->ds->train[tr->cam_order[(tr->cam_pos + v) % tr->cam_order.size()]];
            cam.upload();
            tr->step_args(cam, std::max(1, tr->current_step), a[v], true);
            gt[v] = cam.d_image;
            mk[v] = cam.d_mask;
        }
        MsplatGaussians g = tr->model.gaussians();
        MsplatTuning tun{};
        const int rc = msplat_engine_autotune(tr->eng, &g, a.data(), B, gt.data(), mk.data(), 3, &tun, nullptr);
        if (rc == 0 && out) *out = tun;
        return rc;
    }, -2);
}

int msplat_trainer_learned_stats(MsplatTrainer t, float *last_loss, int *rounds) {
    if (!t) return -1;
    if (last_loss) *last_loss = TR(t)->lrn.last_loss;
    if (rounds) *rounds = TR(t)->lrn.rounds;
    return TR(t)->lrn.enabled ? 1 : 0;
}

int msplat_trainer_learned_eval(MsplatTrainer t, float mse[4]) {
    if (!t || !mse) return -1;
    const auto &l = TR(t)->lrn;
    for (int k = 0; k < 4; k++) mse[k] = l.eval_rounds ? (float)(l.eval_sum[k] / l.eval_rounds) : 0.f;
    return l.eval_rounds;
}

int msplat_trainer_load_ply(MsplatTrainer t, const char *path) {
    if (!t || !path) return -1;
    return guard("load_ply", [&]() { return TR(t)->load_ply(path); }, -2);
}

float msplat_trainer_last_loss(MsplatTrainer t) {
    if (!t) return NAN;
    float v = NAN;
    msplat_engine_loss(TR(t)->eng, &v);
    return v;
}

MsplatEngine *msplat_trainer_engine(MsplatTrainer t) { return t ? TR(t)->eng : nullptr; }

int msplat_trainer_mcmc_stats(MsplatTrainer t, MsplatMcmcStats *out) {
    if (!t) return -1;
    if (out) *out = TR(t)->last_mcmc;
    return TR(t)->mcmc_rounds;
}

// ---- viewer ----

MsplatViewer msplat_viewer_create(const char *ply, int width, int height, float fovY) {
    if (!ply || width <= 0 || height <= 0) return nullptr;
    return guard("viewer", [&]() -> MsplatViewer {
        auto v = std::make_unique<ViewerImpl>();
        int dev = 0;
        CKA(cudaGetDevice(&dev));
        v->eng = msplat_engine_create(dev, 0);
        if (!v->eng) throw std::runtime_error("engine creation failed");
        v->width = width;
        v->height = height;
        v->fovY = fovY;
        v->load(ply);
        return v.release();
    }, (MsplatViewer) nullptr);
}

void msplat_viewer_resize(MsplatViewer v, int w, int h) {
    if (v && w > 0 && h > 0) { VW(v)->width = w; VW(v)->height = h; }
}
void msplat_viewer_set_fov(MsplatViewer v, float fovY) {
    if (v) VW(v)->fovY = fovY;
}
void msplat_viewer_set_background(MsplatViewer v, float r, float g, float b) {
    if (v) { VW(v)->bg[0] = r; VW(v)->bg[1] = g; VW(v)->bg[2] = b; }
}

void msplat_viewer_render(MsplatViewer v, const float c2w[16], uint8_t *out) {
    if (!v || !c2w || !out) return;
    guard("viewer_render", [&]() {
        ViewerImpl *vw = VW(v);
        vw->render(c2w);
        std::vector<float> img((size_t)vw->width * vw->height * 3);
        if (msplat_engine_read(vw->eng, "out_img", img.data(), (long long)img.size() * 4) != 0)
            throw std::runtime_error(msplat_engine_last_error(vw->eng));
        to_rgba(img.data(), out, vw->width * vw->height);
        return 0;
    }, 0);
}

int msplat_viewer_splat_count(MsplatViewer v) { return v ? VW(v)->model.n : 0; }

void msplat_viewer_get_size(MsplatViewer v, int *w, int *h) {
    if (!v) return;
    if (w) *w = VW(v)->width;
    if (h) *h = VW(v)->height;
}

void *msplat_viewer_render_buffer(MsplatViewer v, const float c2w[16], int *w, int *h) {
    if (w) *w = 0;
    if (h) *h = 0;
    if (!v || !c2w) return nullptr;
    return guard("viewer_render_buffer", [&]() -> void * {
        ViewerImpl *vw = VW(v);
        vw->render(c2w);
        if (w) *w = vw->width;
        if (h) *h = vw->height;
        void *p = nullptr;
        msplat_engine_buffer(vw->eng, "out_img", &p);
        return p;
    }, (void *)nullptr);
}

void msplat_viewer_bounds(MsplatViewer v, float lo[3], float hi[3]) {
    if (!v) return;
    if (lo) std::memcpy(lo, VW(v)->bmin, 12);
    if (hi) std::memcpy(hi, VW(v)->bmax, 12);
}

void msplat_viewer_density_center(MsplatViewer v, float c[3]) {
    if (v && c) std::memcpy(c, VW(v)->dcenter, 12);
}

void *msplat_viewer_command_queue(MsplatViewer v) { return v ? msplat_engine_stream(VW(v)->eng) : nullptr; }

void msplat_viewer_destroy(MsplatViewer v) { delete VW(v); }

}  // extern "C"
