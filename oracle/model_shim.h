// Host stand-in for the reference's Model class (core/include/model.hpp:
// 17-130), with only the members its MCMC host code reads and writes, so
// that code compiles unchanged — TEST INFRASTRUCTURE ONLY (it pins the
// oracle's MCMC restatement; nothing in the product uses it).
//
// The reference keeps each parameter group and Adam moment as an MTensor
// (core/include/metal_tensor.hpp) whose storage is shared with the GPU; here
// a HostTensor is a row-major float array with the two accessors the code
// calls (data<T>() and stride0(), the floats per row).  The `*_buf` tensors
// and their active views (means, opacities, ...) are the same arrays, as in
// the reference after refreshViews().
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <limits>
#include <random>
#include <vector>

struct HostTensor {
    float *p = nullptr;
    int64_t row = 1;
    template <class T> T *data() { return reinterpret_cast<T *>(p); }
    template <class T> const T *data() const { return reinterpret_cast<const T *>(p); }
    int64_t stride0() const { return row; }
};

// GPU hooks the MCMC pass calls (core/metal/bindings.h): nothing to wait for
// on the host, and no gradient NaN counters to report.
inline void msplat_gpu_sync() {}
inline void msplat_grad_nan_counts(uint32_t out[16]) {
    for (int k = 0; k < 16; k++) out[k] = 0;
}

class Model {
public:
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

    void refreshViews() {}
    void computeRelocation(float opacity_old_sig, float *scale_old_exp, int N, float &opacity_new_sig,
                           float *scale_new_exp);
    void relocate(const std::vector<int> &dead, const std::vector<int> &alive);
    int addNewGaussians();
    void mcmcAfterTrain(int step);
};
