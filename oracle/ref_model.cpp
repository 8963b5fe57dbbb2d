// The reference's MCMC host code (core/src/model.cpp:311-660:
// computeRelocation, relocate, addNewGaussians, mcmcAfterTrain), compiled
// unchanged against oracle/model_shim.h — TEST INFRASTRUCTURE ONLY.  The
// code is copied into oracle/_ref/model_mcmc.inc by oracle/ref_build.py
// (never committed); this file only wraps it for ctypes.
#include "model_shim.h"

#include "model_mcmc.inc"

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

}  // extern "C"
