// Host wrappers around the reference's per-Gaussian Metal kernels — TEST
// INFRASTRUCTURE ONLY.  Built by oracle/ref_build.py into
// oracle/_ref/libmsplat_ref.so, which the oracle's pinning tests load.
//
// Each k_* function below has the parameter list of the reference kernel it
// runs (core/metal/msplat_metal.metal; address-space qualifiers and buffer
// attributes dropped) and its body is the kernel's body, copied unchanged
// from the reference at build time (oracle/_ref/k_<kernel>.inc).  The
// extern "C" entry points run it once per thread index on the host, in
// order, which is all these kernels need: no threadgroup memory, no
// barriers, and each thread writes only its own elements.
#include "metal_shim.h"

#include <type_traits>
#include <vector>

namespace mshim {
ExpFn g_expf = nullptr;
}

#include "ref_helpers.inc"

namespace {

// project_and_sh_forward_kernel (msplat_metal.metal:1719-1834)
void k_project_fwd(int &num_points, float *means3d, float *scales, float &glob_scale, float *quats, float *viewmat,
                   float *projmat, float4 &intrins, uint2 &img_size, uint3 &tile_bounds, float &clip_thresh,
                   float *xys, float *depths, int *radii, float *conics, int32_t *num_tiles_hit, uint &degree,
                   uint &degrees_to_use, float3 &cam_pos, float *features_dc, float *features_rest, float *colors,
                   float *aabb, atomic_uint *nan_counts, uint3 gp) {
#include "k_project_and_sh_forward_kernel.inc"
}

// project_and_sh_backward_kernel (msplat_metal.metal:1860-2042)
void k_project_bwd(int &num_points, float *means3d, float *scales, float &glob_scale, float *quats, float *viewmat,
                   float *projmat, float4 &intrins, uint2 &img_size, int *radii, float *conics, float *v_xy,
                   float *v_depth, float *v_conic, float *v_mean3d, float *v_scale, float *v_quat, uint &degree,
                   uint &degrees_to_use, float3 &cam_pos, float *v_colors, float *features_dc, float *features_rest,
                   float *dc_exp_avg, float *dc_exp_avg_sq, float *rest_exp_avg, float *rest_exp_avg_sq,
                   SHAdamParams &adam_hp, atomic_uint *nan_counts, uint idx) {
#include "k_project_and_sh_backward_kernel.inc"
}

// fused_adam_kernel (msplat_metal.metal:1680-1713)
void k_adam(float *params, const float *grads, float *exp_avg, float *exp_avg_sq, float &step_size, float &beta1,
            float &beta2, float &bc2_sqrt, float &eps, uint &n, atomic_uint *nan_counts, uint &group_idx, uint tid) {
#include "k_fused_adam_kernel.inc"
}

// sgld_noise_gen_kernel (msplat_metal.metal:3871-3890)
void k_sgld_gen(float *noise, int &N, uint &seed, uint idx) {
#include "k_sgld_noise_gen_kernel.inc"
}

// sgld_noise_kernel (msplat_metal.metal:3892-3967)
void k_sgld(float *means, float *scales, float *quats, float *opacities, float *noise, int &N, float &noise_lr,
            float &xyz_lr, float &max_disp, uint idx) {
#include "k_sgld_noise_kernel.inc"
}

// mcmc_reg_grad_kernel (msplat_metal.metal:3987-4026)
void k_reg(const float *opacities, const float *scales, float *v_opacity, float *v_scale, int &N, float &op_reg,
           float &sc_reg, const int *radii, float &invis_scale, const float *v_dc_sq, uint idx) {
#include "k_mcmc_reg_grad_kernel.inc"
}

template <class T> T *mut(const T *p) { return const_cast<T *>(p); }

}  // namespace

extern "C" {

// exp() of the compiled source: the given function, or libm's expf (NULL).
void ref_set_expf(float (*f)(float)) { mshim::g_expf = f; }

// Projection + SH colour of n Gaussians.  Outputs of culled Gaussians keep
// the values they had (the kernel writes only radii and tiles hit for them).
void ref_project_fwd(int n, const float *means, const float *scales, const float *quats, const float *viewmat,
                     const float *projmat, float fx, float fy, float cx, float cy, int width, int height,
                     float clip_thresh, int sh_degree, int degrees_to_use, const float cam_pos[3],
                     const float *features_dc, const float *features_rest, float *xys, float *depths, int *radii,
                     float *conics, int *num_tiles_hit, float *colors, float *aabb, uint32_t nan_counts[16]) {
    int num_points = n;
    float glob_scale = 1.f;
    float4 intrins(fx, fy, cx, cy);
    uint2 img_size((uint)width, (uint)height);
    uint3 tile_bounds((uint)(width + 15) / 16, (uint)(height + 15) / 16, 1u);
    uint degree = (uint)sh_degree, use = (uint)degrees_to_use;
    float3 cp(cam_pos[0], cam_pos[1], cam_pos[2]);
    for (uint i = 0; i < (uint)n; i++)
        k_project_fwd(num_points, mut(means), mut(scales), glob_scale, mut(quats), mut(viewmat), mut(projmat),
                      intrins, img_size, tile_bounds, clip_thresh, xys, depths, radii, conics, num_tiles_hit, degree,
                      use, cp, mut(features_dc), mut(features_rest), colors, aabb, nan_counts, uint3(i, 0u, 0u));
}

// Projection backward with the fused SH Adam.  v_depth may be NULL (zeros).
// v_mean3d/v_scale/v_quat of culled Gaussians keep their values.
void ref_project_bwd(int n, const float *means, const float *scales, const float *quats, const float *viewmat,
                     const float *projmat, float fx, float fy, float cx, float cy, int width, int height,
                     const int *radii, const float *conics, const float *v_xy, const float *v_depth,
                     const float *v_conic, const float *v_colors, int sh_degree, int degrees_to_use,
                     const float cam_pos[3], float *v_mean3d, float *v_scale, float *v_quat, float *features_dc,
                     float *features_rest, float *dc_exp_avg, float *dc_exp_avg_sq, float *rest_exp_avg,
                     float *rest_exp_avg_sq, float dc_step_size, float dc_bc2_sqrt, float rest_step_size,
                     float rest_bc2_sqrt, float beta1, float beta2, float eps, uint32_t nan_counts[16]) {
    int num_points = n;
    float glob_scale = 1.f;
    float4 intrins(fx, fy, cx, cy);
    uint2 img_size((uint)width, (uint)height);
    uint degree = (uint)sh_degree, use = (uint)degrees_to_use;
    float3 cp(cam_pos[0], cam_pos[1], cam_pos[2]);
    SHAdamParams hp;
    hp.dc_step_size = dc_step_size;
    hp.dc_bc2_sqrt = dc_bc2_sqrt;
    hp.rest_step_size = rest_step_size;
    hp.rest_bc2_sqrt = rest_bc2_sqrt;
    hp.beta1 = beta1;
    hp.beta2 = beta2;
    hp.eps = eps;
    std::vector<float> zeros(v_depth ? 0 : (size_t)n, 0.f);
    float *vd = v_depth ? mut(v_depth) : zeros.data();
    for (uint i = 0; i < (uint)n; i++) {
        k_project_bwd(num_points, mut(means), mut(scales), glob_scale, mut(quats), mut(viewmat), mut(projmat),
                      intrins, img_size, mut(radii), mut(conics), mut(v_xy), vd, mut(v_conic), v_mean3d, v_scale,
                      v_quat, degree, use, cp, mut(v_colors), features_dc, features_rest, dc_exp_avg,
                      dc_exp_avg_sq, rest_exp_avg, rest_exp_avg_sq, hp, nan_counts, i);
    }
}

// One Adam group of n elements.
void ref_adam(int n, float *params, const float *grads, float *exp_avg, float *exp_avg_sq, float step_size,
              float beta1, float beta2, float bc2_sqrt, float eps, int group_idx, uint32_t nan_counts[16]) {
    uint un = (uint)n, g = (uint)group_idx;
    for (uint t = 0; t < un; t++)
        k_adam(params, grads, exp_avg, exp_avg_sq, step_size, beta1, beta2, bc2_sqrt, eps, un, nan_counts, g, t);
}

// SGLD noise samples (n x 3) and the covariance-weighted update of the means.
void ref_sgld(int n, float *means, const float *scales, const float *quats, const float *opacities, uint32_t seed,
              float noise_lr, float xyz_lr, float max_disp, float *noise) {
    int N = n;
    uint s = seed;
    for (uint i = 0; i < (uint)n; i++) k_sgld_gen(noise, N, s, i);
    for (uint i = 0; i < (uint)n; i++)
        k_sgld(means, mut(scales), mut(quats), mut(opacities), noise, N, noise_lr, xyz_lr, max_disp, i);
}

// The regularizer's gradient, added to v_opacity [n] and v_scale [n,3].
void ref_reg_grad(int n, const float *opacities, const float *scales, float *v_opacity, float *v_scale,
                  float op_reg, float sc_reg, const int *radii, float invis_scale, const float *dc_exp_avg_sq) {
    int N = n;
    for (uint i = 0; i < (uint)n; i++)
        k_reg(opacities, scales, v_opacity, v_scale, N, op_reg, sc_reg, radii, invis_scale, dc_exp_avg_sq, i);
}

// Tile rectangle of each splat (get_tile_bbox), [x0, y0, x1, y1] per row.
void ref_tile_rect(int n, const float *xys, const float *aabb, int width, int height, int *rect) {
    const int3 tb((width + 15) / 16, (height + 15) / 16, 1);
    for (int i = 0; i < n; i++) {
        uint2 lo, hi;
        get_tile_bbox(float2(xys[2 * i], xys[2 * i + 1]), float2(aabb[2 * i], aabb[2 * i + 1]), tb, lo, hi);
        rect[4 * i] = (int)lo.x;
        rect[4 * i + 1] = (int)lo.y;
        rect[4 * i + 2] = (int)hi.x;
        rect[4 * i + 3] = (int)hi.y;
    }
}

// gaussian_is_active and make_sort_key of each splat.
void ref_sort_keys(int n, const int *radii, const float *depths, uint8_t *active, uint64_t *keys) {
    for (int i = 0; i < n; i++) {
        active[i] = gaussian_is_active((uint)i, mut(radii), mut(depths)) ? 1 : 0;
        keys[i] = make_sort_key(depths[i], (uint)i);
    }
}

// pad_count of each count.
void ref_pad_count(int n, const uint32_t *c, uint32_t *out) {
    for (int i = 0; i < n; i++) out[i] = pad_count(c[i]);
}

// The SSIM window table.
void ref_gauss_1d(float out[11]) {
    for (int i = 0; i < 11; i++) out[i] = GAUSS_1D[i];
}

}  // extern "C"
