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

namespace mshim {
ExpFn g_expf = nullptr;
GroupState *g_group = nullptr;
thread_local int t_lane = 0, t_sg = 0;
thread_local unsigned t_simd_op = 0;
std::mutex &atomic_lock() {
    static std::mutex m;
    return m;
}
}  // namespace mshim

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

// count_intersections_kernel (msplat_metal.metal:2342-2365)
void k_count(float *xys, int *radii, float *depths, uint3 &tile_bounds, atomic_uint *tile_counts, uint &num_points,
             float *aabb, uint gid) {
#include "k_count_intersections_kernel.inc"
}

// scatter_intersections_kernel (msplat_metal.metal:2440-2480)
void k_scatter(float *xys, float *depths, int *radii, uint3 &tile_bounds, uint *sort_offsets,
               atomic_uint *tile_write_counters, uint64_t *isect_keys_unsorted, uint &num_points, float *aabb,
               uint &capacity, uint2 &tile_range, uint gid) {
#include "k_scatter_intersections_kernel.inc"
}

// Kernels below keep per-threadgroup arrays: `threadgroup` storage becomes a
// function static, shared by the host threads of the group being run.
#undef threadgroup
#define threadgroup static

// prefix_sum_tiles_kernel (msplat_metal.metal:2376-2433)
void k_prefix_sum_tiles(uint *tile_counts_in, uint *exact_offsets, uint *sort_offsets, int *tile_bins,
                        uint &num_tiles, uint &capacity, uint2 &tile_range, uint tid) {
#include "k_prefix_sum_tiles_kernel.inc"
}

// hybrid_sort_pack_kernel (msplat_metal.metal:2489-2627)
void k_sort_pack(uint *tile_counts_in, uint *sort_offsets, uint *exact_offsets, uint64_t *isect_keys_unsorted,
                 float *xys_in, float *conics_in, float *opacities_in, float *colors_in, float *packed_xy_opac,
                 float *packed_conic, float *packed_rgb, int *gaussian_ids, uint &capacity, uint &num_points,
                 atomic_uint *nan_counts, uint2 &tile_range, uint &key_capacity, uint tg_id, uint tid) {
#include "k_hybrid_sort_pack_kernel.inc"
}

// nd_rasterize_forward_kernel (msplat_metal.metal:499-618)
void k_raster_fwd(uint3 &tile_bounds, uint3 &img_size, uint &channels, int *tile_bins, float *packed_xy_opac,
                  float *packed_conic, float *packed_rgb, float *final_Ts, int *final_index, float *out_img,
                  float *background, uint2 &blockDim, uint2 &tile_range, uint2 blockIdx, uint2 threadIdx, uint tr) {
#include "k_nd_rasterize_forward_kernel.inc"
}

// rasterize_backward_kernel (msplat_metal.metal:931-1135)
void k_raster_bwd(uint3 &tile_bounds, uint2 &img_size, int32_t *gaussian_ids_sorted, int *tile_bins,
                  float *packed_xy_opac, float *packed_conic, float *packed_rgb, float *background, float *final_Ts,
                  int *final_index, float *v_output, atomic_float *v_xy, atomic_float *v_conic, atomic_float *v_rgb,
                  atomic_float *v_opacity, uint2 &tile_range, uint3 gp, uint3 blockIdx, uint tr, uint warp_size,
                  uint wr) {
#include "k_rasterize_backward_kernel.inc"
}

// rasterize_forward_chunked_kernel (msplat_metal.metal:2960-3076)
void k_raster_fwd_chunked(uint3 &tile_bounds, uint3 &img_size, uint &channels, int *tile_bins, float *packed_xy_opac,
                          float *packed_conic, float *packed_rgb, float *chunk_T, float *chunk_C, int *chunk_final_idx,
                          uint &chunk_size, uint &K_max, uint2 &blockDim, atomic_uint *nan_counts, uint3 blockIdx,
                          uint tr) {
#include "k_rasterize_forward_chunked_kernel.inc"
}

// rasterize_backward_chunked_kernel (msplat_metal.metal:3179-3366)
void k_raster_bwd_chunked(uint3 &tile_bounds, uint2 &img_size, int32_t *gaussian_ids_sorted, int *tile_bins,
                          float *packed_xy_opac, float *packed_conic, float *packed_rgb, float *background,
                          float *final_Ts, int *chunk_final_idx, float *prefix_T_buf, float *chunk_T_buf,
                          float *after_C_buf, float *v_output, atomic_float *v_xy, atomic_float *v_conic,
                          atomic_float *v_rgb, atomic_float *v_opacity, uint &chunk_size, uint &K_max, uint3 gp,
                          uint3 blockIdx, uint tr, uint warp_size, uint wr) {
#include "k_rasterize_backward_chunked_kernel.inc"
}

// rasterize_forward_merge_kernel (msplat_metal.metal:3081-3134)
void k_raster_merge(uint &num_pixels, uint &K_max, float *chunk_T, float *chunk_C, int *chunk_final_idx,
                    float *final_Ts, int *final_index, float *out_img, float *background, uint2 &img_size, uint2 gp) {
#include "k_rasterize_forward_merge_kernel.inc"
}

// ssim_h_fwd_kernel (msplat_metal.metal:3388-3450)
void k_ssim_h_fwd(float *rendered, uchar *gt, uint2 &img_size, float *ssim_h_buf, uint2 gid, uint2 lid, uint tr,
                  uint2 tgid) {
#include "k_ssim_h_fwd_kernel.inc"
}

// ssim_fused_v_fwd_h_bwd_kernel (msplat_metal.metal:3563-3681)
void k_ssim_fused(float *rendered, uchar *gt, float *ssim_h_buf, uint2 &img_size, float &ssim_weight, float &inv_n,
                  float *deriv_h_buf, atomic_float *loss_sum, atomic_uint *nan_counts, uchar *mask, int &has_mask,
                  uint2 gid, uint2 lid, uint tr, uint2 tgid, uint2 tg_size) {
#include "k_ssim_fused_v_fwd_h_bwd_kernel.inc"
}

// ssim_v_bwd_kernel (msplat_metal.metal:3764-3850)
void k_ssim_v_bwd(float *rendered, uchar *gt, float *ssim_h_buf, uint2 &img_size, float &ssim_weight, float &inv_n,
                  float *v_rendered, atomic_uint *nan_counts, uchar *mask, int &has_mask, uint2 gid, uint2 lid,
                  uint tr, uint2 tgid) {
#include "k_ssim_v_bwd_kernel.inc"
}

#undef threadgroup
#define threadgroup

// compute_chunk_prefix_suffix_kernel (msplat_metal.metal:3139-3175)
void k_chunk_prefix_suffix(uint &num_pixels, uint &K_max, float *chunk_T, float *chunk_C, int *chunk_final_idx,
                           float *prefix_T, float *after_C, uint2 &img_size, uint2 gp) {
#include "k_compute_chunk_prefix_suffix_kernel.inc"
}

// Whether rasterize_backward_chunked_kernel is defined on these inputs: in
// every (8x8 threadgroup, chunk) either every lane returns at its early exit
// (empty chunk, pixel outside the image, or no contributor in the chunk:
// .metal:3242-3247) or none does; otherwise lanes that returned would miss
// the group's barriers and the SIMD-group broadcasts from lane 0.
bool chunked_backward_defined(uint W, uint H, uint tiles_x, const int *bins, const int *chunk_final_idx, uint K,
                              uint chunk) {
    const uint P = W * H;
    for (uint k = 0; k < K; k++)
        for (uint by = 0; by < (H + 7) / 8; by++)
            for (uint bx = 0; bx < (W + 7) / 8; bx++) {
                const uint tile = (by * 8 / 16) * tiles_x + (bx * 8 / 16);
                const int cs = bins[2 * tile] + (int)(k * chunk);
                const int ce = std::min(bins[2 * tile] + (int)((k + 1) * chunk), bins[2 * tile + 1]);
                if (cs >= ce) continue;   // the whole group returns
                int ret = 0;
                for (uint ty = 0; ty < 8; ty++)
                    for (uint tx = 0; tx < 8; tx++) {
                        const uint i = by * 8 + ty, j = bx * 8 + tx;
                        const bool inside = i < H && j < W;
                        const uint pix = std::min(i * W + j, P - 1);
                        const int bin_final = inside ? chunk_final_idx[(size_t)k * P + pix] : -1;
                        ret += bin_final < cs ? 1 : 0;
                    }
                if (ret != 0 && ret != 64) return false;
            }
    return true;
}

// Runs a grid of gx x gy threadgroups of bx x by threads: one host thread
// per GPU thread, the groups one after another, a barrier between groups.
// body(group x, group y, thread x, thread y, thread index).
template <class F> void run_groups(int gx, int gy, int bx, int by, F body) {
    const int T = bx * by;
    mshim::GroupState gs;
    gs.bar.n = T;
    for (auto &sg : gs.sg) sg.bar.n = 32;
    mshim::g_group = &gs;
    mshim::HostBarrier end;
    end.n = T;
    std::vector<mshim::HostThread> threads;
    threads.reserve(T);
    for (int t = 0; t < T; t++)
        threads.emplace_back([&, t]() {
            mshim::t_lane = t % 32;
            mshim::t_sg = t / 32;
            mshim::t_simd_op = 0;
            for (int y = 0; y < gy; y++)
                for (int x = 0; x < gx; x++) {
                    body(x, y, t % bx, t / bx, t);
                    end.wait();
                }
        });
    for (auto &th : threads) th.join();
    mshim::g_group = nullptr;
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

// The pixel stages of one training step of one view, as the reference runs
// them (msplat_metal.mm:1255-1400), every stage a compiled kernel: count,
// tile scan, scatter, per-tile sort + pack (one 1024-thread threadgroup per
// tile), the forward rasterizer, monolithic (k_max <= 1) or chunked in k_max
// chunks of chunk_size splats with the merge (the caller applies the
// reference's K rule, msplat_metal.mm:1204-1224), the three SSIM + L1
// kernels when gt is given (else v_rendered is an input) and the backward
// rasterizer (the chunked one where it is defined).
// Capacity: ids/packing sized by the exact count; returns the intersection
// count, or -1 when more than ids_capacity.
long long ref_raster_step(int n, const float *xys, const float *depths, const int *radii, const float *conics,
                          const float *colors, const float *aabb, const float *opacities, int width, int height,
                          const float background[3], const uint8_t *gt, const uint8_t *mask, float ssim_weight,
                          float loss_inv_n, int *tile_bins_out, int *gaussian_ids, long long ids_capacity,
                          float *out_img, float *final_Ts, int *final_idx, float *loss_sum, float *v_rendered,
                          float *v_xy, float *v_conic, float *v_colors, float *v_opacity, uint32_t nan_counts[16],
                          int k_max, int chunk_size, int *backward_ran) {
    const uint W = (uint)width, H = (uint)height;
    uint3 tile_bounds((W + 15) / 16, (H + 15) / 16, 1u);
    const uint T = tile_bounds.x * tile_bounds.y;
    uint np = (uint)n;
    // count_intersections_kernel
    std::vector<uint> counts(T, 0u);
    for (uint i = 0; i < np; i++)
        k_count(mut(xys), mut(radii), mut(depths), tile_bounds, counts.data(), np, mut(aabb), i);
    // prefix_sum_tiles_kernel: one 1024-thread threadgroup; padded offsets for
    // the sort buckets, exact ones and the [start, end) bins for the lists
    std::vector<uint> sort_off(T + 1, 0u), exact(T, 0u);
    std::vector<int> bins(2 * (size_t)T);
    uint2 all(0u, T);
    {
        uint nt = T, cap_any = 0xffffffffu;
        run_groups(1, 1, 1024, 1, [&](int, int, int, int, int t) {
            k_prefix_sum_tiles(counts.data(), exact.data(), sort_off.data(), bins.data(), nt, cap_any, all, (uint)t);
        });
    }
    const long long M = T ? (long long)bins[2 * (T - 1) + 1] : 0;
    if (M > ids_capacity) return -1;
    // scatter_intersections_kernel (one tile group covering every tile)
    uint cap = sort_off[T];
    std::vector<uint64_t> keys(std::max<uint>(cap, 1u), ~0ull);
    std::vector<uint> wc(T, 0u);
    for (uint i = 0; i < np; i++)
        k_scatter(mut(xys), mut(depths), mut(radii), tile_bounds, sort_off.data(), wc.data(), keys.data(), np,
                  mut(aabb), cap, all, i);
    // hybrid_sort_pack_kernel: one 1024-thread threadgroup per tile
    std::vector<float> pk_xyo(3 * (size_t)std::max<long long>(M, 1)), pk_con(pk_xyo.size()), pk_rgb(pk_xyo.size());
    {
        uint out_cap = (uint)std::max<long long>(M, 1), key_cap = std::max<uint>(cap, 1u);
        run_groups((int)T, 1, 1024, 1, [&](int bx, int, int, int, int t) {
            k_sort_pack(counts.data(), sort_off.data(), exact.data(), keys.data(), mut(xys), mut(conics),
                        mut(opacities), mut(colors), pk_xyo.data(), pk_con.data(), pk_rgb.data(), gaussian_ids,
                        out_cap, np, nan_counts, all, key_cap, (uint)bx, (uint)t);
        });
    }
    if (tile_bins_out) std::copy(bins.begin(), bins.end(), tile_bins_out);
    // forward rasterizer: 8x8 threadgroups
    uint3 img3(W, H, 1u);
    uint channels = 3;
    uint2 block(8u, 8u);
    float bg[3] = {background[0], background[1], background[2]};
    const int gx = (int)((W + 7) / 8), gy = (int)((H + 7) / 8);
    const uint P = W * H;
    uint K = (uint)std::max(1, k_max), chunk = (uint)std::max(1, chunk_size);
    std::vector<float> cT, cC;
    std::vector<int> cI;
    if (K <= 1) {
        run_groups(gx, gy, 8, 8, [&](int bx, int by, int tx, int ty, int t) {
            k_raster_fwd(tile_bounds, img3, channels, bins.data(), pk_xyo.data(), pk_con.data(), pk_rgb.data(),
                         final_Ts, final_idx, out_img, bg, block, all, uint2((uint)bx, (uint)by),
                         uint2((uint)tx, (uint)ty), (uint)t);
        });
    } else {
        // chunked (msplat_metal.mm:1285-1307): one grid layer per chunk, then the merge per pixel
        cT.assign((size_t)K * P, 1.f);
        cC.assign((size_t)K * P * 3, 0.f);
        cI.assign((size_t)K * P, -1);
        for (uint k = 0; k < K; k++)
            run_groups(gx, gy, 8, 8, [&](int bx, int by, int, int, int t) {
                k_raster_fwd_chunked(tile_bounds, img3, channels, bins.data(), pk_xyo.data(), pk_con.data(),
                                     pk_rgb.data(), cT.data(), cC.data(), cI.data(), chunk, K, block, nan_counts,
                                     uint3((uint)bx, (uint)by, k), (uint)t);
            });
        uint2 isz2(W, H);
        uint npx = P;
        for (uint y = 0; y < H; y++)
            for (uint x = 0; x < W; x++)
                k_raster_merge(npx, K, cT.data(), cC.data(), cI.data(), final_Ts, final_idx, out_img, bg, isz2,
                               uint2(x, y));
    }
    uint2 isz(W, H);
    if (gt) {
        // the loss: three kernels over 16x16 threadgroups
        std::vector<float> hbuf((size_t)W * H * 15, 0.f), dbuf((size_t)W * H * 15, 0.f);
        float sw = ssim_weight, invn = loss_inv_n;
        int has_mask = mask ? 1 : 0;
        uchar *gt8 = mut(gt), *m8 = mut(mask);
        *loss_sum = 0.f;
        const int sx = (int)((W + 15) / 16), sy = (int)((H + 15) / 16);
        run_groups(sx, sy, 16, 16, [&](int bx, int by, int tx, int ty, int t) {
            k_ssim_h_fwd(out_img, gt8, isz, hbuf.data(), uint2(bx * 16 + tx, by * 16 + ty), uint2(tx, ty), t,
                         uint2(bx, by));
        });
        run_groups(sx, sy, 16, 16, [&](int bx, int by, int tx, int ty, int t) {
            k_ssim_fused(out_img, gt8, hbuf.data(), isz, sw, invn, dbuf.data(), loss_sum, nan_counts, m8, has_mask,
                         uint2(bx * 16 + tx, by * 16 + ty), uint2(tx, ty), t, uint2(bx, by), uint2(16u, 16u));
        });
        run_groups(sx, sy, 16, 16, [&](int bx, int by, int tx, int ty, int t) {
            k_ssim_v_bwd(out_img, gt8, dbuf.data(), isz, sw, invn, v_rendered, nan_counts, m8, has_mask,
                         uint2(bx * 16 + tx, by * 16 + ty), uint2(tx, ty), t, uint2(bx, by));
        });
    }
    // backward rasterizer: 8x8 threadgroups of two SIMD groups
    std::fill(v_xy, v_xy + 2 * (size_t)n, 0.f);
    std::fill(v_conic, v_conic + 3 * (size_t)n, 0.f);
    std::fill(v_colors, v_colors + 3 * (size_t)n, 0.f);
    std::fill(v_opacity, v_opacity + (size_t)n, 0.f);
    std::vector<int> gids(gaussian_ids, gaussian_ids + std::max<long long>(M, 1));
    if (backward_ran) *backward_ran = 0;
    if (K <= 1) {
        run_groups(gx, gy, 8, 8, [&](int bx, int by, int tx, int ty, int t) {
            k_raster_bwd(tile_bounds, isz, gids.data(), bins.data(), pk_xyo.data(), pk_con.data(), pk_rgb.data(), bg,
                         final_Ts, final_idx, v_rendered, v_xy, v_conic, v_colors, v_opacity, all,
                         uint3((uint)(bx * 8 + tx), (uint)(by * 8 + ty), 0u), uint3((uint)bx, (uint)by, 0u), (uint)t,
                         32u, (uint)(t % 32));
        });
        if (backward_ran) *backward_ran = 1;
    } else if (chunked_backward_defined(W, H, tile_bounds.x, bins.data(), cI.data(), K, chunk)) {
        // chunked (msplat_metal.mm:1370-1400): prefix transmittance and suffix
        // colour per pixel, then one grid layer of 8x8 threadgroups per chunk
        std::vector<float> pT((size_t)K * P, 0.f), aC((size_t)K * P * 3, 0.f);
        uint npx = P, KK = K;
        for (uint y = 0; y < H; y++)
            for (uint x = 0; x < W; x++)
                k_chunk_prefix_suffix(npx, KK, cT.data(), cC.data(), cI.data(), pT.data(), aC.data(), isz, uint2(x, y));
        for (uint k = 0; k < K; k++)
            run_groups(gx, gy, 8, 8, [&](int bx, int by, int tx, int ty, int t) {
                k_raster_bwd_chunked(tile_bounds, isz, gids.data(), bins.data(), pk_xyo.data(), pk_con.data(),
                                     pk_rgb.data(), bg, final_Ts, cI.data(), pT.data(), cT.data(), aC.data(),
                                     v_rendered, v_xy, v_conic, v_colors, v_opacity, chunk, KK,
                                     uint3((uint)(bx * 8 + tx), (uint)(by * 8 + ty), k), uint3((uint)bx, (uint)by, k),
                                     (uint)t, 32u, (uint)(t % 32));
            });
        if (backward_ran) *backward_ran = 1;
    }
    // Otherwise (a chunked forward whose backward is undefined on these
    // inputs) the gradients stay zero and backward_ran says so.
    return M;
}

// The SSIM window table.
void ref_gauss_1d(float out[11]) {
    for (int i = 0; i < 11; i++) out[i] = GAUSS_1D[i];
}

}  // extern "C"
