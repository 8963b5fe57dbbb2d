// Kernel argument blocks and launchers of the msplat GB300 engine (internal).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mlp.h"

namespace msplat {

struct ProjectArgs {
    int n, rest_bases, tiles_x, tiles_y;
    float Wf, Hf;
    const float *means, *scales, *quats, *features_dc, *features_rest, *opacities;
    const StepParams *sp;
    SplatRec *rec;
    float *depths;
    int *radii;
    float2 *aabb;
    int *tiles_hit;
    GradRec *grad;          // zeroed here (nullable)
    unsigned *nan_counts;   // nullable
};

struct TileArgs {
    int n, tiles_x, tiles_y, num_tiles;
    long long capacity;     // intersection slots of keys / isect_ids
    const int *radii;
    const float *depths;
    const SplatRec *rec;
    const float2 *aabb;
    uint32_t *tile_counts;  // zeroed before the step
    uint32_t *tile_write;   // zeroed before the step
    uint32_t *cta_bins;     // [ceil(n / 2048), T] per-CTA tile histograms (block-aggregated path)
    uint32_t *tile_lists;   // [3, T] tiles of each sort class (written by the scan)
    uint32_t *tile_class;   // [6]: list lengths, then the sort kernels' work counters
    uint32_t *tile_offsets; // [T+1]
    uint32_t *max_tile_count;
    uint64_t *keys, *keys_alt;
    uint32_t *isect_ids;    // per-tile sorted Gaussian ids (0xffffffff: transparent)
    unsigned *nan_counts;
};

struct RasterArgs {
    int width, height, tiles_x, num_tiles, k_max;
    long long capacity;
    const StepParams *sp;
    const uint32_t *tile_offsets;
    int n;                      // Gaussians (ids at or past n read as transparent)
    const uint32_t *isect_ids;  // per-tile sorted Gaussian ids
    const SplatRec *rec;        // projection records, gathered by id
    float *out_img, *final_T;
    int *final_idx;
    float *chunk_T, *chunk_C, *prefix_T, *after_C;
    int *chunk_idx;
    const float *v_img;
    GradRec *grad;
    unsigned *nan_counts;
};

struct LossArgs {
    int width, height;
    const StepParams *sp;
    const float *img;
    const uint8_t *gt, *mask;
    float *hbuf;            // [15, P] channel-planar moments
    float *dbuf;            // [9, P] horizontally convolved fields
    float *v_img;           // [P, 3]
    float *loss_sum;
    unsigned *nan_counts;
};

struct ProjectBwdArgs {
    int n, rest_bases, do_optimizer;
    float Wf, Hf;
    const StepParams *sp;
    const float *means, *scales, *quats;
    const int *radii;
    const SplatRec *rec;
    const GradRec *grad;
    float *v_mean, *v_scale, *v_quat;
    float *features_dc, *features_rest, *dc_m, *dc_v, *rest_m, *rest_v;
    // gradient export (no optimizer): when set, the SH gradients and the
    // opacity-logit gradient are written here instead of feeding Adam
    float *v_dc_out, *v_rest_out, *v_opac_out;
    // per-Gaussian activity statistics for the learned relocation proposal
    // (or null): x += |dL/d(pixel centre)| and y += 1 when visible, z += 1
    float4 *gstats;
    // multi-view accumulation (no optimizer): v_mean / v_scale / v_quat and
    // the buffers below are added to for the Gaussians visible in this view
    int accumulate;
    float *acc_opac, *acc_dc, *acc_rest;   // [N], [N,3], [N,rest,3]
    uint8_t *acc_vis;                      // 1 once visible in any view
    unsigned *nan_counts;
};

struct AdamArgs {
    int n;
    const StepParams *sp;
    float *means, *scales, *quats, *opacities;
    float *m[4], *v[4];          // moments of means, scales, quats, opacity
    const float *g_mean, *g_scale, *g_quat;
    const GradRec *grad;         // opacity gradient in grad[i].a.z
    const float *dc_v;           // features_dc second moment (regularizer duty)
    const float *g_opac;         // opacity gradient [N] in place of grad[i].a.z, or null
    unsigned *nan_counts;
};

// Adam on the SH groups from accumulated gradients (multi-view steps): the
// elements of Gaussians visible in at least one view, bands below
// degrees_to_use (the fused per-view SH Adam's rule over the union)
struct ShAdamArgs {
    int n, rest_bases;
    const StepParams *sp;
    float *features_dc, *features_rest, *dc_m, *dc_v, *rest_m, *rest_v;
    const float *acc_dc, *acc_rest;
    const uint8_t *acc_vis;
    unsigned *nan_counts;
};

struct McmcArgs {
    int n, rest_bases;
    float *means, *scales, *quats, *features_dc, *features_rest, *opacities;
    float *exp_avg[6], *exp_avg_sq[6];
    float cull_r2;
    uint32_t *flags, *flag_pos, *upart, *copies;
    double *weights, *cumw, *dpart;
    int *dead_list, *moves;
    unsigned *counters;
    const float *score;   // sampling weight per Gaussian in place of sigmoid(opacity), or null
    float4 *gstats;       // activity statistics, cleared for every slot that receives a copy, or null
};

struct McmcResult {
    int num_dead, num_culled, num_nonfinite, num_relocated, num_grown, num_active;
};

// With MSPLAT_SYNC_CHECK set in the environment, waits for the stream after
// each launch and raises with the kernel's name if it failed.
void debug_sync(cudaStream_t s, const char *what);

void launch_project_fwd(const ProjectArgs &a, cudaStream_t s);
int launch_tiles(const TileArgs &a, int num_sms, cudaStream_t s);

   // returns the kernel launches
size_t sort_pack_smem_bytes();
size_t tile_cta_bins_bytes(int n, int num_tiles);   // 0 when the block-aggregated path is not used
void launch_raster_fwd(const RasterArgs &a, cudaStream_t s);
void launch_loss(const LossArgs &a, cudaStream_t s);
void launch_raster_bwd(const RasterArgs &a, cudaStream_t s);
void launch_project_bwd(const ProjectBwdArgs &a, cudaStream_t s);
void launch_adam(const AdamArgs &a, int num_sms, cudaStream_t s);
void launch_sgld(const AdamArgs &a, cudaStream_t s);
void launch_sh_adam(const ShAdamArgs &a, cudaStream_t s);
void run_mcmc(McmcArgs a, int cap_max, int &relocation_count, McmcResult &res, cudaStream_t s);

}  // namespace msplat
