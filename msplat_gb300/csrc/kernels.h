// Kernel argument blocks and launchers of the msplat GB300 engine (internal).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"
#include "mlp.h"

namespace msplat {

// Table of `count` views (sizes w[v] x h[v]) over n Gaussians.
inline ViewTable make_view_table(int n, int count, const int *w, const int *h) {
    ViewTable vt{};
    vt.count = count;
    vt.n = n;
    for (int v = 0; v < count; v++) {
        vt.width[v] = w[v];
        vt.height[v] = h[v];
        vt.tiles_x[v] = (w[v] + kTile - 1) / kTile;
        vt.tiles_y[v] = (h[v] + kTile - 1) / kTile;
        vt.tile_base[v + 1] = vt.tile_base[v] + vt.tiles_x[v] * vt.tiles_y[v];
        vt.pix_base[v + 1] = vt.pix_base[v] + (long long)w[v] * h[v];
    }
    for (int v = count; v < kMaxViews; v++) {   // past the end: empty views at the end of the ranges
        vt.tile_base[v + 1] = vt.tile_base[v];
        vt.pix_base[v + 1] = vt.pix_base[v];
    }
    vt.tiles = vt.tile_base[count];
    vt.pixels = vt.pix_base[count];
    return vt;
}
inline ViewTable single_view_table(int n, int w, int h) { return make_view_table(n, 1, &w, &h); }

// Block-aggregated tile mapping: a CTA of kAggThreads covers kAggPerCta
// Gaussians of one view; used while every view has at most kAggMaxTiles tiles.
// The depth-presorted ordering's radix sort: kGsBits-bit digits in
// kGsPasses passes over the 32-bit key, kGsPerCta keys per block.  Three
// 11-bit passes over 4096-key blocks give the same lists but measured
// slower at 1M Gaussians (tile stage 0.250 -> 0.268 ms, 8 views 1.90 ->
// 2.12 ms): the 2048-digit histograms, scans and ranking cost more than the
// pass they save.
constexpr int kGsBits = 8;
constexpr int kGsDigits = 1 << kGsBits;
constexpr int kGsPasses = (32 + kGsBits - 1) / kGsBits;
constexpr int kGsPerCta = kGsBits == 8 ? 1024 : 4096;
constexpr int kAggShift = 10;
constexpr int kAggPerCta = 1 << kAggShift;   // Gaussians per count / scatter CTA
constexpr int kAggThreads = 512;      // count / scatter CTA width (256 measured slower)
constexpr int kAggMaxTiles = 20480;   // 80 KB of histogram: two 512-thread CTAs per SM at the largest

inline int max_view_tiles(const ViewTable &vt) {
    int m = 0;
    for (int v = 0; v < vt.count; v++) m = vt.tiles_x[v] * vt.tiles_y[v] > m ? vt.tiles_x[v] * vt.tiles_y[v] : m;
    return m;
}

// Record arrays (rec, depths, radii, aabb, tiles_hit, grad) are [views, n]
// (see ViewTable); the parameters are read once per view.
struct ProjectArgs {
    ViewTable vt;
    int rest_bases;
    const float *means, *scales, *quats, *features_dc, *features_rest, *opacities;
    const StepParams *sp;   // [views]
    SplatRec *rec;
    float *depths;
    int *radii;
    float2 *aabb;
    int *tiles_hit;
    ushort4 *rect;          // tile rectangle (x0, y0, x1, y1) where radii > 0 (nullable)
    GradRec *grad;          // zeroed here (nullable)
    unsigned *nan_counts;   // nullable
};

struct TileArgs {
    ViewTable vt;
    int num_tiles;          // over all views
    int sort_width;         // CTA width of the lightest shared-memory sort class: 256 or 512
    // tile group being built (fixed intersection budget): tiles [tile_lo,
    // tile_hi) only, their intersections stored from global slot isect_lo on
    // (the whole range and 0 when the view fits)
    int tile_lo, tile_hi;
    long long isect_lo;
    long long capacity;     // intersection slots of keys / isect_ids (held from isect_lo on)
    const int *radii;
    const float *depths;
    const SplatRec *rec;
    const float2 *aabb;
    uint32_t *tile_counts;  // zeroed before the step
    uint32_t *tile_write;   // zeroed before the step
    uint32_t *cta_bins;     // per view: [ceil(n / kAggPerCta), T_v] per-CTA tile histograms (block-aggregated path)
    uint32_t *tile_lists;   // [4, T] tiles of each sort class (written by the scan)
    uint32_t *tile_class;   // [8]: list lengths, then the sort kernels' work counters
    uint32_t *tile_offsets; // [T+1]
    uint32_t *max_tile_count;
    uint64_t *keys, *keys_alt;
    uint32_t *isect_ids;    // per-tile sorted Gaussian ids (0xffffffff: transparent)
    unsigned *nan_counts;
    // depth-presorted ordering (block-aggregated path only): one stable
    // radix sort of each view's Gaussians by depth, the count and scatter in
    // that order, then each tile's per-CTA runs put in order
    int presorted;
    uint32_t *gs_key[2], *gs_val[2];   // [views, n] sort buffers; ids in depth order end in gs_val[kGsPasses & 1]
    uint32_t *gs_hist;                 // [views, kGsDigits, ceil(n / kGsPerCta)] digit counts, then offsets
    uint32_t *gs_dtot;                 // [views, kGsDigits] keys per digit
    const ushort4 *rect;               // [views, n] tile rectangles from the projection
    ushort4 *srect;                    // [views, n] tile rectangles in depth order
};

struct RasterArgs {
    ViewTable vt;
    int num_tiles, k_max;       // tiles of this launch; depth chunks of its views (1 = monolithic)
    int tile_lo;                // first global tile of this launch (tile group), 0 otherwise
    long long isect_lo;         // global intersection slot held at isect_ids[0]
    int chunk;                  // splats per depth chunk (chunked raster)
    int batch;                  // splats staged per shared-memory round: 128 or 256
    int bwd_px;                 // pixels per thread of the backward: 1 (256 threads) or 2 (128)
    int split;                  // CTAs per tile of the monolithic rasterizers: 1, or 2 (16x8 halves)
    long long capacity;
    const StepParams *sp;       // [views]
    const uint32_t *tile_offsets;
    uint32_t n;                 // records, views * Gaussians (ids at or past n read as transparent)
    const uint32_t *isect_ids;  // per-tile sorted Gaussian ids
    const SplatRec *rec;        // projection records, gathered by id
    float *out_img, *final_T;
    int *final_idx;
    // chunked raster: this launch's chunk buffers hold the pixels
    // [chunk_p0, chunk_p0 + chunk_P) of its views, entry (k, p) at
    // k * chunk_P + p - chunk_p0
    float *chunk_T, *chunk_C, *prefix_T, *after_C;
    int *chunk_idx;
    long long chunk_p0, chunk_P;
    const float *v_img;
    GradRec *grad;
    unsigned *nan_counts;
};

struct LossArgs {
    ViewTable vt;
    const StepParams *sp;   // [views]
    const float *img;
    const uint8_t *gt, *mask;   // one view: override StepParams' target and mask (nullable)
    float *v_img;           // [P, 3]
    float *loss_sum;        // [views]
    unsigned *nan_counts;
};

struct ProjectBwdArgs {
    ViewTable vt;
    int rest_bases, do_optimizer;
    const StepParams *sp;   // [views]; the optimizer scalars are view 0's
    const float *means, *scales, *quats;
    const int *radii;       // [views, n]
    const SplatRec *rec;    // [views, n]
    const GradRec *grad;    // [views, n]
    float *v_mean, *v_scale, *v_quat;   // [n]: summed over the views
    float *v_opac;          // [n] summed opacity-logit gradient (several views; Adam reads it)
    float4 *sh_in;          // [n] one view: colour gradient and whether it feeds the SH walk (scratch)
    float *features_dc, *features_rest, *dc_m, *dc_v, *rest_m, *rest_v;
    // gradient export (one view, no optimizer): when set, the SH gradients
    // and the opacity-logit gradient are written here instead of feeding Adam
    float *v_dc_out, *v_rest_out, *v_opac_out;
    // per-Gaussian activity statistics for the learned relocation proposal
    // (or null): per view x += |dL/d(pixel centre)| and y += 1 when visible;
    // z += 1 per step
    float4 *gstats;
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
// Tile mapping in two halves: counting + scans (all tiles), then the build
// (scatter + per-tile sorts) of the tiles [tile_lo, tile_hi); launch_tiles
// runs both.  Each returns its kernel launches.
int launch_tile_count(const TileArgs &a, cudaStream_t s);
int launch_tile_build(const TileArgs &a, int num_sms, cudaStream_t s);
int launch_tiles(const TileArgs &a, int num_sms, cudaStream_t s);
// the depth-presorted ordering (depth_order.cu): sort + rectangles + count,
// then the column and tile scans (tiles.cu); and its build
int launch_presorted_count(const TileArgs &a, cudaStream_t s);
int launch_tile_scans(const TileArgs &a, cudaStream_t s);
int launch_presorted_build(const TileArgs &a, cudaStream_t s);
size_t sort_pack_smem_bytes();
// cta_bins bytes for these views, 0 when the block-aggregated path is not used
size_t tile_cta_bins_bytes(const ViewTable &vt);
void launch_raster_fwd(const RasterArgs &a, cudaStream_t s);
// returns the kernels launched (0 or 1), or -1 when the per-device set-up
// (window upload, shared-memory limit) failed; nothing is launched then
int launch_loss(const LossArgs &a, cudaStream_t s);
void launch_raster_bwd(const RasterArgs &a, cudaStream_t s);
void launch_project_bwd(const ProjectBwdArgs &a, cudaStream_t s);
void launch_adam(const AdamArgs &a, int num_sms, cudaStream_t s);
void launch_sgld(const AdamArgs &a, cudaStream_t s);
void run_mcmc(McmcArgs a, int cap_max, int &relocation_count, McmcResult &res, cudaStream_t s);

}  // namespace msplat
