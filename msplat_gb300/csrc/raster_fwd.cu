// Front-to-back alpha compositing.  Monolithic: one CTA per 16x16 tile, or
// two (its 16x8 halves, MsplatTuning.tile_split), one thread per pixel,
// splats staged through shared memory in batches of 128 or 256 (each thread
// gathers splat records by the ids in the tile list); a CTA leaves as soon as
// all its pixels have saturated.  Chunked: one CTA per (tile, 512-splat
// depth chunk) with chunk-local transmittance, then a per-pixel merge.
// Follows nd_rasterize_forward_kernel (msplat_metal.metal:499-618),
// rasterize_forward_chunked_kernel (:2960-3076) and
// rasterize_forward_merge_kernel (:3081-3134).  Built with --fmad=false; the
// per-pixel arithmetic is the reference's, fused only where it writes fma(),
// so the image is bit-identical to the oracle's float path.  One launch
// covers the tiles of every view of the step (the view of a CTA is found from
// its global tile index; chunk buffers are [K, pixels of the launch's views]).
#include "common.cuh"
#include "kernels.h"

namespace msplat {

// kSplit CTAs per tile (1, or 2: each a 16x8 half of it, four warps): the
// CTA's threads take places [part * kCtaThreads, (part + 1) * kCtaThreads)
// of the 256-thread tile layout (tile_px / tile_py), so a half is the tile's
// warps 4 part .. 4 part + 3.
template <int kSplit> struct SplitTile {
    static constexpr int kCtaThreads = kTileThreads / kSplit;
    static constexpr int kWarps = kCtaThreads / 32;
};

// kBatch splats staged per round (the tile batch: 128 or 256)
template <int kBatch, int kSplit> struct BatchSmem {
    float4 xyo[kBatch];   // x, y, opacity, sigma_cut(opacity)
    float4 con[kBatch];   // conic
    float4 rgb[kBatch];   // clamped colour max(raw + 0.5, 0)
    uint32_t wm[kBatch];  // bits of this CTA's warps the splat reaches (warp_reach)
    uint16_t wl[SplitTile<kSplit>::kWarps][kBatch];   // per warp: the batch positions it takes, ascending
};

// The positions t < nb of the staged batch whose warp bit is set, written
// ascending to list (one ballot per 32 positions); returns their count.
template <int kBatch>
__device__ __forceinline__ int warp_batch_list(const uint32_t *wm, int nb, int warp, uint16_t *list) {
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    int cnt = 0;
    for (int base = 0; base < nb; base += 32) {
        const int t = base + lane;
        const bool hit = t < nb && ((wm[t] >> warp) & 1u);
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (hit) list[cnt + __popc(m & below)] = (uint16_t)t;
        cnt += __popc(m);
    }
    __syncwarp();
    return cnt;
}

// Splats [b0, min(b0 + kBatch, end)) into the batch; (ox, oy): the tile's
// first pixel; part: the CTA's part of the tile (its warps' reach bits).
template <int kBatch, int kSplit>
__device__ __forceinline__ void load_batch(BatchSmem<kBatch, kSplit> &sm, const RasterArgs &a, int b0, int end,
                                           float ox, float oy, int part) {
    for (int t = threadIdx.x; t < kBatch; t += SplitTile<kSplit>::kCtaThreads) {
        const int idx = b0 + t;
        if (idx >= end) break;
        const SplatRec r = isect_record(a.isect_ids, a.rec, a.n, idx);
        uint32_t reach = warp_reach(r.a.x, r.a.y, r.b.w, r.c.w, ox, oy);
        if (kSplit == 2) reach = (reach >> (4 * part)) & 0xFu;
        sm.xyo[t] = make_float4(r.a.x, r.a.y, r.a.z, sigma_cut(r.a.z));
        sm.wm[t] = reach;
        sm.con[t] = r.b;
        sm.rgb[t] = make_float4(fmaxf(r.c.x + 0.5f, 0.f), fmaxf(r.c.y + 0.5f, 0.f), fmaxf(r.c.z + 0.5f, 0.f), 0.f);
    }
}

// Walks [s, e) for this pixel; the whole CTA iterates together.  A warp
// takes only the splats that can reach its 8x4 block: after each batch is
// staged it lists their positions (ballots over the reach bits) and walks
// that list.
// done: in/out per-thread flag; returns (T, C, last).
template <int kBatch, int kSplit>
__device__ __forceinline__ void composite_range(BatchSmem<kBatch, kSplit> &sm, const RasterArgs &a, int s, int e,
                                                float px, float py, float ox, float oy, int part, bool done, float &T,
                                                float3 &C, int &last, unsigned *nan_sigma) {
    T = 1.f;
    C = make_float3(0.f, 0.f, 0.f);
    last = s - 1;
    const int warp = threadIdx.x >> 5;
    for (int b0 = s; b0 < e; b0 += kBatch) {
        if (__syncthreads_count(done) == SplitTile<kSplit>::kCtaThreads) break;
        load_batch<kBatch, kSplit>(sm, a, b0, e, ox, oy, part);
        __syncthreads();
        const int nb = min(kBatch, e - b0);
        const int cnt = warp_batch_list<kBatch>(sm.wm, nb, warp, sm.wl[warp]);
        if (done) continue;
        for (int i = 0; i < cnt; i++) {
            const int t = sm.wl[warp][i];
            const float4 xo = sm.xyo[t];
            const float4 cn = sm.con[t];
            const float dx = xo.x - px, dy = xo.y - py;
            const float sigma = __fmaf_rn(0.5f, __fmaf_rn(cn.x, dx * dx, cn.z * dy * dy), cn.y * dx * dy);
            if (!(sigma >= 0.f && sigma < 5.55f)) {   // NaN fails too
                if (nan_sigma && !finite_bits(sigma)) atomicAdd(nan_sigma, 1u);
                continue;
            }
            if (sigma > xo.w) continue;   // alpha < 1/255 for certain
            const float alpha = fminf(0.999f, xo.z * det_expf_neg(-sigma));
            if (alpha < 1.f / 255.f) continue;
            const float nT = T * (1.f - alpha);
            if (nT <= 1e-4f) {
                last = b0 + t - 1;
                done = true;
                break;
            }
            const float vis = alpha * T;
            const float4 c = sm.rgb[t];
            C.x = __fmaf_rn(c.x, vis, C.x);
            C.y = __fmaf_rn(c.y, vis, C.y);
            C.z = __fmaf_rn(c.z, vis, C.z);
            T = nT;
            last = b0 + t;
        }
    }
}

__device__ __forceinline__ float sat01(float x) { return fminf(fmaxf(x, 0.f), 1.f); }

// Pixel of this thread in the CTA's tile: view, coordinates, the view's row
// length and first global pixel (the global index is formed where it is
// used, so nothing wider than the coordinates stays live across the walk).
struct TilePixel {
    int view, x, y, width;
    bool inside;
    long long pix_base;
    __device__ __forceinline__ long long p() const { return pix_base + (long long)y * width + x; }
};

// kViews: look the view up from the global tile index; false: one view.
// place: the thread's place in the 256-thread tile layout.
template <bool kViews> __device__ __forceinline__ TilePixel tile_pixel(const RasterArgs &a, int tile, int place) {
    TilePixel tp;
    tp.view = kViews ? view_of_tile(a.vt, tile) : 0;
    const ViewGeom vg = view_geom(a.vt, tp.view);
    const int lt = tile - vg.tile_base;
    const int tx = lt % vg.tiles_x, ty = lt / vg.tiles_x;
    tp.x = tx * kTile + tile_px(place);
    tp.y = ty * kTile + tile_py(place);
    tp.width = vg.width;
    tp.inside = tp.x < vg.width && tp.y < vg.height;
    tp.pix_base = vg.pix_base;
    return tp;
}

template <bool kViews, int kBatch, int kSplit>
__global__ void __launch_bounds__(SplitTile<kSplit>::kCtaThreads, 8 * kSplit) k_raster_fwd(RasterArgs a) {
    pdl_enter();
    __shared__ BatchSmem<kBatch, kSplit> sm;
    const int tile = (kSplit == 1 ? blockIdx.x : blockIdx.x / kSplit) + a.tile_lo;
    const int part = kSplit == 1 ? 0 : blockIdx.x % kSplit;
    const int place = threadIdx.x + part * SplitTile<kSplit>::kCtaThreads;
    const TilePixel tp = tile_pixel<kViews>(a, tile, place);
    int s = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    if (!MS_GUARD(s >= 0 && s <= e && e <= a.capacity, 5, tile, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) e = s = 0;
    float T;
    float3 C;
    int last;
    composite_range(sm, a, s, e, (float)tp.x, (float)tp.y, (float)(tp.x - tile_px(place)),
                    (float)(tp.y - tile_py(place)), part, !tp.inside, T, C, last, nullptr);
    if (!tp.inside) return;
    const long long p = tp.p();
    if (!MS_GUARD(p >= 0 && p < a.vt.pixels, 6, p, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) return;
    const StepParams &sp = a.sp[tp.view];
    a.final_T[p] = T;
    a.final_idx[p] = last;
    a.out_img[3 * p + 0] = sat01(__fmaf_rn(sp.bg[0], T, C.x));
    a.out_img[3 * p + 1] = sat01(__fmaf_rn(sp.bg[1], T, C.y));
    a.out_img[3 * p + 2] = sat01(__fmaf_rn(sp.bg[2], T, C.z));
}

template <bool kViews, int kBatch>
__global__ void __launch_bounds__(kTileThreads, 8) k_raster_fwd_chunked(RasterArgs a) {
    pdl_enter();
    __shared__ BatchSmem<kBatch, 1> sm;
    const int tile = blockIdx.x + a.tile_lo, k = blockIdx.y;
    const TilePixel tp = tile_pixel<kViews>(a, tile, threadIdx.x);
    const int s0 = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e0 = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    const int cs = s0 + k * a.chunk, ce = min(s0 + (k + 1) * a.chunk, e0);
    const size_t o = (size_t)k * (size_t)a.chunk_P + (size_t)(tp.p() - a.chunk_p0);
    if (cs >= ce) {
        if (tp.inside) {
            a.chunk_T[o] = 1.f;
            a.chunk_C[3 * o] = a.chunk_C[3 * o + 1] = a.chunk_C[3 * o + 2] = 0.f;
            a.chunk_idx[o] = -1;
        }
        return;
    }
    float T;
    float3 C;
    int last;
    composite_range(sm, a, cs, ce, (float)tp.x, (float)tp.y, (float)(tp.x - tile_px(threadIdx.x)),
                    (float)(tp.y - tile_py(threadIdx.x)), 0, !tp.inside, T, C, last,
                    a.nan_counts ? a.nan_counts + kNanRasterSigma : nullptr);
    if (!tp.inside) return;
    a.chunk_T[o] = T;
    a.chunk_C[3 * o] = C.x;
    a.chunk_C[3 * o + 1] = C.y;
    a.chunk_C[3 * o + 2] = C.z;
    a.chunk_idx[o] = last;
}

__global__ void __launch_bounds__(256) k_raster_merge(RasterArgs a) {
    pdl_enter();
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // pixel of the launch's views
    const long long P = a.chunk_P;
    if (q >= P) return;
    const long long p = a.chunk_p0 + q;
    float Tr = 1.f, cr = 0.f, cg = 0.f, cb = 0.f;
    int last = -1, cut = a.k_max;
    for (int k = 0; k < a.k_max; k++) {
        const size_t o = (size_t)k * P + q;
        const int cf = a.chunk_idx[o];
        if (cf < 0 && k > 0) break;
        cr = __fmaf_rn(a.chunk_C[3 * o], Tr, cr);
        cg = __fmaf_rn(a.chunk_C[3 * o + 1], Tr, cg);
        cb = __fmaf_rn(a.chunk_C[3 * o + 2], Tr, cb);
        Tr = Tr * a.chunk_T[o];
        if (cf >= 0) last = cf;
        if (Tr <= 1e-4f) { cut = k + 1; break; }
    }
    for (int k = cut; k < a.k_max; k++) a.chunk_idx[(size_t)k * P + q] = -1;
    const StepParams &sp = a.sp[a.vt.count > 1 ? view_of_pixel(a.vt, p) : 0];
    a.final_T[p] = Tr;
    a.final_idx[p] = last;
    a.out_img[3 * p + 0] = sat01(__fmaf_rn(sp.bg[0], Tr, cr));
    a.out_img[3 * p + 1] = sat01(__fmaf_rn(sp.bg[1], Tr, cg));
    a.out_img[3 * p + 2] = sat01(__fmaf_rn(sp.bg[2], Tr, cb));
}

template <int kBatch> static void raster_fwd_batch(const RasterArgs &a, cudaStream_t s) {
    const bool views = a.vt.count > 1;
    if (a.k_max <= 1 && a.split == 2) {
        constexpr int kT = SplitTile<2>::kCtaThreads;
        if (views) launch_pdl(k_raster_fwd<true, kBatch, 2>, 2 * a.num_tiles, kT, 0, s, a);
        else launch_pdl(k_raster_fwd<false, kBatch, 2>, 2 * a.num_tiles, kT, 0, s, a);
    } else if (a.k_max <= 1) {
        if (views) launch_pdl(k_raster_fwd<true, kBatch, 1>, a.num_tiles, kTileThreads, 0, s, a);
        else launch_pdl(k_raster_fwd<false, kBatch, 1>, a.num_tiles, kTileThreads, 0, s, a);
    } else {
        if (views) launch_pdl(k_raster_fwd_chunked<true, kBatch>, dim3(a.num_tiles, a.k_max), kTileThreads, 0, s, a);
        else launch_pdl(k_raster_fwd_chunked<false, kBatch>, dim3(a.num_tiles, a.k_max), kTileThreads, 0, s, a);
        launch_pdl(k_raster_merge, (unsigned)((a.chunk_P + 255) / 256), 256, 0, s, a);
    }
}

void launch_raster_fwd(const RasterArgs &a, cudaStream_t s) {
    if (a.batch == 128) raster_fwd_batch<128>(a, s);
    else raster_fwd_batch<256>(a, s);
}

}  // namespace msplat
