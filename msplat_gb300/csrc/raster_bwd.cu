// Back-to-front rasterizer VJP w.r.t. splat centre, conic, raw colour and
// opacity logit.  One CTA per 16x16 tile (chunked: per (tile, chunk)), in one
// of the layouts below (MsplatTuning.bwd_pixels, tile_split): one pixel per
// thread, 256 threads, each warp an 8x4 block, or the same split into two
// 128-thread CTAs per tile (16x8 halves); or two pixels per thread (four
// rows apart), 128 threads, each warp an 8x8 block, so one warp reduction
// serves 64 pixels (fewer reductions, more work per CTA).  Per splat each warp
// reduces its pixels' 9 partial gradients with a transpose-reduce (9
// shuffles for 8 values plus 5 for the ninth, instead of 45; paired fp32
// adds), warps combine through shared-memory adds, and each batch flushes one
// set of three float4 vector atomics per (splat, tile) instead of the
// reference's nine scalar atomics per (splat, warp).  A warp takes only the
// splats whose reach box meets its block: after each batch is staged it
// lists their positions (one ballot per 32) and walks that list.
// Follows rasterize_backward_kernel (msplat_metal.metal:931-1135),
// compute_chunk_prefix_suffix_kernel (:3139-3175) and
// rasterize_backward_chunked_kernel (:3179-3366), including its quirk that a
// splat whose alpha was clamped to 0.999 gets no gradient and leaves the
// transmittance unchanged (:1085).  One launch covers the tiles of every
// view of the step; gradients go to the record (view, Gaussian) of each id.
#include "common.cuh"
#include "kernels.h"

namespace msplat {

// Thread layouts, by CTA and pixel:
//   1: one CTA per tile, 256 threads, one pixel each; warp w covers the 8x4
//      block of tile_px / tile_py.
//   2: one CTA per tile, 128 threads, two pixels each; warp w covers x in
//      [8(w&1), 8(w&1)+8), y in [8(w>>1), 8(w>>1)+8); the thread's column
//      is lane & 7, its rows (lane >> 3) and (lane >> 3) + 4.
//   3: two CTAs per tile (MsplatTuning.tile_split), 128 threads, one pixel
//      each: CTA `part` is the tile's 16x8 half covered by layout 1's warps
//      4 part .. 4 part + 3.
// A thread's place is its index in the tile's layout-1 numbering
// (threadIdx.x + 128 part in layout 3, threadIdx.x otherwise).
template <int kL> struct BwdLayout;
template <> struct BwdLayout<1> {
    static constexpr int kThreads = 256, kPix = 1, kSplit = 1;
    static __device__ __forceinline__ int px(int place) { return tile_px(place); }
    static __device__ __forceinline__ int py(int place) { return tile_py(place); }
    static __device__ __forceinline__ uint32_t reach(float x, float y, float hx, float hy, float ox, float oy, int) {
        return warp_reach(x, y, hx, hy, ox, oy);
    }
};
template <> struct BwdLayout<3> {
    static constexpr int kThreads = 128, kPix = 1, kSplit = 2;
    static __device__ __forceinline__ int px(int place) { return tile_px(place); }
    static __device__ __forceinline__ int py(int place) { return tile_py(place); }
    static __device__ __forceinline__ uint32_t reach(float x, float y, float hx, float hy, float ox, float oy,
                                                     int part) {
        return (warp_reach(x, y, hx, hy, ox, oy) >> (4 * part)) & 0xFu;
    }
};
template <> struct BwdLayout<2> {
    static constexpr int kThreads = 128, kPix = 2, kSplit = 1;
    static __device__ __forceinline__ int px(int tid) { return (tid & 7) | ((tid >> 2) & 8); }
    static __device__ __forceinline__ int py(int tid) { return (tid >> 3) & 11; }
    // warp_reach for the 8x8 blocks: bit w when block w meets the splat's
    // reach box (the same conservative margins)
    static __device__ __forceinline__ uint32_t reach(float x, float y, float hx, float hy, float ox, float oy, int) {
        if (!(hx <= 3.0e38f && hy <= 3.0e38f)) return 0xFu;
        if (hx < 0.f || hy < 0.f) return 0u;
        const float lx = x - ox, ly = y - oy;
        const float rx = hx + 0.02f + 1e-6f * (fabsf(lx) + hx + fabsf(ox));
        const float ry = hy + 0.02f + 1e-6f * (fabsf(ly) + hy + fabsf(oy));
        const float x0 = lx - rx, x1 = lx + rx, y0 = ly - ry, y1 = ly + ry;
        const uint32_t cols = (x1 >= 0.f && x0 <= 7.f ? 0x5u : 0u) | (x1 >= 8.f && x0 <= 15.f ? 0xAu : 0u);
        const uint32_t rows = (y1 >= 0.f && y0 <= 7.f ? 0x3u : 0u) | (y1 >= 8.f && y0 <= 15.f ? 0xCu : 0u);
        return cols & rows;
    }
};

// kBB splats staged per round (the tile batch: 128 or 256)
template <int kBB, int kL> struct BwdSmem {
    float4 xyo[kBB];    // x, y, opacity, id bits
    float4 con[kBB];    // conic, sigma_cut(opacity)
    float4 rgb[kBB];    // clamped colour, w: bits of the channels with raw + 0.5 >= 0
    float acc[kBB][9];  // r g b | ca cb cc | x y | opacity
    uint32_t wm[kBB];   // bits of the warps the splat reaches
    uint16_t wl[BwdLayout<kL>::kThreads / 32][kBB];   // per warp: the batch positions it takes, ascending
    int wmax[BwdLayout<kL>::kThreads / 32];
};

// Sums over the warp of 8 per-lane values v[] and of one more value w: lane
// 4*j ends with the total of v[j] (returned), every lane with the total of
// w (in w).  A transpose-reduce: at each of the first three levels a lane
// keeps half of its values and sends the other half, so 7 shuffles reduce
// 8 values; the additions run on paired fp32 arithmetic where two are
// independent (the same IEEE sums, half the instructions).
__device__ __forceinline__ float transpose_reduce8(float v[8], float &w, int lane) {
    const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4;
    float2 keep[2], recv[2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float s0 = b16 ? v[2 * h] : v[2 * h + 4], s1 = b16 ? v[2 * h + 1] : v[2 * h + 5];
        keep[h] = make_float2(b16 ? v[2 * h + 4] : v[2 * h], b16 ? v[2 * h + 5] : v[2 * h + 1]);
        recv[h] = make_float2(__shfl_xor_sync(0xffffffffu, s0, 16), __shfl_xor_sync(0xffffffffu, s1, 16));
    }
    const float2 v01 = __fadd2_rn(keep[0], recv[0]), v23 = __fadd2_rn(keep[1], recv[1]);
    // level 8: pairs (0, 2) and (1, 3)
    const float t0 = b8 ? v01.x : v23.x, t1 = b8 ? v01.y : v23.y;
    const float2 k8 = make_float2(b8 ? v23.x : v01.x, b8 ? v23.y : v01.y);
    const float2 r8 = make_float2(__shfl_xor_sync(0xffffffffu, t0, 8), __shfl_xor_sync(0xffffffffu, t1, 8));
    const float2 u = __fadd2_rn(k8, r8);
    // level 4: one value per lane from here, reduced together with w
    const float send = b4 ? u.x : u.y;
    float2 x = make_float2(b4 ? u.y : u.x, w);
    w += __shfl_xor_sync(0xffffffffu, w, 16);
    w += __shfl_xor_sync(0xffffffffu, w, 8);
    x = make_float2(x.x + __shfl_xor_sync(0xffffffffu, send, 4), w + __shfl_xor_sync(0xffffffffu, w, 4));
    x = __fadd2_rn(x, make_float2(__shfl_xor_sync(0xffffffffu, x.x, 2), __shfl_xor_sync(0xffffffffu, x.y, 2)));
    x = __fadd2_rn(x, make_float2(__shfl_xor_sync(0xffffffffu, x.x, 1), __shfl_xor_sync(0xffffffffu, x.y, 1)));
    w = x.y;
    return x.x;
}

// Per-pixel state of the back-to-front walk.  The reference keeps the colour
// behind the splat per channel (buffer) and T_final * background; both only
// enter dL/dalpha through their dot product with dL/dpixel, so the walk keeps
// that one number: S = (buffer + T_final * background) . dL/dpixel, updated
// by fac * (colour . dL/dpixel) per splat.
struct PixelState {
    float T;                  // transmittance in front of the current splat
    float S;                  // (colour behind + T_final * background) . dL/dpixel
    float vr, vg, vb;         // dL/dpixel
    float py;                 // row (the column is shared by the thread's pixels)
    int bin_final;            // last splat index this pixel may take gradient from (-1: none)
};

// One pixel's part of a splat it takes: its transmittance and S updates and
// its gradient contributions in v, v8 (an alpha clamped to 0.999 is skipped
// here).  kAdd: add to v (the thread's second pixel), else assign (its first).
template <bool kAdd>
__device__ __forceinline__ void pixel_step(PixelState &ps, float dx, float dy, float alpha, const float4 &rc,
                                           float v[8], float &v8) {
    if (!(alpha < 0.999f)) return;
    const float ra = __fdividef(1.f, 1.f - alpha);   // fast reciprocal, 1 - alpha in [0.001, 0.997]
    ps.T *= ra;
    const float fac = alpha * ps.T;
    const float cv = __fmaf_rn(rc.x, ps.vr, __fmaf_rn(rc.y, ps.vg, rc.z * ps.vb));
    const float v_alpha = __fmaf_rn(ps.T, cv, -ra * ps.S);
    ps.S = __fmaf_rn(fac, cv, ps.S);
    const float v_sigma = -alpha * v_alpha;
    const float A = v_sigma * dx, B = v_sigma * dy;
    const float c[9] = {fac * ps.vr, fac * ps.vg, fac * ps.vb, A * dx, A * dy, B * dy, A, B, v_sigma};
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = kAdd ? v[k] + c[k] : c[k];
    v8 = kAdd ? v8 + c[8] : c[8];
}

// sigma exactly as the forward pass rounds it (no contraction) and alpha from
// the hardware exponential (__expf: documented within 2 + floor(1.173 |x|)
// ulp, so 8 ulp or 1e-6 relative for x = -sigma in (-5.55, 0]); with the
// forward's det_expf (2 ulp) and the product's rounding the two alphas differ
// by less than 1.5e-6 relative.  Where this alpha lies within 4e-6 relative
// of a decision the forward takes (alpha >= 1/255, the 0.999 clamp), alpha is
// recomputed with the forward's own exponential, so both passes take the same
// splats and clamp the same ones; elsewhere the difference only enters the
// gradients and the transmittance reconstruction.  false when the pixel does
// not take the splat.
__device__ __forceinline__ bool splat_alpha(const float4 &xo, const float4 &cn, float dx, float dy, float &alpha) {
    const float sigma = __fmaf_rn(0.5f, __fmaf_rn(cn.x, __fmul_rn(dx, dx), __fmul_rn(__fmul_rn(cn.z, dy), dy)),
                                  __fmul_rn(__fmul_rn(cn.y, dx), dy));
    if (!(sigma >= 0.f && sigma < 5.55f)) return false;   // NaN fails too
    if (sigma > cn.w) return false;                        // alpha < 1/255 for certain
    float a = __fmul_rn(xo.z, __expf(-sigma));
    if (fabsf(a - 1.f / 255.f) <= 4e-6f * (1.f / 255.f) || fabsf(a - 0.999f) <= 4e-6f)
        a = __fmul_rn(xo.z, det_expf_neg(-sigma));
    alpha = fminf(0.999f, a);
    return !(alpha < 1.f / 255.f);
}

// Processes splat indices [s, hi] back to front for the whole CTA; px is
// the thread's column, ps its pixels; place / part: as in BwdLayout.
template <int kBB, int kL>
__device__ void backward_range(BwdSmem<kBB, kL> &sm, const RasterArgs &a, int s, int hi,
                               PixelState (&ps)[BwdLayout<kL>::kPix], float px, int place, int part, GradRec *grad) {
    using L = BwdLayout<kL>;
    constexpr int kPx = L::kPix;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int bmax = ps[0].bin_final;
#pragma unroll
    for (int r = 1; r < kPx; r++) bmax = max(bmax, ps[r].bin_final);
    const int wbin = __reduce_max_sync(0xffffffffu, bmax);
    const float ox = px - (float)L::px(place), oy = ps[0].py - (float)L::py(place);   // the tile's first pixel
    for (int batch_end = hi; batch_end >= s; batch_end -= kBB) {
        __syncthreads();
        for (int k = tid; k < kBB; k += L::kThreads) {
            const int idx = batch_end - k;
            if (idx >= s) {
                const SplatRec r = isect_record(a.isect_ids, a.rec, a.n, idx);
                sm.xyo[k] = r.a;
                const uint32_t reach = L::reach(r.a.x, r.a.y, r.b.w, r.c.w, ox, oy, part);
                sm.con[k] = make_float4(r.b.x, r.b.y, r.b.z, sigma_cut(r.a.z));
                sm.wm[k] = reach;
                // clamped colour max(raw + 0.5, 0); w: channels whose raw + 0.5 >= 0
                // (the only ones that pass a colour gradient back)
                const float cr = r.c.x + 0.5f, cg = r.c.y + 0.5f, cb = r.c.z + 0.5f;
                const int mask = (cr >= 0.f ? 1 : 0) | (cg >= 0.f ? 2 : 0) | (cb >= 0.f ? 4 : 0);
                sm.rgb[k] = make_float4(fmaxf(cr, 0.f), fmaxf(cg, 0.f), fmaxf(cb, 0.f), __int_as_float(mask));
            }
#pragma unroll
            for (int j = 0; j < 9; j++) sm.acc[k][j] = 0.f;
        }
        __syncthreads();
        const int nb = min(kBB, batch_end - s + 1);
        // the positions from t0 on whose splat can reach this warp's pixels
        // (ascending: back to front), listed with one ballot per 32
        const int t0 = max(0, batch_end - wbin);
        int cnt = 0;
        {
            const unsigned below = (1u << lane) - 1u;
            for (int base = t0; base < nb; base += 32) {
                const int t = base + lane;
                const bool hit = t < nb && ((sm.wm[t] >> warp) & 1u);
                const unsigned m = __ballot_sync(0xffffffffu, hit);
                if (hit) sm.wl[warp][cnt + __popc(m & below)] = (uint16_t)t;
                cnt += __popc(m);
            }
            __syncwarp();
        }
        for (int i = 0; i < cnt; i++) {
            const int t = sm.wl[warp][i];
            const float4 cn = sm.con[t];
            const int sidx = batch_end - t;
            const float4 xo = sm.xyo[t];
            const float dx = __fsub_rn(xo.x, px);
            float dy[kPx], al[kPx];
            bool on[kPx], any_on = false;
#pragma unroll
            for (int r = 0; r < kPx; r++) {
                dy[r] = __fsub_rn(xo.y, ps[r].py);
                al[r] = 0.f;
                on[r] = sidx <= ps[r].bin_final && splat_alpha(xo, cn, dx, dy[r], al[r]);
                any_on |= on[r];
            }
            if (!__any_sync(0xffffffffu, any_on)) continue;
            // per lane, with A = dL/dsigma dx and B = dL/dsigma dy: v[0..2] the
            // colour gradient, v[3..5] = (A dx, A dy, B dy) (half the conic
            // gradient), v[6..7] = (A, B), v8 = dL/dsigma, both pixels summed.
            // The splat's constants are applied once to the sums: conic x 0.5,
            // centre = conic-weighted (A, B), opacity logit -(1 - opacity) x
            // sum(dL/dsigma)
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float v8 = 0.f;
            const float4 rc = sm.rgb[t];
            if (on[0]) pixel_step<false>(ps[0], dx, dy[0], al[0], rc, v, v8);
#pragma unroll
            for (int r = 1; r < kPx; r++)
                if (on[r]) pixel_step<true>(ps[r], dx, dy[r], al[r], rc, v, v8);
            const float s8 = transpose_reduce8(v, v8, lane);
            if ((lane & 3) == 0) atomicAdd(&sm.acc[t][lane >> 2], s8);
            if (lane == 1) atomicAdd(&sm.acc[t][8], v8);
        }
        __syncthreads();
        for (int k = tid; k < nb; k += L::kThreads) {
            const float *g = sm.acc[k];
            const int mask = __float_as_int(sm.rgb[k].w);
            const float gr = (mask & 1) ? g[0] : 0.f;
            const float gg = (mask & 2) ? g[1] : 0.f;
            const float gb = (mask & 4) ? g[2] : 0.f;
            const float4 cn = sm.con[k];
            const float gop = -(1.f - sm.xyo[k].z) * g[8];
            const float gx = __fmaf_rn(cn.x, g[6], cn.y * g[7]), gy = __fmaf_rn(cn.y, g[6], cn.z * g[7]);
            const float ca = 0.5f * g[3], cb = 0.5f * g[4], cc = 0.5f * g[5];
            const bool any = (gr != 0.f) | (gg != 0.f) | (gb != 0.f) | (ca != 0.f) | (cb != 0.f) | (cc != 0.f) |
                             (gx != 0.f) | (gy != 0.f) | (gop != 0.f);
            if (any) {
                GradRec *dst = grad + __float_as_int(sm.xyo[k].w);
                atomic_add_f4(&dst->a, make_float4(gx, gy, gop, 0.f));
                atomic_add_f4(&dst->b, make_float4(ca, cb, cc, 0.f));
                atomic_add_f4(&dst->c, make_float4(gr, gg, gb, 0.f));
            }
        }
    }
}

template <int kWarps> __device__ __forceinline__ int block_max(int v, int *wmax) {
    const int w = __reduce_max_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = w;
    __syncthreads();
    int m = wmax[0];
#pragma unroll
    for (int k = 1; k < kWarps; k++) m = max(m, wmax[k]);
    __syncthreads();
    return m;
}

struct BwdPixel {
    int view, x, y;
    bool inside;
    long long p;   // global pixel index (0 when outside)
};

// kViews: look the view up from the global tile index; false: one view
// row: the thread's r-th pixel (4 r rows down)
template <bool kViews, int kL>
__device__ __forceinline__ BwdPixel bwd_pixel(const RasterArgs &a, int tile, int row, int place) {
    BwdPixel tp;
    tp.view = kViews ? view_of_tile(a.vt, tile) : 0;
    const ViewGeom vg = view_geom(a.vt, tp.view);
    const int lt = tile - vg.tile_base;
    const int tx = lt % vg.tiles_x, ty = lt / vg.tiles_x;
    tp.x = tx * kTile + BwdLayout<kL>::px(place);
    tp.y = ty * kTile + BwdLayout<kL>::py(place) + 4 * row;
    tp.inside = tp.x < vg.width && tp.y < vg.height;
    tp.p = tp.inside ? vg.pix_base + (long long)tp.y * vg.width + tp.x : 0;
    return tp;
}

// S at the back of the walk: (colour behind + T_final * background) . dL/dpixel
__device__ __forceinline__ void init_pixel(PixelState &ps, const RasterArgs &a, const BwdPixel &tp, float T0,
                                           float behind_r, float behind_g, float behind_b) {
    const StepParams &sp = a.sp[tp.view];
    const long long p = tp.p;
    const float Tf = tp.inside ? a.final_T[p] : 0.f;
    ps.T = T0;
    ps.vr = tp.inside ? a.v_img[3 * p] : 0.f;
    ps.vg = tp.inside ? a.v_img[3 * p + 1] : 0.f;
    ps.vb = tp.inside ? a.v_img[3 * p + 2] : 0.f;
    ps.S = (behind_r + Tf * sp.bg[0]) * ps.vr + (behind_g + Tf * sp.bg[1]) * ps.vg + (behind_b + Tf * sp.bg[2]) * ps.vb;
    ps.py = (float)tp.y;
}

// blocks per SM each layout is built for (registers and shared memory)
template <int kL> constexpr int bwd_min_blocks() { return kL == 1 ? 6 : (kL == 2 ? 8 : 12); }

template <bool kViews, int kBB, int kL>
__global__ void __launch_bounds__(BwdLayout<kL>::kThreads, bwd_min_blocks<kL>()) k_raster_bwd(RasterArgs a) {
    pdl_enter();
    using L = BwdLayout<kL>;
    constexpr int kPx = L::kPix;
    __shared__ BwdSmem<kBB, kL> sm;
    const int tile = (L::kSplit == 1 ? blockIdx.x : blockIdx.x / L::kSplit) + a.tile_lo;
    const int part = L::kSplit == 1 ? 0 : blockIdx.x % L::kSplit;
    const int place = threadIdx.x + part * L::kThreads;
    const int s = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    if (s >= e) return;
    PixelState ps[kPx];
    float px = 0.f;
    int bmax = -1;
#pragma unroll
    for (int r = 0; r < kPx; r++) {
        const BwdPixel tp = bwd_pixel<kViews, kL>(a, tile, r, place);
        const float Tf = tp.inside ? a.final_T[tp.p] : 0.f;
        init_pixel(ps[r], a, tp, Tf, 0.f, 0.f, 0.f);
        ps[r].bin_final = tp.inside ? a.final_idx[tp.p] : -1;
        bmax = max(bmax, ps[r].bin_final);
        px = (float)tp.x;
    }
    const int hi = min(e - 1, block_max<L::kThreads / 32>(bmax, sm.wmax));
    if (hi < s) return;
    backward_range<kBB, kL>(sm, a, s, hi, ps, px, place, part, a.grad);
}

__global__ void __launch_bounds__(256) k_chunk_prefix_suffix(RasterArgs a) {
    pdl_enter();
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // pixel of the launch's views
    const long long P = a.chunk_P;
    if (q >= P) return;
    float pT = 1.f;
    for (int k = 0; k < a.k_max; k++) {
        const size_t o = (size_t)k * P + q;
        a.prefix_T[o] = pT;
        pT *= a.chunk_T[o];
    }
    float r = 0.f, g = 0.f, b = 0.f;
    for (int k = a.k_max - 1; k >= 0; k--) {
        const size_t o = (size_t)k * P + q;
        a.after_C[3 * o] = r;
        a.after_C[3 * o + 1] = g;
        a.after_C[3 * o + 2] = b;
        const float t = a.prefix_T[o];
        r += t * a.chunk_C[3 * o];
        g += t * a.chunk_C[3 * o + 1];
        b += t * a.chunk_C[3 * o + 2];
    }
}

template <bool kViews, int kBB, int kL>
__global__ void __launch_bounds__(BwdLayout<kL>::kThreads, bwd_min_blocks<kL>()) k_raster_bwd_chunked(RasterArgs a) {
    pdl_enter();
    constexpr int kPx = BwdLayout<kL>::kPix;
    __shared__ BwdSmem<kBB, kL> sm;
    const int tile = blockIdx.x + a.tile_lo, k = blockIdx.y;
    const int s0 = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e0 = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    const int cs = s0 + k * a.chunk, ce = min(s0 + (k + 1) * a.chunk, e0);
    if (cs >= ce) return;
    const size_t P = (size_t)a.chunk_P;
    PixelState ps[kPx];
    float px = 0.f;
    int bmax = -1;
#pragma unroll
    for (int r = 0; r < kPx; r++) {
        const BwdPixel tp = bwd_pixel<kViews, kL>(a, tile, r, threadIdx.x);
        const size_t o = (size_t)k * P + (size_t)(tp.p - a.chunk_p0);
        init_pixel(ps[r], a, tp, tp.inside ? a.prefix_T[o] * a.chunk_T[o] : 0.f, tp.inside ? a.after_C[3 * o] : 0.f,
                   tp.inside ? a.after_C[3 * o + 1] : 0.f, tp.inside ? a.after_C[3 * o + 2] : 0.f);
        const int bf = tp.inside ? a.chunk_idx[o] : -1;
        ps[r].bin_final = (bf >= cs) ? bf : -1;
        bmax = max(bmax, ps[r].bin_final);
        px = (float)tp.x;
    }
    const int hi = min(ce - 1, block_max<BwdLayout<kL>::kThreads / 32>(bmax, sm.wmax));
    if (hi < cs) return;
    backward_range<kBB, kL>(sm, a, cs, hi, ps, px, threadIdx.x, 0, a.grad);
}

template <int kBB, int kL> static void raster_bwd_batch(const RasterArgs &a, cudaStream_t s) {
    const bool views = a.vt.count > 1;
    constexpr int kT = BwdLayout<kL>::kThreads;
    if (a.k_max <= 1) {
        // monolithic: one pixel per thread takes the tuned CTAs per tile
        if (kL == 1 && a.split == 2) {
            constexpr int kT3 = BwdLayout<3>::kThreads;
            if (views) launch_pdl(k_raster_bwd<true, kBB, 3>, 2 * a.num_tiles, kT3, 0, s, a);
            else launch_pdl(k_raster_bwd<false, kBB, 3>, 2 * a.num_tiles, kT3, 0, s, a);
        } else {
            if (views) launch_pdl(k_raster_bwd<true, kBB, kL>, a.num_tiles, kT, 0, s, a);
            else launch_pdl(k_raster_bwd<false, kBB, kL>, a.num_tiles, kT, 0, s, a);
        }
    } else {
        launch_pdl(k_chunk_prefix_suffix, (unsigned)((a.chunk_P + 255) / 256), 256, 0, s, a);
        if (views) launch_pdl(k_raster_bwd_chunked<true, kBB, kL>, dim3(a.num_tiles, a.k_max), kT, 0, s, a);
        else launch_pdl(k_raster_bwd_chunked<false, kBB, kL>, dim3(a.num_tiles, a.k_max), kT, 0, s, a);
    }
}

void launch_raster_bwd(const RasterArgs &a, cudaStream_t s) {
    if (a.bwd_px == 2) {
        if (a.batch == 128) raster_bwd_batch<128, 2>(a, s);
        else raster_bwd_batch<256, 2>(a, s);
    } else {
        if (a.batch == 128) raster_bwd_batch<128, 1>(a, s);
        else raster_bwd_batch<256, 1>(a, s);
    }
}

}  // namespace msplat
