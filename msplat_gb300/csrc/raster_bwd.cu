// Back-to-front rasterizer VJP w.r.t. splat centre, conic, raw colour and
// opacity logit.  One CTA per 16x16 tile (chunked: per (tile, chunk)), one
// thread per pixel.  Per splat each warp reduces its pixels' 9 partial
// gradients with a transpose-reduce (9 shuffles for 8 values plus 5 for the
// ninth, instead of 45; paired fp32 adds), warps combine through
// shared-memory adds, and each
// batch flushes one set of three float4 vector atomics per (splat, tile)
// instead of the reference's nine scalar atomics per (splat, warp).  A warp
// skips the splats whose reach box (warp_reach) misses its 8x4 pixel block.
// Follows rasterize_backward_kernel (msplat_metal.metal:931-1135),
// compute_chunk_prefix_suffix_kernel (:3139-3175) and
// rasterize_backward_chunked_kernel (:3179-3366), including its quirk that a
// splat whose alpha was clamped to 0.999 gets no gradient and leaves the
// transmittance unchanged (:1085).  One launch covers the tiles of every
// view of the step; gradients go to the record (view, Gaussian) of each id.
#include "common.cuh"
#include "kernels.h"

namespace msplat {

// kBB splats staged per round (the tile batch: 128 or 256)
template <int kBB> struct BwdSmem {
    float4 xyo[kBB];    // x, y, opacity, id bits
    float4 con[kBB];    // conic, bits of the warps the splat reaches (warp_reach)
    float4 rgb[kBB];    // clamped colour, w: bits of the channels with raw + 0.5 >= 0
    float acc[kBB][9];  // r g b | ca cb cc | x y | opacity
    int wmax[8];
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
    float px, py;
    int bin_final;            // last splat index this pixel may take gradient from (-1: none)
};

// Processes splat indices [s, hi] back to front for the whole CTA.
template <int kBB>
__device__ void backward_range(BwdSmem<kBB> &sm, const RasterArgs &a, int s, int hi, PixelState &ps, GradRec *grad) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wbin = __reduce_max_sync(0xffffffffu, ps.bin_final);
    const float ox = ps.px - (float)tile_px(tid), oy = ps.py - (float)tile_py(tid);
    for (int batch_end = hi; batch_end >= s; batch_end -= kBB) {
        __syncthreads();
        const int idx = batch_end - tid;
        if (tid < kBB) {
            if (idx >= s) {
                const SplatRec r = isect_record(a.isect_ids, a.rec, a.n, idx);
                sm.xyo[tid] = r.a;
                sm.con[tid] = make_float4(r.b.x, r.b.y, r.b.z,
                                          __uint_as_float(warp_reach(r.a.x, r.a.y, r.b.w, r.c.w, ox, oy)));
                // clamped colour max(raw + 0.5, 0); w: channels whose raw + 0.5 >= 0
                // (the only ones that pass a colour gradient back)
                const float cr = r.c.x + 0.5f, cg = r.c.y + 0.5f, cb = r.c.z + 0.5f;
                const int mask = (cr >= 0.f ? 1 : 0) | (cg >= 0.f ? 2 : 0) | (cb >= 0.f ? 4 : 0);
                sm.rgb[tid] = make_float4(fmaxf(cr, 0.f), fmaxf(cg, 0.f), fmaxf(cb, 0.f), __int_as_float(mask));
            }
#pragma unroll
            for (int k = 0; k < 9; k++) sm.acc[tid][k] = 0.f;
        }
        __syncthreads();
        const int nb = min(kBB, batch_end - s + 1);
        for (int t = max(0, batch_end - wbin); t < nb; t++) {
            const float4 cn = sm.con[t];
            if (!((__float_as_uint(cn.w) >> warp) & 1u)) continue;   // no pixel of this warp takes it
            const int sidx = batch_end - t;
            const float4 xo = sm.xyo[t];
            bool valid = sidx <= ps.bin_final;
            float dx = 0.f, dy = 0.f, alpha = 0.f;
            if (valid) {
                // sigma and alpha exactly as the forward pass rounds them (no
                // contraction), so both passes take the same splats
                dx = __fsub_rn(xo.x, ps.px);
                dy = __fsub_rn(xo.y, ps.py);
                const float sigma = __fmaf_rn(0.5f, __fmaf_rn(cn.x, __fmul_rn(dx, dx), __fmul_rn(__fmul_rn(cn.z, dy), dy)),
                                              __fmul_rn(__fmul_rn(cn.y, dx), dy));
                if (!(sigma >= 0.f && sigma < 5.55f)) {   // NaN fails too
                    valid = false;
                } else {
                    alpha = fminf(0.999f, __fmul_rn(xo.z, det_expf_neg(-sigma)));
                    if (alpha < 1.f / 255.f) valid = false;
                }
            }
            if (!__any_sync(0xffffffffu, valid)) continue;
            // per lane, with A = dL/dsigma dx and B = dL/dsigma dy: v[0..2] the
            // colour gradient, v[3..5] = (A dx, A dy, B dy) (half the conic
            // gradient), v[6..7] = (A, B), v8 = dL/dsigma.  The splat's constants
            // are applied once to the sums: conic x 0.5, centre = conic-weighted
            // (A, B), opacity logit -(1 - opacity) x sum(dL/dsigma)
            float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float v8 = 0.f;
            if (valid && alpha < 0.999f) {
                const float4 rc = sm.rgb[t];
                const float ra = __fdividef(1.f, 1.f - alpha);   // fast reciprocal, 1 - alpha in [0.001, 0.997]
                ps.T *= ra;
                const float fac = alpha * ps.T;
                const float cv = __fmaf_rn(rc.x, ps.vr, __fmaf_rn(rc.y, ps.vg, rc.z * ps.vb));
                const float v_alpha = __fmaf_rn(ps.T, cv, -ra * ps.S);
                ps.S = __fmaf_rn(fac, cv, ps.S);
                const float v_sigma = -alpha * v_alpha;
                const float A = v_sigma * dx, B = v_sigma * dy;
                v[0] = fac * ps.vr;
                v[1] = fac * ps.vg;
                v[2] = fac * ps.vb;
                v[3] = A * dx;
                v[4] = A * dy;
                v[5] = B * dy;
                v[6] = A;
                v[7] = B;
                v8 = v_sigma;
            }
            const float s8 = transpose_reduce8(v, v8, lane);
            if ((lane & 3) == 0) atomicAdd(&sm.acc[t][lane >> 2], s8);
            if (lane == 1) atomicAdd(&sm.acc[t][8], v8);
        }
        __syncthreads();
        if (tid < nb) {
            const float *g = sm.acc[tid];
            const int mask = __float_as_int(sm.rgb[tid].w);
            const float gr = (mask & 1) ? g[0] : 0.f;
            const float gg = (mask & 2) ? g[1] : 0.f;
            const float gb = (mask & 4) ? g[2] : 0.f;
            const float4 cn = sm.con[tid];
            const float gop = -(1.f - sm.xyo[tid].z) * g[8];
            const float gx = __fmaf_rn(cn.x, g[6], cn.y * g[7]), gy = __fmaf_rn(cn.y, g[6], cn.z * g[7]);
            const float ca = 0.5f * g[3], cb = 0.5f * g[4], cc = 0.5f * g[5];
            const bool any = (gr != 0.f) | (gg != 0.f) | (gb != 0.f) | (ca != 0.f) | (cb != 0.f) | (cc != 0.f) |
                             (gx != 0.f) | (gy != 0.f) | (gop != 0.f);
            if (any) {
                GradRec *dst = grad + __float_as_int(sm.xyo[tid].w);
                atomic_add_f4(&dst->a, make_float4(gx, gy, gop, 0.f));
                atomic_add_f4(&dst->b, make_float4(ca, cb, cc, 0.f));
                atomic_add_f4(&dst->c, make_float4(gr, gg, gb, 0.f));
            }
        }
    }
}

__device__ __forceinline__ int block_max(int v, int *wmax) {
    const int w = __reduce_max_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = w;
    __syncthreads();
    int m = wmax[0];
#pragma unroll
    for (int k = 1; k < kTileThreads / 32; k++) m = max(m, wmax[k]);
    __syncthreads();
    return m;
}

struct BwdPixel {
    int view, x, y;
    bool inside;
    long long p;   // global pixel index (0 when outside)
};

// kViews: look the view up from the global tile index; false: one view
template <bool kViews> __device__ __forceinline__ BwdPixel bwd_pixel(const RasterArgs &a, int tile) {
    BwdPixel tp;
    tp.view = kViews ? view_of_tile(a.vt, tile) : 0;
    const ViewGeom vg = view_geom(a.vt, tp.view);
    const int lt = tile - vg.tile_base;
    const int tx = lt % vg.tiles_x, ty = lt / vg.tiles_x;
    tp.x = tx * kTile + tile_px(threadIdx.x);
    tp.y = ty * kTile + tile_py(threadIdx.x);
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
    ps.px = (float)tp.x;
    ps.py = (float)tp.y;
}

template <bool kViews, int kBB>
__global__ void __launch_bounds__(kTileThreads) k_raster_bwd(RasterArgs a) {
    pdl_enter();
    __shared__ BwdSmem<kBB> sm;
    const int tile = blockIdx.x + a.tile_lo;
    const int s = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    if (s >= e) return;
    const BwdPixel tp = bwd_pixel<kViews>(a, tile);
    PixelState ps;
    const float Tf = tp.inside ? a.final_T[tp.p] : 0.f;
    init_pixel(ps, a, tp, Tf, 0.f, 0.f, 0.f);
    ps.bin_final = tp.inside ? a.final_idx[tp.p] : -1;
    const int hi = min(e - 1, block_max(ps.bin_final, sm.wmax));
    if (hi < s) return;
    backward_range<kBB>(sm, a, s, hi, ps, a.grad);
}

__global__ void __launch_bounds__(256) k_chunk_prefix_suffix(RasterArgs a) {
    pdl_enter();
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long P = a.vt.pixels;
    if (p >= P) return;
    float pT = 1.f;
    for (int k = 0; k < a.k_max; k++) {
        const size_t o = (size_t)k * P + p;
        a.prefix_T[o] = pT;
        pT *= a.chunk_T[o];
    }
    float r = 0.f, g = 0.f, b = 0.f;
    for (int k = a.k_max - 1; k >= 0; k--) {
        const size_t o = (size_t)k * P + p;
        a.after_C[3 * o] = r;
        a.after_C[3 * o + 1] = g;
        a.after_C[3 * o + 2] = b;
        const float t = a.prefix_T[o];
        r += t * a.chunk_C[3 * o];
        g += t * a.chunk_C[3 * o + 1];
        b += t * a.chunk_C[3 * o + 2];
    }
}

template <bool kViews, int kBB>
__global__ void __launch_bounds__(kTileThreads) k_raster_bwd_chunked(RasterArgs a) {
    pdl_enter();
    __shared__ BwdSmem<kBB> sm;
    const int tile = blockIdx.x + a.tile_lo, k = blockIdx.y;
    const int s0 = clamp_off(a.tile_offsets[tile], a.isect_lo, a.capacity), e0 = clamp_off(a.tile_offsets[tile + 1], a.isect_lo, a.capacity);
    const int cs = s0 + k * a.chunk, ce = min(s0 + (k + 1) * a.chunk, e0);
    if (cs >= ce) return;
    const BwdPixel tp = bwd_pixel<kViews>(a, tile);
    const size_t P = (size_t)a.vt.pixels;
    const size_t o = (size_t)k * P + (size_t)tp.p;
    PixelState ps;
    init_pixel(ps, a, tp, tp.inside ? a.prefix_T[o] * a.chunk_T[o] : 0.f, tp.inside ? a.after_C[3 * o] : 0.f,
               tp.inside ? a.after_C[3 * o + 1] : 0.f, tp.inside ? a.after_C[3 * o + 2] : 0.f);
    const int bf = tp.inside ? a.chunk_idx[o] : -1;
    ps.bin_final = (bf >= cs) ? bf : -1;
    const int hi = min(ce - 1, block_max(ps.bin_final, sm.wmax));
    if (hi < cs) return;
    backward_range<kBB>(sm, a, cs, hi, ps, a.grad);
}

template <int kBB> static void raster_bwd_batch(const RasterArgs &a, cudaStream_t s) {
    const bool views = a.vt.count > 1;
    if (a.k_max <= 1) {
        if (views) launch_pdl(k_raster_bwd<true, kBB>, a.num_tiles, kTileThreads, 0, s, a);
        else launch_pdl(k_raster_bwd<false, kBB>, a.num_tiles, kTileThreads, 0, s, a);
    } else {
        const long long P = a.vt.pixels;
        launch_pdl(k_chunk_prefix_suffix, (unsigned)((P + 255) / 256), 256, 0, s, a);
        if (views) launch_pdl(k_raster_bwd_chunked<true, kBB>, dim3(a.num_tiles, a.k_max), kTileThreads, 0, s, a);
        else launch_pdl(k_raster_bwd_chunked<false, kBB>, dim3(a.num_tiles, a.k_max), kTileThreads, 0, s, a);
    }
}

void launch_raster_bwd(const RasterArgs &a, cudaStream_t s) {
    if (a.batch == 128) raster_bwd_batch<128>(a, s);
    else raster_bwd_batch<256>(a, s);
}

}  // namespace msplat
