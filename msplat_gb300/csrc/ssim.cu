// Training loss L = w * (1 - mean SSIM) + (1 - w) * mean |x - gt| and its
// image gradient, as three separable passes over 16x16 pixel tiles:
//   1. horizontal 11-tap moments of (gt, x, gt^2, x^2, gt*x), zero padding
//   2. vertical moments -> SSIM, L1, loss sum and the derivative fields
//      (f1, f2, f3), then the horizontal transpose convolution of the fields
//   3. vertical transpose convolution -> dL/dx
// Follows ssim_h_fwd_kernel, ssim_fused_v_fwd_h_bwd_kernel and
// ssim_v_bwd_kernel (msplat_metal.metal:3388-3450, 3563-3681, 3764-3850),
// including their treatment of window centres in the out-of-image columns a
// border tile reaches (fields from zero moments).  Intermediates are stored
// channel-planar so every tile load and store is coalesced.  The 16x16 blocks
// are the tiles: one launch per pass covers every view of the step (the
// rendered image, the planes and dL/dx are indexed by global pixel, each
// view's target and mask by its own pixel).
#include "common.cuh"
#include "kernels.h"

namespace msplat {

__constant__ float kGauss[11];
constexpr float kC1 = 0.0001f, kC2 = 0.0009f;
constexpr int kS = 16, kHalo = 5, kSpan = kS + 2 * kHalo;   // 26

// Target and mask: the arguments' when set (one view), else the view's in StepParams.
__device__ __forceinline__ const uint8_t *step_gt(const LossArgs &a, int v) { return a.gt ? a.gt : a.sp[v].gt; }
__device__ __forceinline__ const uint8_t *step_mask(const LossArgs &a, int v) { return a.gt ? a.mask : a.sp[v].mask; }

// The CTA's block: view, geometry, block origin (pixels).  kViews: the grid
// is the global tile range of several views; false: one view, a 2D grid of
// its blocks, geometry straight from the parameter bank.
struct LossBlock {
    int view, W, H, x0, y0;
    long long pb;   // global index of the view's pixel 0
};
template <bool kViews> __device__ __forceinline__ LossBlock loss_block(const LossArgs &a) {
    LossBlock b;
    if (!kViews) {
        b.view = 0;
        b.W = a.vt.width[0];
        b.H = a.vt.height[0];
        b.x0 = blockIdx.x * kS;
        b.y0 = blockIdx.y * kS;
        b.pb = 0;
        return b;
    }
    const int tile = blockIdx.x;
    b.view = view_of_tile(a.vt, tile);
    const ViewGeom vg = view_geom(a.vt, b.view);
    const int lt = tile - vg.tile_base;
    b.W = vg.width;
    b.H = vg.height;
    b.x0 = (lt % vg.tiles_x) * kS;
    b.y0 = (lt / vg.tiles_x) * kS;
    b.pb = vg.pix_base;
    return b;
}

template <bool kViews>
__global__ void __launch_bounds__(256) k_ssim_h(LossArgs a) {
    __shared__ float sg[3][kS][kSpan], sr[3][kS][kSpan];
    const LossBlock lb = loss_block<kViews>(a);
    const uint8_t *gt = step_gt(a, lb.view);
    const int W = lb.W, H = lb.H;
    const int bx = lb.x0 - kHalo, by = lb.y0;
    const int tid = threadIdx.x;
    for (int i = tid; i < kS * kSpan; i += 256) {
        const int sy = i / kSpan, sx = i % kSpan;
        const int gy = by + sy, gx = bx + sx;
        const bool in = gx >= 0 && gx < W && gy < H;
        const size_t p = in ? ((size_t)gy * W + gx) : 0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            sg[c][sy][sx] = in ? (float)gt[3 * p + c] * (1.0f / 255.0f) : 0.f;
            sr[c][sy][sx] = in ? a.img[3 * (lb.pb + p) + c] : 0.f;
        }
    }
    __syncthreads();
    const int lx = tid & 15, ly = tid >> 4;
    const int x = lb.x0 + lx, y = by + ly;
    if (x >= W || y >= H) return;
    const size_t P = (size_t)a.vt.pixels, p = lb.pb + (size_t)y * W + x;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float mx = 0.f, my = 0.f, sx = 0.f, sy = 0.f, cr = 0.f;
#pragma unroll
        for (int d = 0; d < 11; d++) {
            const float w = kGauss[d], g = sg[c][ly][lx + d], r = sr[c][ly][lx + d];
            mx += w * g; my += w * r; sx += w * g * g; sy += w * r * r; cr += w * g * r;
        }
        a.hbuf[(c * 5 + 0) * P + p] = mx;
        a.hbuf[(c * 5 + 1) * P + p] = my;
        a.hbuf[(c * 5 + 2) * P + p] = sx;
        a.hbuf[(c * 5 + 3) * P + p] = sy;
        a.hbuf[(c * 5 + 4) * P + p] = cr;
    }
}

template <bool kViews>
__global__ void __launch_bounds__(256, 6) k_ssim_fields(LossArgs a) {
    __shared__ float hp[5][kSpan][kSpan];
    __shared__ float mv[5][kS][kSpan];   // vertical moments at the window centres
    __shared__ float fl[3][kS][kSpan];
    __shared__ float red[8];
    const LossBlock lb = loss_block<kViews>(a);
    const int W = lb.W, H = lb.H;
    const size_t P = (size_t)a.vt.pixels;
    const int bx = lb.x0 - kHalo, by = lb.y0 - kHalo;
    const int tid = threadIdx.x, lx = tid & 15, ly = tid >> 4;
    const StepParams &sp = a.sp[lb.view];
    const uint8_t *gt = step_gt(a, lb.view), *mask = step_mask(a, lb.view);
    const float sw = sp.ssim_weight;
    float ssim_acc = 0.f, l1_acc = 0.f;
    unsigned nwin = 0;
    for (int c = 0; c < 3; c++) {
        for (int i = tid; i < kSpan * kSpan; i += 256) {
            const int sy = i / kSpan, sx = i % kSpan;
            const int gy = by + sy, gx = bx + sx;
            const bool in = gx >= 0 && gx < W && gy >= 0 && gy < H;
            const size_t p = in ? lb.pb + ((size_t)gy * W + gx) : 0;
#pragma unroll
            for (int f = 0; f < 5; f++) hp[f][sy][sx] = in ? a.hbuf[(c * 5 + f) * P + p] : 0.f;
        }
        __syncthreads();
        // vertical 11-tap pass, one (moment, column) per thread: the 26 inputs
        // of the column are read once into registers for all 16 outputs
        if (tid < 5 * kSpan) {
            const int f = tid / kSpan, fx = tid % kSpan;
            float col[kSpan];
#pragma unroll
            for (int r = 0; r < kSpan; r++) col[r] = hp[f][r][fx];
#pragma unroll
            for (int fy = 0; fy < kS; fy++) {
                float acc = 0.f;
#pragma unroll
                for (int k = 0; k < 11; k++) acc += kGauss[k] * col[fy + k];
                mv[f][fy][fx] = acc;
            }
        }
        __syncthreads();
        for (int i = tid; i < kS * kSpan; i += 256) {
            const int fy = i / kSpan, fx = i % kSpan;     // field row (output rows), column incl. halo
            const int gx = bx + fx, gy = lb.y0 + fy;
            float m[5];
#pragma unroll
            for (int f = 0; f < 5; f++) m[f] = mv[f][fy][fx];
            float mval = 1.f;
            const bool in_img = gx >= 0 && gx < W && gy < H;
            if (sp.has_mask && in_img && mask[(size_t)gy * W + gx] < 128) mval = 0.f;
            if (!(finite_bits(m[0]) && finite_bits(m[1]) && finite_bits(m[2]) && finite_bits(m[3]) && finite_bits(m[4]))) {
                fl[0][fy][fx] = fl[1][fy][fx] = fl[2][fy][fx] = 0.f;
                nwin++;
                continue;
            }
            const float mu_x = m[0], mu_y = m[1];
            const float sxq = fmaxf(m[2] - mu_x * mu_x, 0.f), syq = fmaxf(m[3] - mu_y * mu_y, 0.f);
            const float sxy = m[4] - mu_x * mu_y;
            const float A = 2.f * mu_x * mu_y + kC1, B = 2.f * sxy + kC2;
            const float Cd = mu_x * mu_x + mu_y * mu_y + kC1, D = sxq + syq + kC2;
            // two fast reciprocals (within 2 ulp) in place of four IEEE divisions
            const float rCd = __fdividef(1.f, Cd), rD = __fdividef(1.f, D);
            const float iCD = rCd * rD;
            const float dmu = 2.f * B * (mu_x * Cd - A * mu_y) * iCD * rCd;
            const float dsyq = -A * B * iCD * rD, dsxy = 2.f * A * iCD;
            fl[0][fy][fx] = mval * (dmu - 2.f * mu_y * dsyq - mu_x * dsxy);
            fl[1][fy][fx] = mval * (2.f * dsyq);
            fl[2][fy][fx] = mval * dsxy;
            if (fx >= kHalo && fx < kHalo + kS && in_img) {
                ssim_acc += mval * (A * B) * iCD;
                const size_t p = (size_t)gy * W + gx;
                l1_acc += mval * fabsf((float)gt[3 * p + c] * (1.0f / 255.0f) - a.img[3 * (lb.pb + p) + c]);
            }
        }
        __syncthreads();
        const int x = lb.x0 + lx, y = lb.y0 + ly;
        if (x < W && y < H) {
            float h1 = 0.f, h2 = 0.f, h3 = 0.f;
#pragma unroll
            for (int d = 0; d < 11; d++) {
                const float w = kGauss[10 - d];
                h1 += w * fl[0][ly][lx + d];
                h2 += w * fl[1][ly][lx + d];
                h3 += w * fl[2][ly][lx + d];
            }
            const size_t p = lb.pb + (size_t)y * W + x;
            a.dbuf[(c * 3 + 0) * P + p] = h1;
            a.dbuf[(c * 3 + 1) * P + p] = h2;
            a.dbuf[(c * 3 + 2) * P + p] = h3;
        }
        __syncthreads();
    }
    // loss: each thread whose own pixel is in the image adds w*(1 - s/3) + (1-w)*l/3
    // over the window centres it evaluated (the reference's partition, so a
    // partial edge tile sums the same terms)
    const int x = lb.x0 + lx, y = lb.y0 + ly;
    float v = (x < W && y < H) ? sw * (1.f - ssim_acc / 3.f) + (1.f - sw) * l1_acc / 3.f : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        float s = 0.f;
        for (int k = 0; k < 8; k++) s += red[k];
        atomicAdd(a.loss_sum + lb.view, s);
    }
    if (nwin && a.nan_counts) atomicAdd(a.nan_counts + kNanSsimWin, nwin);
}

template <bool kViews>
__global__ void __launch_bounds__(256) k_ssim_bwd(LossArgs a) {
    __shared__ float sh[9][kSpan][kS];
    const LossBlock lb = loss_block<kViews>(a);
    const int W = lb.W, H = lb.H;
    const size_t P = (size_t)a.vt.pixels;
    const int bx = lb.x0, by = lb.y0 - kHalo;
    const int tid = threadIdx.x, lx = tid & 15, ly = tid >> 4;
    for (int i = tid; i < kSpan * kS; i += 256) {
        const int sy = i / kS, sx = i % kS;
        const int gy = by + sy, gx = bx + sx;
        const bool in = gx < W && gy >= 0 && gy < H;
        const size_t p = in ? lb.pb + ((size_t)gy * W + gx) : 0;
#pragma unroll
        for (int f = 0; f < 9; f++) sh[f][sy][sx] = in ? a.dbuf[f * P + p] : 0.f;
    }
    __syncthreads();
    const int x = bx + lx, y = lb.y0 + ly;
    if (x >= W || y >= H) return;
    const StepParams &sp = a.sp[lb.view];
    const uint8_t *gt = step_gt(a, lb.view), *mask = step_mask(a, lb.view);
    const float sw = sp.ssim_weight, invn = sp.loss_inv_n;
    const size_t pl = (size_t)y * W + x, p = lb.pb + pl;   // this view's pixel, global pixel
    float mc = 1.f;
    if (sp.has_mask && mask[pl] < 128) mc = 0.f;
    unsigned nbad = 0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float c1 = 0.f, c2 = 0.f, c3 = 0.f;
#pragma unroll
        for (int d = 0; d < 11; d++) {
            const float w = kGauss[10 - d];
            c1 += w * sh[c * 3 + 0][ly + d][lx];
            c2 += w * sh[c * 3 + 1][ly + d][lx];
            c3 += w * sh[c * 3 + 2][ly + d][lx];
        }
        const float r = a.img[3 * p + c], g = (float)gt[3 * pl + c] * (1.0f / 255.0f);
        const float vs = c1 + r * c2 + g * c3;
        const float vl = mc * ((g > r) ? -1.f : ((g < r) ? 1.f : 0.f));
        float v = invn * (-sw * vs + (1.f - sw) * vl);
        if (!finite_bits(v)) { nbad++; v = 0.f; }
        a.v_img[3 * p + c] = v;
    }
    if (nbad && a.nan_counts) atomicAdd(a.nan_counts + kNanVRendered, nbad);
}

// The window lives in each device's constant bank: upload it once per device.
static bool g_gauss_ready[64] = {false};

void launch_loss(const LossArgs &a, cudaStream_t s) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !g_gauss_ready[dev]) {
        double g[11], sum = 0;
        for (int i = 0; i < 11; i++) { g[i] = exp(-((i - 5) * (i - 5)) / (2.0 * 1.5 * 1.5)); sum += g[i]; }
        float w[11];
        for (int i = 0; i < 11; i++) w[i] = (float)(g[i] / sum);
        cudaMemcpyToSymbol(kGauss, w, sizeof(w));
        if (dev >= 0 && dev < 64) g_gauss_ready[dev] = true;
    }
    if (a.vt.count > 1) {
        k_ssim_h<true><<<a.num_tiles, 256, 0, s>>>(a);
        k_ssim_fields<true><<<a.num_tiles, 256, 0, s>>>(a);
        k_ssim_bwd<true><<<a.num_tiles, 256, 0, s>>>(a);
    } else {
        const dim3 grid(a.vt.tiles_x[0], a.vt.tiles_y[0]);
        k_ssim_h<false><<<grid, 256, 0, s>>>(a);
        k_ssim_fields<false><<<grid, 256, 0, s>>>(a);
        k_ssim_bwd<false><<<grid, 256, 0, s>>>(a);
    }
}

}  // namespace msplat
