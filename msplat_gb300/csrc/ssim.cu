// Training loss L = w * (1 - mean SSIM) + (1 - w) * mean |x - gt| and its
// image gradient in one kernel: one CTA per 32x32 block of output pixels,
// the three channels in turn, everything between the image and dL/dx in
// shared memory (no intermediate planes in HBM):
//   load    target and render over the block plus a 10-pixel halo (once)
//   A       vertical 11-tap moments of (gt, x, gt^2, x^2, gt*x) at the 42
//           window-centre rows, every input column (zero padding)
//   B       horizontal 11-tap moments at the 42x42 window centres -> SSIM,
//           L1 and the derivative fields (f1, f2, f3)
//   C       horizontal transpose convolution of the fields
//   D       vertical transpose convolution -> dL/dx of the block
// The loss and gradient are those of ssim_h_fwd_kernel,
// ssim_fused_v_fwd_h_bwd_kernel and ssim_v_bwd_kernel
// (msplat_metal.metal:3388-3450, 3563-3681, 3764-3850) with their edge
// rules: moments at window centres in out-of-image columns are zero (the
// reference's horizontal moments exist only inside the image) and their
// fields still enter the horizontal transpose convolution, centres in
// out-of-image rows contribute nothing, and the loss sum keeps the
// reference's 16x16-tile partition (loss_counted).  One launch covers every view of the
// step (blocks are numbered view by view; the render and dL/dx are indexed
// by global pixel, each view's target and mask by its own pixel).
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace msplat {

__constant__ float kGauss[11];
constexpr float kC1 = 0.0001f, kC2 = 0.0009f;

// Target and mask: the arguments' when set (one view), else the view's in StepParams.
__device__ __forceinline__ const uint8_t *step_gt(const LossArgs &a, int v) { return a.gt ? a.gt : a.sp[v].gt; }
__device__ __forceinline__ const uint8_t *step_mask(const LossArgs &a, int v) { return a.gt ? a.mask : a.sp[v].mask; }

constexpr int kFB = 32;              // output block edge
constexpr int kFIn = kFB + 20;       // 52: input rows / columns (halo 10)
constexpr int kFF = kFB + 10;        // 42: window-centre rows / columns (halo 5)

// Padded row strides keep the column-wise and row-wise walks conflict-free.
struct FusedSmem {
    float r[3][kFIn + 2][kFIn + 1];      // render, channel-planar, zero outside the image (+2 pad rows)
    uint8_t g[3][kFIn + 2][kFIn + 4];    // target, channel-planar, zero outside the image (+2 pad rows)
    union {
        struct {                     // A: vertical moments [centre row][input column]
            float2 m01[kFF][kFIn + 1];   // (gt, x)
            float2 m23[kFF][kFIn + 1];   // (gt^2, x^2)
            float m4[kFF][kFIn + 1];     // gt * x
        } v;
        struct {                     // C: horizontally transposed fields [centre row][output column]
            float2 f12[kFF][kFB + 1];
            float f3[kFF][kFB + 1];
        } dh;
    } u;
    float2 f12[kFF][kFF + 1];        // B: fields (f1, f2) at the window centres
    float f3[kFF][kFF + 1];          //    and f3
    float red[8];
};

struct FusedBlock {
    int view, W, H, x0, y0;
    long long pb;   // global index of the view's pixel 0
};

// kViews: blocks numbered view by view over every view of the step; false:
// one view, a 2D grid, geometry from the parameter bank
template <bool kViews> __device__ __forceinline__ FusedBlock fused_block(const LossArgs &a) {
    FusedBlock b;
    if (!kViews) {
        b.view = 0;
        b.W = a.vt.width[0];
        b.H = a.vt.height[0];
        b.x0 = blockIdx.x * kFB;
        b.y0 = blockIdx.y * kFB;
        b.pb = 0;
        return b;
    }
    const int blk = blockIdx.x;
    int v = 0, base = 0, run = 0;
#pragma unroll
    for (int k = 0; k < kMaxViews; k++) {
        if (k < a.vt.count) {
            if (blk >= run) { v = k; base = run; }
            run += ((a.vt.width[k] + kFB - 1) / kFB) * ((a.vt.height[k] + kFB - 1) / kFB);
        }
    }
    const ViewGeom vg = view_geom(a.vt, v);
    const int bxn = (vg.width + kFB - 1) / kFB, lb = blk - base;
    b.view = v;
    b.W = vg.width;
    b.H = vg.height;
    b.x0 = (lb % bxn) * kFB;
    b.y0 = (lb / bxn) * kFB;
    b.pb = vg.pix_base;
    return b;
}

static int fused_blocks(const ViewTable &vt) {
    int nb = 0;
    for (int k = 0; k < vt.count; k++) nb += ((vt.width[k] + kFB - 1) / kFB) * ((vt.height[k] + kFB - 1) / kFB);
    return nb;
}

// Whether the reference's loss sum includes window centre (x, y) of the
// image.  It sums per thread of a 16x16 tile: thread t evaluates centres t
// and t + 256 of the tile's 16 x 26 centre grid (its own rows, columns with a
// 5-pixel halo), and only a thread whose own pixel lies in the image adds
// what it evaluated (.metal:3598-3671).  Centres of full tiles always count;
// in a partial edge tile some in-image centres fall to threads outside.
__device__ __forceinline__ bool loss_counted(int x, int y, int W, int H) {
    const int i = (y & 15) * 26 + (x & 15) + 5;
    const int t = i < 256 ? i : i - 256;
    return (x & ~15) + (t & 15) < W && (y & ~15) + (t >> 4) < H;
}

template <bool kViews>
__global__ void __launch_bounds__(256, 2) k_ssim_fused(LossArgs a) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FusedSmem &sm = *reinterpret_cast<FusedSmem *>(smem_raw);
    const FusedBlock fb = fused_block<kViews>(a);
    const int W = fb.W, H = fb.H, X0 = fb.x0, Y0 = fb.y0;
    const StepParams &sp = a.sp[fb.view];
    const uint8_t *gt = step_gt(a, fb.view), *mask = step_mask(a, fb.view);
    const bool has_mask = sp.has_mask != 0;
    const float sw = sp.ssim_weight, invn = sp.loss_inv_n;
    const int tid = threadIdx.x;
    const int dx_ = tid & 31, dy0 = (tid >> 5) * 4;   // D: output column, first of four output rows
    float ssim_acc = 0.f, l1_acc = 0.f, inside = 0.f;
    unsigned nwin = 0, nbad = 0;

    // the block's render and target with their halo, all three channels:
    // each row's 52 pixels are 156 contiguous floats / bytes.  Eight loads of
    // each kind in flight per thread, then the shared-memory stores.
    constexpr int kLoadElems = kFIn * kFIn * 3, kLoadUnroll = 8;
    for (int base = 0; base < kLoadElems; base += 256 * kLoadUnroll) {
        float rv[kLoadUnroll];
        uint32_t gv[kLoadUnroll];
#pragma unroll
        for (int u = 0; u < kLoadUnroll; u++) {
            const int i = base + u * 256 + tid;
            const int iy = i / (kFIn * 3), e = i - iy * (kFIn * 3);
            const int ix = e / 3, c = e - ix * 3;
            const int y = Y0 - 10 + iy, x = X0 - 10 + ix;
            rv[u] = 0.f;
            gv[u] = 0;
            if (i < kLoadElems && x >= 0 && x < W && y >= 0 && y < H) {
                const size_t pl = (size_t)y * W + x;
                gv[u] = gt[3 * pl + c];
                rv[u] = a.img[3 * (fb.pb + pl) + c];
            }
        }
#pragma unroll
        for (int u = 0; u < kLoadUnroll; u++) {
            const int i = base + u * 256 + tid;
            if (i < kLoadElems) {
                const int iy = i / (kFIn * 3), e = i - iy * (kFIn * 3);
                const int ix = e / 3, c = e - ix * 3;
                sm.r[c][iy][ix] = rv[u];
                sm.g[c][iy][ix] = (uint8_t)gv[u];
            }
        }
    }
    for (int i = tid; i < 3 * 2 * kFIn; i += 256) {   // the pad rows A reads past the last input row
        const int c = i / (2 * kFIn), e = i - c * 2 * kFIn;
        sm.r[c][kFIn + e / kFIn][e % kFIn] = 0.f;
        sm.g[c][kFIn + e / kFIn][e % kFIn] = 0;
    }
    __syncthreads();

    for (int c = 0; c < 3; c++) {
        // A: (input column, 11 centre rows) per item; the 21 inputs and their
        // products in registers, moments in pairs (paired fp32 arithmetic).
        // The target stays in 0..255 here (exact in float); its moments are
        // scaled by 1/255 (mean, cross moment) and by 1/255 twice (second
        // moment) at the end.
        for (int it = tid; it < kFIn * 4; it += 256) {
            const int ix = it % kFIn, s = it / kFIn;
            const int vy0 = 11 * s, n = min(11, kFF - vy0);
            float2 gr[21];   // (gt, x), then (gt^2, x^2)
            float gx[21];    // gt * x
#pragma unroll
            for (int j = 0; j < 21; j++) {
                gr[j] = make_float2((float)sm.g[c][vy0 + j][ix], sm.r[c][vy0 + j][ix]);
                gx[j] = gr[j].x * gr[j].y;
            }
#pragma unroll
            for (int k = 0; k < 11; k++) {
                if (k < n) {
                    float2 m01 = make_float2(0.f, 0.f);
                    float m4 = 0.f;
#pragma unroll
                    for (int d = 0; d < 11; d++) {
                        const float w = kGauss[d];
                        m01 = __ffma2_rn(make_float2(w, w), gr[k + d], m01);
                        m4 = fmaf(w, gx[k + d], m4);
                    }
                    sm.u.v.m01[vy0 + k][ix] = __fmul2_rn(m01, make_float2(1.0f / 255.0f, 1.f));
                    sm.u.v.m4[vy0 + k][ix] = m4 * (1.0f / 255.0f);
                }
            }
#pragma unroll
            for (int j = 0; j < 21; j++) gr[j] = __fmul2_rn(gr[j], gr[j]);
#pragma unroll
            for (int k = 0; k < 11; k++) {
                if (k < n) {
                    float2 m23 = make_float2(0.f, 0.f);
#pragma unroll
                    for (int d = 0; d < 11; d++) m23 = __ffma2_rn(make_float2(kGauss[d], kGauss[d]), gr[k + d], m23);
                    // scaled by 1/255 twice, as the mean is once: a single 1/65025 (one
                    // ulp below (1/255)^2 in float) biased every variance low
                    const float2 s255 = make_float2(1.0f / 255.0f, 1.f);
                    sm.u.v.m23[vy0 + k][ix] = __fmul2_rn(__fmul2_rn(m23, s255), s255);
                }
            }
        }
        __syncthreads();

        // B: (centre row, 7 centre columns) per item -> moments, SSIM, fields
        for (int it = tid; it < kFF * 6; it += 256) {
            const int fy = it % kFF, s = it / kFF, fx0 = 7 * s;
            float2 m01[7], m23[7];
            float m4[7];
            {
                float2 row[17];
#pragma unroll
                for (int j = 0; j < 17; j++) row[j] = sm.u.v.m01[fy][fx0 + j];
#pragma unroll
                for (int k = 0; k < 7; k++) {
                    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                    for (int d = 0; d < 11; d++) acc = __ffma2_rn(make_float2(kGauss[d], kGauss[d]), row[k + d], acc);
                    m01[k] = acc;
                }
#pragma unroll
                for (int j = 0; j < 17; j++) row[j] = sm.u.v.m23[fy][fx0 + j];
#pragma unroll
                for (int k = 0; k < 7; k++) {
                    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                    for (int d = 0; d < 11; d++) acc = __ffma2_rn(make_float2(kGauss[d], kGauss[d]), row[k + d], acc);
                    m23[k] = acc;
                }
            }
            {
                float row[17];
#pragma unroll
                for (int j = 0; j < 17; j++) row[j] = sm.u.v.m4[fy][fx0 + j];
#pragma unroll
                for (int k = 0; k < 7; k++) {
                    float acc = 0.f;
#pragma unroll
                    for (int d = 0; d < 11; d++) acc += kGauss[d] * row[k + d];
                    m4[k] = acc;
                }
            }
            const int yc = Y0 - 5 + fy;
            const bool in_row = yc >= 0 && yc < H;
            const bool own_row = fy >= 5 && fy < 5 + kFB;
#pragma unroll
            for (int k = 0; k < 7; k++) {
                const int fx = fx0 + k, xc = X0 - 5 + fx;
                const bool in_col = xc >= 0 && xc < W;
                const bool in_img = in_row && in_col;
                const bool own = in_img && own_row && fx >= 5 && fx < 5 + kFB;
                float mu_x = m01[k].x, mu_y = m01[k].y, q_x = m23[k].x, q_y = m23[k].y, q_xy = m4[k];
                if (!in_col) mu_x = mu_y = q_x = q_y = q_xy = 0.f;
                float f1 = 0.f, f2 = 0.f, f3 = 0.f;
                if (!(finite_bits(mu_x) && finite_bits(mu_y) && finite_bits(q_x) && finite_bits(q_y) &&
                      finite_bits(q_xy))) {
                    if (own) nwin++;
                } else {
                    float mval = 1.f;
                    if (has_mask && in_img && mask[(size_t)yc * W + xc] < 128) mval = 0.f;
                    const float sxq = fmaxf(q_x - mu_x * mu_x, 0.f), syq = fmaxf(q_y - mu_y * mu_y, 0.f);
                    const float sxy = q_xy - mu_x * mu_y;
                    const float A = 2.f * mu_x * mu_y + kC1, B = 2.f * sxy + kC2;
                    const float Cd = mu_x * mu_x + mu_y * mu_y + kC1, D = sxq + syq + kC2;
                    // two fast reciprocals (within 2 ulp) in place of four IEEE divisions
                    const float rCd = __fdividef(1.f, Cd), rD = __fdividef(1.f, D);
                    const float iCD = rCd * rD;
                    const float dmu = 2.f * B * (mu_x * Cd - A * mu_y) * iCD * rCd;
                    const float dsyq = -A * B * iCD * rD, dsxy = 2.f * A * iCD;
                    if (in_row) {
                        f1 = mval * (dmu - 2.f * mu_y * dsyq - mu_x * dsxy);
                        f2 = mval * (2.f * dsyq);
                        f3 = mval * dsxy;
                    }
                    if (own && loss_counted(xc, yc, W, H)) {
                        // the loss value takes the reference's one IEEE division: the fast
                        // reciprocals' bias, summed over every pixel, is visible at low loss
                        ssim_acc += mval * __fdiv_rn(A * B, Cd * D);
                        l1_acc += mval * fabsf((float)sm.g[c][fy + 5][fx + 5] * (1.0f / 255.0f) - sm.r[c][fy + 5][fx + 5]);
                    }
                }
                sm.f12[fy][fx] = make_float2(f1, f2);
                sm.f3[fy][fx] = f3;
            }
        }
        __syncthreads();

        // C: (centre row, 8 output columns) per item
        for (int it = tid; it < kFF * 4; it += 256) {
            const int fy = it % kFF, ox0 = 8 * (it / kFF);
            {
                float2 row[18];
#pragma unroll
                for (int t = 0; t < 18; t++) row[t] = sm.f12[fy][ox0 + t];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                    for (int d = 0; d < 11; d++)
                        acc = __ffma2_rn(make_float2(kGauss[10 - d], kGauss[10 - d]), row[k + d], acc);
                    sm.u.dh.f12[fy][ox0 + k] = acc;
                }
            }
            {
                float row[18];
#pragma unroll
                for (int t = 0; t < 18; t++) row[t] = sm.f3[fy][ox0 + t];
#pragma unroll
                for (int k = 0; k < 8; k++) {
                    float acc = 0.f;
#pragma unroll
                    for (int d = 0; d < 11; d++) acc += kGauss[10 - d] * row[k + d];
                    sm.u.dh.f3[fy][ox0 + k] = acc;
                }
            }
        }
        __syncthreads();

        // D: (output column, 4 output rows) per thread -> dL/dx of channel c
        {
            float2 c12[4];
            float c3[4];
            {
                float2 col[14];
#pragma unroll
                for (int t = 0; t < 14; t++) col[t] = sm.u.dh.f12[dy0 + t][dx_];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    float2 acc = make_float2(0.f, 0.f);
#pragma unroll
                    for (int d = 0; d < 11; d++)
                        acc = __ffma2_rn(make_float2(kGauss[10 - d], kGauss[10 - d]), col[k + d], acc);
                    c12[k] = acc;
                }
            }
            {
                float col[14];
#pragma unroll
                for (int t = 0; t < 14; t++) col[t] = sm.u.dh.f3[dy0 + t][dx_];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    float acc = 0.f;
#pragma unroll
                    for (int d = 0; d < 11; d++) acc += kGauss[10 - d] * col[k + d];
                    c3[k] = acc;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int y = Y0 + dy0 + k, x = X0 + dx_;
                if (x < W && y < H) {
                    const float R = sm.r[c][dy0 + k + 10][dx_ + 10];
                    const float G = (float)sm.g[c][dy0 + k + 10][dx_ + 10] * (1.0f / 255.0f);
                    const float mc = (has_mask && mask[(size_t)y * W + x] < 128) ? 0.f : 1.f;
                    const float vs = c12[k].x + R * c12[k].y + G * c3[k];
                    const float vl = mc * ((G > R) ? -1.f : ((G < R) ? 1.f : 0.f));
                    float v = invn * (-sw * vs + (1.f - sw) * vl);
                    if (!finite_bits(v)) { nbad++; v = 0.f; }
                    if (c == 0) inside += 1.f;
                    a.v_img[3 * (fb.pb + (size_t)y * W + x) + c] = v;
                }
            }
        }
        __syncthreads();   // the next channel's moments overwrite dh
    }

    // loss: sum over the block's pixels in the image of w*(1 - s/3) + (1-w)*l/3,
    // s and l summed over the channels
    float v = sw * (inside - ssim_acc / 3.f) + (1.f - sw) * l1_acc / 3.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((tid & 31) == 0) sm.red[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        float t = 0.f;
        for (int k = 0; k < 8; k++) t += sm.red[k];
        atomicAdd(a.loss_sum + fb.view, t);
    }
    if (nwin && a.nan_counts) atomicAdd(a.nan_counts + kNanSsimWin, nwin);
    if (nbad && a.nan_counts) atomicAdd(a.nan_counts + kNanVRendered, nbad);
}

// Per-device set-up, done once per device under a lock: the window goes to
// the device's constant bank and both kernel instantiations get their
// shared-memory limit.  A device is marked ready only when every call
// succeeded, so a failed first call is retried by the next one.
static bool g_loss_ready[64] = {false};
static std::mutex g_loss_mu;

static cudaError_t loss_setup(int dev) {
    std::lock_guard<std::mutex> lk(g_loss_mu);
    if (g_loss_ready[dev]) return cudaSuccess;
    double g[11], sum = 0;
    for (int i = 0; i < 11; i++) { g[i] = exp(-((i - 5) * (i - 5)) / (2.0 * 1.5 * 1.5)); sum += g[i]; }
    float w[11];
    for (int i = 0; i < 11; i++) w[i] = (float)(g[i] / sum);
    cudaError_t e = cudaMemcpyToSymbol(kGauss, w, sizeof(w));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_ssim_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(FusedSmem));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_ssim_fused<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(FusedSmem));
    if (e == cudaSuccess) g_loss_ready[dev] = true;
    return e;
}

int launch_loss(const LossArgs &a, cudaStream_t s) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -1;
    const cudaError_t e = loss_setup(dev);
    if (e != cudaSuccess) {
        fprintf(stderr, "msplat loss set-up: %s\n", cudaGetErrorString(e));
        return -1;
    }
    const size_t smem = sizeof(FusedSmem);
    if (a.vt.count > 1) {
        const int nb = fused_blocks(a.vt);
        if (nb <= 0) return 0;
        launch_pdl(k_ssim_fused<true>, nb, 256, smem, s, a);
    } else {
        const dim3 grid((a.vt.width[0] + kFB - 1) / kFB, (a.vt.height[0] + kFB - 1) / kFB);
        if (grid.x == 0 || grid.y == 0) return 0;
        launch_pdl(k_ssim_fused<false>, grid, 256, smem, s, a);
    }
    return 1;
}

}  // namespace msplat
