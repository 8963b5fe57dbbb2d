// Host camera setup and evaluation metrics.
//  * prepare camera: world->camera and projection matrices from an OpenGL
//    camera-to-world pose (core/src/model.cpp:845-889);
//  * PSNR / L1 over float images (model.cpp:34-49) and the evaluation SSIM
//    with replicate padding (core/src/ssim.cpp:61-123).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "msplat_gb300.h"

extern "C" {

void msplat_prepare_camera(const float c2w[16], int width, int height, float fx, float fy, float viewmat[16],
                           float projmat[16], float cam_pos[3]) {
    const float fov_x = 2.0f * std::atan((float)width / (2.0f * fx));
    const float fov_y = 2.0f * std::atan((float)height / (2.0f * fy));
    // OpenGL -> OpenCV axes: negate the camera's y and z columns
    float R[3][3], T[3];
    for (int i = 0; i < 3; i++) {
        R[i][0] = c2w[i * 4 + 0];
        R[i][1] = -c2w[i * 4 + 1];
        R[i][2] = -c2w[i * 4 + 2];
        T[i] = c2w[i * 4 + 3];
    }
    float v[16] = {0};
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) v[i * 4 + j] = R[j][i];   // R^T
        v[i * 4 + 3] = -(R[0][i] * T[0] + R[1][i] * T[1] + R[2][i] * T[2]);
    }
    v[15] = 1.0f;
    const float znear = 0.001f, zfar = 1000.0f;
    const float top = znear * std::tan(0.5f * fov_y), right = znear * std::tan(0.5f * fov_x);
    float p[16] = {0};
    p[0] = znear / right;
    p[5] = znear / top;
    p[10] = (zfar + znear) / (zfar - znear);
    p[11] = -zfar * znear / (zfar - znear);
    p[14] = 1.0f;
    float pv[16] = {0};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++) pv[i * 4 + j] += p[i * 4 + k] * v[k * 4 + j];
    std::memcpy(viewmat, v, sizeof(v));
    std::memcpy(projmat, pv, sizeof(pv));
    for (int i = 0; i < 3; i++) cam_pos[i] = T[i];
}

float msplat_psnr(const float *img, const float *gt, long long n) {
    double mse = 0;
    for (long long i = 0; i < n; i++) {
        const double d = img[i] - gt[i];
        mse += d * d;
    }
    mse /= (double)n;
    return 10.0f * std::log10(1.0 / mse);
}

float msplat_l1(const float *img, const float *gt, long long n) {
    double s = 0;
    for (long long i = 0; i < n; i++) s += std::abs(img[i] - gt[i]);
    return (float)(s / (double)n);
}

float msplat_ssim_eval(const float *img, const float *gt, int height, int width) {
    const int ks = 11, half = 5;
    float kern[11], ksum = 0;
    for (int i = 0; i < ks; i++) {
        const float x = (float)(i - half);
        kern[i] = std::exp(-(x * x) / (2.0f * 1.5f * 1.5f));
        ksum += kern[i];
    }
    for (int i = 0; i < ks; i++) kern[i] /= ksum;
    const int H = height, W = width;
    const size_t HW = (size_t)H * W;
    std::vector<float> a(HW), b(HW), aa(HW), bb(HW), ab(HW), m1(HW), m2(HW), s11(HW), s22(HW), s12(HW), tmp(HW);
    auto blur = [&](const std::vector<float> &in, std::vector<float> &out) {
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                float s = 0;
                for (int k = 0; k < ks; k++) s += in[(size_t)y * W + std::min(std::max(x + k - half, 0), W - 1)] * kern[k];
                tmp[(size_t)y * W + x] = s;
            }
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                float s = 0;
                for (int k = 0; k < ks; k++) s += tmp[(size_t)std::min(std::max(y + k - half, 0), H - 1) * W + x] * kern[k];
                out[(size_t)y * W + x] = s;
            }
    };
    const float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
    double total = 0;
    for (int c = 0; c < 3; c++) {
        for (size_t i = 0; i < HW; i++) {
            a[i] = img[i * 3 + c];
            b[i] = gt[i * 3 + c];
            aa[i] = a[i] * a[i];
            bb[i] = b[i] * b[i];
            ab[i] = a[i] * b[i];
        }
        blur(a, m1); blur(b, m2); blur(aa, s11); blur(bb, s22); blur(ab, s12);
        for (size_t i = 0; i < HW; i++) {
            const float u1 = m1[i] * m1[i], u2 = m2[i] * m2[i], u12 = m1[i] * m2[i];
            const float num = (2.0f * u12 + C1) * (2.0f * (s12[i] - u12) + C2);
            const float den = (u1 + u2 + C1) * ((s11[i] - u1) + (s22[i] - u2) + C2);
            total += num / den;
        }
    }
    return (float)(total / (double)(3 * HW));
}

}  // extern "C"
