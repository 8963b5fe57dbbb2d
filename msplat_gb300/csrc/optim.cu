// Optimizer tail of the step:
//  * one launch of fused Adam over the four flat parameter groups (means,
//    log-scales, quaternions, opacity logits), with the MCMC opacity/scale
//    regularizer gradient added in registers (mcmc_reg_grad_kernel +
//    fused_adam_kernel, msplat_metal.metal:3987-4026 and :1680-1713;
//    launched as 1 + 4 dispatches by msplat_metal.mm:1454-1488);
//  * SGLD position noise with the normal samples generated in the same
//    thread (sgld_noise_gen_kernel + sgld_noise_kernel, :3862-3967).
#include "common.cuh"
#include "kernels.h"

namespace msplat {

// Regularizer gradient of element j of group grp (1: log-scales, 3: opacity
// logits) added to g (mcmc_reg_grad_kernel, msplat_metal.metal:3987-4026).
__device__ __forceinline__ float reg_grad(const AdamArgs &a, const StepParams &sp, int grp, long long j, float pv,
                                          float g, float invN_base) {
    const long long gi = grp == 1 ? j / 3 : j;
    float duty = 1.0f;
    if (sp.invis_scale != 1.0f) {
        const float *dv = a.dc_v + 3 * gi;
        duty = (dv[0] + dv[1] + dv[2] == 0.0f) ? 1.0f : sp.invis_scale;
    }
    const float invN = duty * invN_base;
    if (grp == 3) {
        const float sig = 1.0f / (1.0f + det_expf(-pv));
        return g + sp.op_reg * sig * (1.0f - sig) * invN;
    }
    return g + sp.sc_reg * det_expf(fminf(fmaxf(pv, -15.0f), 15.0f)) * (invN * (1.0f / 3.0f));
}

// Adam on one element; returns false (and leaves it) for a non-finite gradient.
__device__ __forceinline__ bool adam_step(float &p, float &m, float &v, float g, float b1, float b2, float eps,
                                          float st, float bc) {
    if (!finite_bits(g)) return false;
    const float mm = fmaf(b1, m, (1.0f - b1) * g);
    const float vv = fmaf(b2, v, (1.0f - b2) * g * g);
    p = p - adam_delta(st, mm, vv, bc, eps);
    m = mm;
    v = vv;
    return true;
}

// The four groups (means 3N, log-scales 3N, quaternions 4N, opacity logits N)
// in one launch.  Each group is walked in 16-byte steps (parameter, moments
// and gradient loaded as float4, every load of a step issued before any
// use); a group length that is not a multiple of 4 ends with scalar steps.
__global__ void __launch_bounds__(256) k_adam(AdamArgs a) {
    pdl_enter();
    const StepParams &sp = *a.sp;
    const float b1 = sp.beta1, b2 = sp.beta2, eps = sp.eps;
    const bool reg = sp.op_reg > 0.f || sp.sc_reg > 0.f;
    const float invN_base = 1.0f / (float)a.n;
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    unsigned bad[4] = {0, 0, 0, 0};
#pragma unroll 1
    for (int grp = 0; grp < 4; grp++) {
        float *p, *m, *v;
        const float *gsrc = nullptr;
        long long len;
        if (grp == 0) { p = a.means; m = a.m[0]; v = a.v[0]; gsrc = a.g_mean; len = 3LL * a.n; }
        else if (grp == 1) { p = a.scales; m = a.m[1]; v = a.v[1]; gsrc = a.g_scale; len = 3LL * a.n; }
        else if (grp == 2) { p = a.quats; m = a.m[2]; v = a.v[2]; gsrc = a.g_quat; len = 4LL * a.n; }
        else { p = a.opacities; m = a.m[3]; v = a.v[3]; len = a.n; }
        const int sg = grp == 3 ? 5 : grp;
        const float st = sp.step_size[sg], bc = sp.bc2_sqrt[sg];
        const bool greg = reg && (grp == 1 || grp == 3);
        // float4 steps need 16-byte aligned arrays (caller-owned parameters may not be)
        const uintptr_t al = (uintptr_t)p | (uintptr_t)m | (uintptr_t)v | (uintptr_t)gsrc |
                             (uintptr_t)(grp == 3 ? a.g_opac : nullptr);
        const long long n4 = (al & 15u) ? 0 : len / 4;
        for (long long q = tid; q < n4; q += nthreads) {
            float4 P = reinterpret_cast<const float4 *>(p)[q];
            float4 M = reinterpret_cast<const float4 *>(m)[q];
            float4 V = reinterpret_cast<const float4 *>(v)[q];
            float4 G;
            if (grp == 3 && a.g_opac) {
                G = reinterpret_cast<const float4 *>(a.g_opac)[q];
            } else if (grp == 3) {
                const long long j = 4 * q;
                G = make_float4(a.grad[j].a.z, a.grad[j + 1].a.z, a.grad[j + 2].a.z, a.grad[j + 3].a.z);
            } else {
                G = reinterpret_cast<const float4 *>(gsrc)[q];
            }
            float *pp = &P.x, *mm = &M.x, *vv = &V.x, *gg = &G.x;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float g = gg[k];
                if (greg) g = reg_grad(a, sp, grp, 4 * q + k, pp[k], g, invN_base);
                if (!adam_step(pp[k], mm[k], vv[k], g, b1, b2, eps, st, bc)) bad[grp]++;
            }
            reinterpret_cast<float4 *>(p)[q] = P;
            reinterpret_cast<float4 *>(m)[q] = M;
            reinterpret_cast<float4 *>(v)[q] = V;
        }
        for (long long j = 4 * n4 + tid; j < len; j += nthreads) {
            float pv = p[j], mv = m[j], vv = v[j];
            float g = grp == 3 ? (a.g_opac ? a.g_opac[j] : a.grad[j].a.z) : gsrc[j];
            if (greg) g = reg_grad(a, sp, grp, j, pv, g, invN_base);
            if (!adam_step(pv, mv, vv, g, b1, b2, eps, st, bc)) { bad[grp]++; continue; }
            p[j] = pv;
            m[j] = mv;
            v[j] = vv;
        }
    }
    if (a.nan_counts) {
        if (bad[0]) atomicAdd(a.nan_counts + kNanMean, bad[0]);
        if (bad[1]) atomicAdd(a.nan_counts + kNanScale, bad[1]);
        if (bad[2]) atomicAdd(a.nan_counts + kNanQuat, bad[2]);
        if (bad[3]) atomicAdd(a.nan_counts + kNanOpacity, bad[3]);
    }
}

__device__ __forceinline__ uint32_t pcg_hash32(uint32_t seed, uint32_t idx) {
    uint32_t x = seed * 747796405u + idx * 2891336453u;
    x = ((x >> ((x >> 28) + 4)) ^ x) * 277803737u;
    return (x >> 22) ^ x;
}
__device__ __forceinline__ float pcg_unit(uint32_t h) {
    return ((float)(h >> 9) + 0.5f) * (1.0f / (float)(1u << 23));
}

__global__ void __launch_bounds__(256) k_sgld(AdamArgs a) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const StepParams &sp = *a.sp;
    // every input is loaded before the arithmetic, so the loads are in flight together
    const float opl = a.opacities[i];
    const float4 q = *reinterpret_cast<const float4 *>(a.quats + 4 * (size_t)i);
    const float sc0 = a.scales[3 * i], sc1 = a.scales[3 * i + 1], sc2 = a.scales[3 * i + 2];
    const float m0 = a.means[3 * i], m1 = a.means[3 * i + 1], m2 = a.means[3 * i + 2];
    const uint32_t base = (uint32_t)i * 4u;
    const float u0 = pcg_unit(pcg_hash32(sp.seed, base)), u1 = pcg_unit(pcg_hash32(sp.seed, base + 1u));
    const float u2 = pcg_unit(pcg_hash32(sp.seed, base + 2u)), u3 = pcg_unit(pcg_hash32(sp.seed, base + 3u));
    const float r01 = sqrtf(-2.0f * logf(u0)), r23 = sqrtf(-2.0f * logf(u2));
    const float a01 = 6.283185307179586f * u1, a23 = 6.283185307179586f * u3;
    const float op = 1.0f / (1.0f + det_expf(-opl));
    const float wgt = 1.0f / (1.0f + det_expf(-100.0f * ((1.0f - op) - 0.995f)));
    const float ns = sp.noise_lr * sp.xyz_lr * wgt;
    float s01, c01;
    sincosf(a01, &s01, &c01);   // one range reduction for both
    const float n0 = r01 * c01 * ns, n1 = r01 * s01 * ns, n2 = r23 * cosf(a23) * ns;
    const float rql = 1.0f / sqrtf(fmaxf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w, 1e-8f));
    const float qw = q.x * rql, qx = q.y * rql, qy = q.z * rql, qz = q.w * rql;
    const float s[3] = {det_expf(fminf(fmaxf(sc0, -15.0f), 15.0f)), det_expf(fminf(fmaxf(sc1, -15.0f), 15.0f)),
                        det_expf(fminf(fmaxf(sc2, -15.0f), 15.0f))};
    const float r00 = 1 - 2 * (qy * qy + qz * qz), r01_ = 2 * (qx * qy - qw * qz), r02 = 2 * (qx * qz + qw * qy);
    const float r10 = 2 * (qx * qy + qw * qz), r11 = 1 - 2 * (qx * qx + qz * qz), r12 = 2 * (qy * qz - qw * qx);
    const float r20 = 2 * (qx * qz - qw * qy), r21 = 2 * (qy * qz + qw * qx), r22 = 1 - 2 * (qx * qx + qy * qy);
    float t0 = r00 * n0 + r10 * n1 + r20 * n2;
    float t1 = r01_ * n0 + r11 * n1 + r21 * n2;
    float t2 = r02 * n0 + r12 * n1 + r22 * n2;
    t0 *= s[0] * s[0]; t1 *= s[1] * s[1]; t2 *= s[2] * s[2];
    float v0 = r00 * t0 + r01_ * t1 + r02 * t2;
    float v1 = r10 * t0 + r11 * t1 + r12 * t2;
    float v2 = r20 * t0 + r21 * t1 + r22 * t2;
    if (!finite_bits(v0) || !finite_bits(v1) || !finite_bits(v2)) return;
    const float len2 = v0 * v0 + v1 * v1 + v2 * v2;
    if (!finite_bits(len2)) return;
    if (len2 > sp.max_disp * sp.max_disp) {
        const float inv = sp.max_disp / sqrtf(len2);
        v0 *= inv; v1 *= inv; v2 *= inv;
    }
    a.means[3 * i] = m0 + v0;
    a.means[3 * i + 1] = m1 + v1;
    a.means[3 * i + 2] = m2 + v2;
}

void launch_adam(const AdamArgs &a, int num_sms, cudaStream_t s) {
    if (a.n <= 0) return;
    const long long total = 11LL * a.n;
    long long blocks = (total + 255) / 256;
    const long long cap = (long long)num_sms * 8;
    if (blocks > cap) blocks = cap;
    launch_pdl(k_adam, (unsigned)blocks, 256, 0, s, a);
}

void launch_sgld(const AdamArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    launch_pdl(k_sgld, (a.n + 255) / 256, 256, 0, s, a);
}

}  // namespace msplat
