// Projection VJP (centre, conic -> mean, log-scale, quaternion) with the SH
// colour VJP fused straight into Adam for features_dc / features_rest, one
// thread per Gaussian.  The 3D covariance is recomputed in registers.
// Follows project_and_sh_backward_kernel (msplat_metal.metal:1860-2042) and
// the VJPs it calls (:1252-1569): gradients flow to the raw quaternion as if
// it were normalised, and bands above degrees_to_use are not updated.
#include "common.cuh"
#include "kernels.h"

namespace msplat {

__constant__ float kBC0 = 0.28209479177387814f;
__constant__ float kBC1 = 0.4886025119029199f;
__constant__ float kBC2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                              -1.0925484305920792f, 0.5462742152960396f};
__constant__ float kBC3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                              0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                              -0.5900435899266435f};

__device__ __forceinline__ void adam_el(float *p, float *m, float *v, float g, float step, float bc2s, float b1,
                                        float b2, float eps) {
    const float mm = fmaf(b1, *m, (1.0f - b1) * g);
    const float vv = fmaf(b2, *v, (1.0f - b2) * g * g);
    *p -= step * mm / (sqrtf(vv) / bc2s + eps);
    *m = mm;
    *v = vv;
}

__device__ __forceinline__ void mat3mul(const float A[3][3], const float B[3][3], float C[3][3]) {
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) C[r][c] = A[r][0] * B[0][c] + A[r][1] * B[1][c] + A[r][2] * B[2][c];
}

__global__ void __launch_bounds__(256) k_project_bwd(ProjectBwdArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    float *vmean = a.v_mean + 3 * (size_t)i, *vscale = a.v_scale + 3 * (size_t)i, *vquat = a.v_quat + 4 * (size_t)i;
    if (a.radii[i] <= 0) {
        vmean[0] = vmean[1] = vmean[2] = 0.f;
        vscale[0] = vscale[1] = vscale[2] = 0.f;
        *reinterpret_cast<float4 *>(vquat) = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const StepParams &sp = *a.sp;
    const GradRec gr = a.grad[i];
    const SplatRec rec = a.rec[i];
    const float px = a.means[3 * i], py = a.means[3 * i + 1], pz = a.means[3 * i + 2];

    // project_pix_vjp
    const float *m = sp.projmat;
    const float hw = m[12] * px + m[13] * py + m[14] * pz + m[15];
    const float rw = 1.f / (hw + 1e-6f);
    const float vnx = 0.5f * a.Wf * gr.a.x, vny = 0.5f * a.Hf * gr.a.y;
    const float vp0 = vnx * rw, vp1 = vny * rw;
    float vm[3];
#pragma unroll
    for (int c = 0; c < 3; c++) vm[c] = m[c] * vp0 + m[4 + c] * vp1;

    // cov2d_to_conic_vjp: v_Sigma = -X G X
    const float X00 = rec.b.x, X01 = rec.b.y, X11 = rec.b.z;
    const float G00 = gr.b.x, G01 = gr.b.y, G11 = gr.b.z;
    const float XG00 = X00 * G00 + X01 * G01, XG01 = X00 * G01 + X01 * G11;
    const float XG10 = X01 * G00 + X11 * G01, XG11 = X01 * G01 + X11 * G11;
    const float VS00 = -(XG00 * X00 + XG01 * X01), VS01 = -(XG00 * X01 + XG01 * X11);
    const float VS10 = -(XG10 * X00 + XG11 * X01), VS11 = -(XG10 * X01 + XG11 * X11);
    const float vc_a = VS00, vc_b = VS10 + VS01, vc_c = VS11;

    // recompute cov3d
    float s[3];
#pragma unroll
    for (int k = 0; k < 3; k++) s[k] = det_expf(fminf(fmaxf(a.scales[3 * i + k], -15.f), 15.f));
    const float4 q = *reinterpret_cast<const float4 *>(a.quats + 4 * (size_t)i);
    const float qn = 1.0f / sqrtf(fmaxf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z, 1e-8f));
    const float w = q.x * qn, x = q.y * qn, y = q.z * qn, z = q.w * qn;
    float R[3][3];
    R[0][0] = 1.f - 2.f * (y * y + z * z); R[1][0] = 2.f * (x * y + w * z); R[2][0] = 2.f * (x * z - w * y);
    R[0][1] = 2.f * (x * y - w * z); R[1][1] = 1.f - 2.f * (x * x + z * z); R[2][1] = 2.f * (y * z + w * x);
    R[0][2] = 2.f * (x * z + w * y); R[1][2] = 2.f * (y * z - w * x); R[2][2] = 1.f - 2.f * (x * x + y * y);
    float M[3][3], V[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) M[r][c] = R[r][c] * s[c];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) V[r][c] = M[r][0] * M[c][0] + M[r][1] * M[c][1] + M[r][2] * M[c][2];

    // project_cov3d_ewa_vjp
    const float *v = sp.viewmat;
    const float vx = v[0] * px + v[1] * py + v[2] * pz + v[3];
    const float vy = v[4] * px + v[5] * py + v[6] * pz + v[7];
    const float vz = v[8] * px + v[9] * py + v[10] * pz + v[11];
    const float lim_x = 1.3f * sp.tan_fovx, lim_y = 1.3f * sp.tan_fovy;
    const float cvx = vz * fminf(lim_x, fmaxf(-lim_x, vx / vz));
    const float cvy = vz * fminf(lim_y, fmaxf(-lim_y, vy / vz));
    const float rz = 1.f / vz, rz2 = rz * rz, rz3 = rz2 * rz;
    float Wm[3][3], J[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) Wm[r][c] = v[4 * r + c];
    J[0][0] = sp.fx * rz; J[1][1] = sp.fy * rz;
    J[0][2] = -sp.fx * cvx * rz2; J[1][2] = -sp.fy * cvy * rz2;
    float Tm[3][3];
    mat3mul(J, Wm, Tm);
    // v_cov (symmetric, only the upper-left 2x2 non-zero)
    const float c00 = vc_a, c01 = 0.5f * vc_b, c11 = vc_c;
    // v_V = T^T v_cov T ; only rows 0,1 of T matter
    float vV[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float t0r = Tm[0][r], t1r = Tm[1][r];
            vV[r][c] = (t0r * c00 + t1r * c01) * Tm[0][c] + (t0r * c01 + t1r * c11) * Tm[1][c];
        }
    // v_T = v_cov T V^T + v_cov^T T V = 2 v_cov T V (V symmetric)
    float TV[3][3];
    mat3mul(Tm, V, TV);
    float vT[3][3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        vT[0][c] = 2.f * (c00 * TV[0][c] + c01 * TV[1][c]);
        vT[1][c] = 2.f * (c01 * TV[0][c] + c11 * TV[1][c]);
        vT[2][c] = 0.f;
    }
    // v_J = v_T W^T
    float vJ[2][3];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) vJ[r][c] = vT[r][0] * Wm[c][0] + vT[r][1] * Wm[c][1] + vT[r][2] * Wm[c][2];
    const float fxr = sp.fx * rz2, fyr = sp.fy * rz2;
    const float vt0 = -fxr * vJ[0][2], vt1 = -fyr * vJ[1][2];
    const float vt2 = -fxr * vJ[0][0] + 2.f * sp.fx * cvx * rz3 * vJ[0][2] - fyr * vJ[1][1] +
                      2.f * sp.fy * cvy * rz3 * vJ[1][2];
#pragma unroll
    for (int c = 0; c < 3; c++) vm[c] += vt0 * Wm[0][c] + vt1 * Wm[1][c] + vt2 * Wm[2][c];
    vmean[0] = vm[0]; vmean[1] = vm[1]; vmean[2] = vm[2];

    // scale_rot_to_cov3d_vjp + quat_to_rotmat_vjp
    const float v00 = vV[0][0], v01 = 0.5f * (vV[0][1] + vV[1][0]), v02 = 0.5f * (vV[0][2] + vV[2][0]);
    const float v11 = vV[1][1], v12 = 0.5f * (vV[1][2] + vV[2][1]), v22 = vV[2][2];
    const float vVs[3][3] = {{v00, v01, v02}, {v01, v11, v12}, {v02, v12, v22}};
    float vM[3][3];
    mat3mul(vVs, M, vM);
    float gR[3][3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float acc = 0.f;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            vM[r][c] *= 2.f;
            acc += R[r][c] * vM[r][c];
            gR[r][c] = vM[r][c] * s[c];
        }
        vscale[c] = acc * s[c];
    }
    // gR[row][col]; the reference indexes v_R[col][row]
    vquat[0] = 2.f * (x * (gR[2][1] - gR[1][2]) + y * (gR[0][2] - gR[2][0]) + z * (gR[1][0] - gR[0][1]));
    vquat[1] = 2.f * (-2.f * x * (gR[1][1] + gR[2][2]) + y * (gR[1][0] + gR[0][1]) + z * (gR[2][0] + gR[0][2]) +
                      w * (gR[2][1] - gR[1][2]));
    vquat[2] = 2.f * (x * (gR[1][0] + gR[0][1]) - 2.f * y * (gR[0][0] + gR[2][2]) + z * (gR[2][1] + gR[1][2]) +
                      w * (gR[0][2] - gR[2][0]));
    vquat[3] = 2.f * (x * (gR[2][0] + gR[0][2]) + y * (gR[2][1] + gR[1][2]) - 2.f * z * (gR[0][0] + gR[1][1]) +
                      w * (gR[1][0] - gR[0][1]));

    // fused SH backward + Adam
    if (!a.do_optimizer) return;
    const float vc0 = gr.c.x, vc1 = gr.c.y, vc2 = gr.c.z;
    if (!(finite_bits(vc0) && finite_bits(vc1) && finite_bits(vc2))) {
        if (a.nan_counts) atomicAdd(a.nan_counts + kNanSH, 1u);
        return;
    }
    const float b1 = sp.beta1, b2 = sp.beta2, eps = sp.eps;
    {
        float *p = a.features_dc + 3 * (size_t)i, *mm = a.dc_m + 3 * (size_t)i, *vv = a.dc_v + 3 * (size_t)i;
        adam_el(p + 0, mm + 0, vv + 0, kBC0 * vc0, sp.step_size[3], sp.bc2_sqrt[3], b1, b2, eps);
        adam_el(p + 1, mm + 1, vv + 1, kBC0 * vc1, sp.step_size[3], sp.bc2_sqrt[3], b1, b2, eps);
        adam_el(p + 2, mm + 2, vv + 2, kBC0 * vc2, sp.step_size[3], sp.bc2_sqrt[3], b1, b2, eps);
    }
    const int deg = sp.degrees_to_use;
    int nb = deg >= 3 ? 15 : deg == 2 ? 8 : deg == 1 ? 3 : 0;
    nb = min(nb, a.rest_bases);
    if (nb == 0) return;
    const float dx = px - sp.cam_pos[0], dy = py - sp.cam_pos[1], dz = pz - sp.cam_pos[2];
    const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
    const float X = dx * inv, Y = dy * inv, Z = dz * inv;
    const float xx = X * X, xy = X * Y, xz = X * Z, yy = Y * Y, yz = Y * Z, zz = Z * Z;
    float bas[15];
    bas[0] = -kBC1 * Y; bas[1] = kBC1 * Z; bas[2] = -kBC1 * X;
    bas[3] = kBC2[0] * xy; bas[4] = kBC2[1] * yz; bas[5] = kBC2[2] * (2.f * zz - xx - yy);
    bas[6] = kBC2[3] * xz; bas[7] = kBC2[4] * (xx - yy);
    bas[8] = kBC3[0] * Y * (3.f * xx - yy); bas[9] = kBC3[1] * xy * Z;
    bas[10] = kBC3[2] * Y * (4.f * zz - xx - yy); bas[11] = kBC3[3] * Z * (2.f * zz - 3.f * xx - 3.f * yy);
    bas[12] = kBC3[4] * X * (4.f * zz - xx - yy); bas[13] = kBC3[5] * Z * (xx - yy);
    bas[14] = kBC3[6] * X * (xx - 3.f * yy);
    const size_t base = (size_t)a.rest_bases * 3 * i;
    float *p = a.features_rest + base, *mm = a.rest_m + base, *vv = a.rest_v + base;
    const float st = sp.step_size[4], bc = sp.bc2_sqrt[4];
#pragma unroll 1
    for (int b = 0; b < nb; b++) {
        adam_el(p + 3 * b + 0, mm + 3 * b + 0, vv + 3 * b + 0, bas[b] * vc0, st, bc, b1, b2, eps);
        adam_el(p + 3 * b + 1, mm + 3 * b + 1, vv + 3 * b + 1, bas[b] * vc1, st, bc, b1, b2, eps);
        adam_el(p + 3 * b + 2, mm + 3 * b + 2, vv + 3 * b + 2, bas[b] * vc2, st, bc, b1, b2, eps);
    }
}

void launch_project_bwd(const ProjectBwdArgs &a, cudaStream_t s) {
    if (a.n <= 0) return;
    k_project_bwd<<<(a.n + 255) / 256, 256, 0, s>>>(a);
}

}  // namespace msplat
