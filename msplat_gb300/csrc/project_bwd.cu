// Projection VJP (centre, conic -> mean, log-scale, quaternion) with the SH
// colour VJP fused straight into Adam for features_dc / features_rest, one
// thread per Gaussian.  The 3D covariance is recomputed in registers.  With
// several views the thread walks the Gaussian's record in each view and
// sums the gradients (the views' image gradients already carry 1/views), so
// one launch ends the backward of the whole step and the SH Adam sees the
// summed gradient.
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
    *p -= adam_delta(step, mm, vv, bc2s, eps);
    *m = mm;
    *v = vv;
}

__device__ __forceinline__ void adam4(float4 &p, float4 &m, float4 &v, const float g[4], unsigned active, float st,
                                      float bc, float b1, float b2, float eps) {
    float *pp = &p.x, *mm = &m.x, *vv = &v.x;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (!(active & (1u << k))) continue;
        const float nm = fmaf(b1, mm[k], (1.0f - b1) * g[k]);
        const float nv = fmaf(b2, vv[k], (1.0f - b2) * g[k] * g[k]);
        pp[k] -= adam_delta(st, nm, nv, bc, eps);
        mm[k] = nm;
        vv[k] = nv;
    }
}


// Per-warp staging of the SH gradients: the warp's 32 Gaussians' rows of
// dL/d(features_rest) and dL/d(features_dc), laid out exactly like their rows
// in global memory (so the walk reads the gradient of element e at offset e),
// kInactive in the slots of elements Adam leaves alone (culled Gaussian,
// non-finite colour gradient, band not in use).  The row stride of 45 floats
// keeps the 32 lanes writing their own rows on distinct banks.
constexpr uint32_t kInactive = 0xffffffffu;
struct ShFlat {
    float rest[32 * 45];
    float dc[32 * 3];
};

__device__ __forceinline__ bool active_slot(float g) { return __float_as_uint(g) != kInactive; }

// View-independent state of one Gaussian: mean, scales, normalised
// quaternion, rotation, M = R S and the 3D covariance V = M M^T.
struct CovState {
    float px, py, pz;
    float s[3];
    float w, x, y, z;
    float R[3][3], M[3][3], V[3][3];
};

__device__ __forceinline__ void cov_state(const ProjectBwdArgs &a, int i, CovState &cs) {
    cs.px = a.means[3 * i]; cs.py = a.means[3 * i + 1]; cs.pz = a.means[3 * i + 2];
#pragma unroll
    for (int k = 0; k < 3; k++) cs.s[k] = det_expf(fminf(fmaxf(a.scales[3 * i + k], -15.f), 15.f));
    const float4 q = *reinterpret_cast<const float4 *>(a.quats + 4 * (size_t)i);
    const float qn = 1.0f / sqrtf(fmaxf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z, 1e-8f));
    const float w = q.x * qn, x = q.y * qn, y = q.z * qn, z = q.w * qn;
    cs.w = w; cs.x = x; cs.y = y; cs.z = z;
    float (&R)[3][3] = cs.R;
    R[0][0] = 1.f - 2.f * (y * y + z * z); R[1][0] = 2.f * (x * y + w * z); R[2][0] = 2.f * (x * z - w * y);
    R[0][1] = 2.f * (x * y - w * z); R[1][1] = 1.f - 2.f * (x * x + z * z); R[2][1] = 2.f * (y * z + w * x);
    R[0][2] = 2.f * (x * z + w * y); R[1][2] = 2.f * (y * z - w * x); R[2][2] = 1.f - 2.f * (x * x + y * y);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) cs.M[r][c] = R[r][c] * cs.s[c];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            cs.V[r][c] = cs.M[r][0] * cs.M[c][0] + cs.M[r][1] * cs.M[c][1] + cs.M[r][2] * cs.M[c][2];
}

// First half of one view's VJP, before the 3D covariance is needed:
// project_pix_vjp (dL/dmean through the projected centre, gm) and
// cov2d_to_conic_vjp (v_Sigma = -X G X, symmetric part c00, c01, c11).
struct PixConicVjp {
    float gm[3];
    float c00, c01, c11;
};

__device__ __forceinline__ PixConicVjp pix_conic_vjp(float px, float py, float pz, const StepParams &sp, float Wf,
                                                     float Hf, const GradRec &gr, const SplatRec &rec) {
    PixConicVjp o;
    const float *m = sp.projmat;
    const float hw = m[12] * px + m[13] * py + m[14] * pz + m[15];
    const float rw = 1.f / (hw + 1e-6f);
    const float vnx = 0.5f * Wf * gr.a.x, vny = 0.5f * Hf * gr.a.y;
    const float vp0 = vnx * rw, vp1 = vny * rw;
#pragma unroll
    for (int c = 0; c < 3; c++) o.gm[c] = m[c] * vp0 + m[4 + c] * vp1;
    const float X00 = rec.b.x, X01 = rec.b.y, X11 = rec.b.z;
    const float G00 = gr.b.x, G01 = gr.b.y, G11 = gr.b.z;
    const float XG00 = X00 * G00 + X01 * G01, XG01 = X00 * G01 + X01 * G11;
    const float XG10 = X01 * G00 + X11 * G01, XG11 = X01 * G01 + X11 * G11;
    const float VS00 = -(XG00 * X00 + XG01 * X01), VS01 = -(XG00 * X01 + XG01 * X11);
    const float VS10 = -(XG10 * X00 + XG11 * X01), VS11 = -(XG10 * X01 + XG11 * X11);
    o.c00 = VS00;
    o.c01 = 0.5f * (VS10 + VS01);
    o.c11 = VS11;
    return o;
}

// Second half (project_cov3d_ewa_vjp, scale_rot_to_cov3d_vjp,
// quat_to_rotmat_vjp); the whole VJP is added into vm, vsc, vq.
__device__ __forceinline__ void cov_vjp(const CovState &cs, const StepParams &sp, const PixConicVjp &pc, float vm[3],
                                        float vsc[3], float vq[4]) {
    const float px = cs.px, py = cs.py, pz = cs.pz;
    const float *gm = pc.gm;
    const float c00 = pc.c00, c01 = pc.c01, c11 = pc.c11;

    // project_cov3d_ewa_vjp
    const float *v = sp.viewmat;
    const float vx = v[0] * px + v[1] * py + v[2] * pz + v[3];
    const float vy = v[4] * px + v[5] * py + v[6] * pz + v[7];
    const float vz = v[8] * px + v[9] * py + v[10] * pz + v[11];
    const float lim_x = 1.3f * sp.tan_fovx, lim_y = 1.3f * sp.tan_fovy;
    const float cvx = vz * fminf(lim_x, fmaxf(-lim_x, vx / vz));
    const float cvy = vz * fminf(lim_y, fmaxf(-lim_y, vy / vz));
    const float rz = 1.f / vz, rz2 = rz * rz, rz3 = rz2 * rz;
    // rows 0, 1 of T = J W (row 2 of J is zero)
    const float j00 = sp.fx * rz, j11 = sp.fy * rz, j02 = -sp.fx * cvx * rz2, j12 = -sp.fy * cvy * rz2;
    float T0[3], T1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        T0[c] = j00 * v[c] + j02 * v[8 + c];
        T1[c] = j11 * v[4 + c] + j12 * v[8 + c];
    }
    // v_V = T^T v_cov T
    float vV[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            vV[r][c] = (T0[r] * c00 + T1[r] * c01) * T0[c] + (T0[r] * c01 + T1[r] * c11) * T1[c];
    // v_T = 2 v_cov T V (rows 0, 1), v_J = v_T W^T
    float TV0[3], TV1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        TV0[c] = T0[0] * cs.V[0][c] + T0[1] * cs.V[1][c] + T0[2] * cs.V[2][c];
        TV1[c] = T1[0] * cs.V[0][c] + T1[1] * cs.V[1][c] + T1[2] * cs.V[2][c];
    }
    float vT0[3], vT1[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        vT0[c] = 2.f * (c00 * TV0[c] + c01 * TV1[c]);
        vT1[c] = 2.f * (c01 * TV0[c] + c11 * TV1[c]);
    }
    const float vJ00 = vT0[0] * v[0] + vT0[1] * v[1] + vT0[2] * v[2];
    const float vJ02 = vT0[0] * v[8] + vT0[1] * v[9] + vT0[2] * v[10];
    const float vJ11 = vT1[0] * v[4] + vT1[1] * v[5] + vT1[2] * v[6];
    const float vJ12 = vT1[0] * v[8] + vT1[1] * v[9] + vT1[2] * v[10];
    const float fxr = sp.fx * rz2, fyr = sp.fy * rz2;
    const float vt0 = -fxr * vJ02, vt1 = -fyr * vJ12;
    const float vt2 = -fxr * vJ00 + 2.f * sp.fx * cvx * rz3 * vJ02 - fyr * vJ11 + 2.f * sp.fy * cvy * rz3 * vJ12;
#pragma unroll
    for (int c = 0; c < 3; c++) vm[c] += gm[c] + (vt0 * v[c] + vt1 * v[4 + c] + vt2 * v[8 + c]);

    // scale_rot_to_cov3d_vjp + quat_to_rotmat_vjp
    const float v01 = 0.5f * (vV[0][1] + vV[1][0]), v02 = 0.5f * (vV[0][2] + vV[2][0]);
    const float v12 = 0.5f * (vV[1][2] + vV[2][1]);
    const float vVs[3][3] = {{vV[0][0], v01, v02}, {v01, vV[1][1], v12}, {v02, v12, vV[2][2]}};
    float gR[3][3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float acc = 0.f;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            const float vMrc = 2.f * (vVs[r][0] * cs.M[0][c] + vVs[r][1] * cs.M[1][c] + vVs[r][2] * cs.M[2][c]);
            acc += cs.R[r][c] * vMrc;
            gR[r][c] = vMrc * cs.s[c];
        }
        vsc[c] += acc * cs.s[c];
    }
    // gR[row][col]; the reference indexes v_R[col][row]
    const float w = cs.w, x = cs.x, y = cs.y, z = cs.z;
    vq[0] += 2.f * (x * (gR[2][1] - gR[1][2]) + y * (gR[0][2] - gR[2][0]) + z * (gR[1][0] - gR[0][1]));
    vq[1] += 2.f * (-2.f * x * (gR[1][1] + gR[2][2]) + y * (gR[1][0] + gR[0][1]) + z * (gR[2][0] + gR[0][2]) +
                    w * (gR[2][1] - gR[1][2]));
    vq[2] += 2.f * (x * (gR[1][0] + gR[0][1]) - 2.f * y * (gR[0][0] + gR[2][2]) + z * (gR[2][1] + gR[1][2]) +
                    w * (gR[0][2] - gR[2][0]));
    vq[3] += 2.f * (x * (gR[2][0] + gR[0][2]) + y * (gR[2][1] + gR[1][2]) - 2.f * z * (gR[0][0] + gR[1][1]) +
                    w * (gR[1][0] - gR[0][1]));
}

// SH basis (bands 1..3 in b[0..14], the DC constant in b[15]) of the
// direction from the camera to the Gaussian
__device__ __forceinline__ void sh_basis(const CovState &cs, const StepParams &sp, float b[16]) {
    const float dx = cs.px - sp.cam_pos[0], dy = cs.py - sp.cam_pos[1], dz = cs.pz - sp.cam_pos[2];
    const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
    const float X = dx * inv, Y = dy * inv, Z = dz * inv;
    const float xx = X * X, xy = X * Y, xz = X * Z, yy = Y * Y, yz = Y * Z, zz = Z * Z;
    b[0] = -kBC1 * Y; b[1] = kBC1 * Z; b[2] = -kBC1 * X;
    b[3] = kBC2[0] * xy; b[4] = kBC2[1] * yz; b[5] = kBC2[2] * (2.f * zz - xx - yy);
    b[6] = kBC2[3] * xz; b[7] = kBC2[4] * (xx - yy);
    b[8] = kBC3[0] * Y * (3.f * xx - yy); b[9] = kBC3[1] * xy * Z;
    b[10] = kBC3[2] * Y * (4.f * zz - xx - yy); b[11] = kBC3[3] * Z * (2.f * zz - 3.f * xx - 3.f * yy);
    b[12] = kBC3[4] * X * (4.f * zz - xx - yy); b[13] = kBC3[5] * Z * (xx - yy);
    b[14] = kBC3[6] * X * (xx - 3.f * yy);
    b[15] = kBC0;
}

__device__ __forceinline__ int bands_in_use(const StepParams &sp, int rest_bases) {
    const int deg = sp.degrees_to_use;
    const int nb = deg >= 3 ? 15 : deg == 2 ? 8 : deg == 1 ? 3 : 0;
    return min(nb, rest_bases);
}

// Fused SH Adam (or the gradient export), warp-cooperative: the warp's 32
// Gaussians own contiguous rows of features_dc / features_rest and their
// moments, walked with coalesced 16-byte accesses; the gradient of element e
// is slot e of the staged rows.
template <int kRowF>
__device__ __forceinline__ void sh_update(const ProjectBwdArgs &a, const StepParams &sp, const ShFlat &st, int i0,
                                          int ng, int lane) {
    const int rowf = kRowF > 0 ? kRowF : 3 * a.rest_bases;
    if (a.v_dc_out) {
        // export: zero where Adam would not update
        for (int e = lane; e < 3 * ng; e += 32) {
            const float g = st.dc[e];
            a.v_dc_out[3 * (size_t)i0 + e] = active_slot(g) ? g : 0.f;
        }
        for (int e = lane; e < rowf * ng; e += 32) {
            const float g = st.rest[e];
            a.v_rest_out[(size_t)rowf * i0 + e] = active_slot(g) ? g : 0.f;
        }
        return;
    }
    const float b1 = sp.beta1, b2 = sp.beta2, eps = sp.eps;
    {   // features_dc: 3 floats per Gaussian
        const int total = 3 * ng;
        float *p = a.features_dc + 3 * (size_t)i0, *mm = a.dc_m + 3 * (size_t)i0, *vv = a.dc_v + 3 * (size_t)i0;
        const float stp = sp.step_size[3], bc = sp.bc2_sqrt[3];
        for (int e0 = lane * 4; e0 < total; e0 += 128) {
            float g[4];
            unsigned act = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                g[k] = e0 + k < total ? st.dc[e0 + k] : __uint_as_float(kInactive);
                if (active_slot(g[k])) act |= 1u << k;
            }
            if (!act) continue;
            if (e0 + 4 <= total) {
                float4 P = *reinterpret_cast<float4 *>(p + e0), Mv = *reinterpret_cast<float4 *>(mm + e0),
                       Vv = *reinterpret_cast<float4 *>(vv + e0);
                adam4(P, Mv, Vv, g, act, stp, bc, b1, b2, eps);
                *reinterpret_cast<float4 *>(p + e0) = P;
                *reinterpret_cast<float4 *>(mm + e0) = Mv;
                *reinterpret_cast<float4 *>(vv + e0) = Vv;
            } else {
                for (int k = 0; k < 4 && e0 + k < total; k++)
                    if (act & (1u << k)) adam_el(p + e0 + k, mm + e0 + k, vv + e0 + k, g[k], stp, bc, b1, b2, eps);
            }
        }
    }
    if (a.rest_bases == 0) return;
    {   // features_rest: rowf floats per Gaussian; kRestUnroll 16-byte steps
        // per lane are loaded before any is updated, so a warp keeps
        // 3 * kRestUnroll loads in flight
        constexpr int kRestUnroll = 3;
        const int total = rowf * ng;
        float *p = a.features_rest + (size_t)rowf * i0, *mm = a.rest_m + (size_t)rowf * i0,
              *vv = a.rest_v + (size_t)rowf * i0;
        const float stp = sp.step_size[4], bc = sp.bc2_sqrt[4];
        for (int base = lane * 4; base < total; base += 128 * kRestUnroll) {
            float4 P[kRestUnroll], Mv[kRestUnroll], Vv[kRestUnroll];
#pragma unroll
            for (int u = 0; u < kRestUnroll; u++) {
                const int e0 = base + 128 * u;
                if (e0 + 4 <= total) {
                    P[u] = *reinterpret_cast<const float4 *>(p + e0);
                    Mv[u] = *reinterpret_cast<const float4 *>(mm + e0);
                    Vv[u] = *reinterpret_cast<const float4 *>(vv + e0);
                }
            }
#pragma unroll
            for (int u = 0; u < kRestUnroll; u++) {
                const int e0 = base + 128 * u;
                if (e0 >= total) break;
                float g[4];
                unsigned act = 0;
                if (e0 + 4 <= total) {
                    const float4 g4 = *reinterpret_cast<const float4 *>(st.rest + e0);
                    g[0] = g4.x; g[1] = g4.y; g[2] = g4.z; g[3] = g4.w;
                } else {
#pragma unroll
                    for (int k = 0; k < 4; k++) g[k] = e0 + k < total ? st.rest[e0 + k] : __uint_as_float(kInactive);
                }
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (active_slot(g[k])) act |= 1u << k;
                if (!act) continue;
                if (e0 + 4 <= total) {
                    adam4(P[u], Mv[u], Vv[u], g, act, stp, bc, b1, b2, eps);
                    *reinterpret_cast<float4 *>(p + e0) = P[u];
                    *reinterpret_cast<float4 *>(mm + e0) = Mv[u];
                    *reinterpret_cast<float4 *>(vv + e0) = Vv[u];
                } else {
                    for (int k = 0; k < 4 && e0 + k < total; k++)
                        if (act & (1u << k)) adam_el(p + e0 + k, mm + e0 + k, vv + e0 + k, g[k], stp, bc, b1, b2, eps);
                }
            }
        }
    }
}

// Stage one Gaussian's SH gradient rows (this lane's): dc[c] = C0 * vc_c,
// rest[3 band + c] = basis_band * vc_c for bands below nb, the other rest
// slots inactive.
template <int kRowF>
__device__ __forceinline__ void stage_sh_row(ShFlat &st, int lane, int rest_bases, int nb, const float b[16],
                                             float vc0, float vc1, float vc2) {
    const int rowf = kRowF > 0 ? kRowF : 3 * rest_bases;
    float *gd = st.dc + 3 * lane, *gr = st.rest + rowf * lane;
    const float off = __uint_as_float(kInactive);
    gd[0] = b[15] * vc0;
    gd[1] = b[15] * vc1;
    gd[2] = b[15] * vc2;
#pragma unroll
    for (int band = 0; band < 15; band++) {
        if (band >= rest_bases) break;
        const bool on = band < nb;
        gr[3 * band + 0] = on ? b[band] * vc0 : off;
        gr[3 * band + 1] = on ? b[band] * vc1 : off;
        gr[3 * band + 2] = on ? b[band] * vc2 : off;
    }
}

// Every slot of this lane's rows inactive.
template <int kRowF> __device__ __forceinline__ void stage_sh_inactive(ShFlat &st, int lane, int rest_bases) {
    const int rowf = kRowF > 0 ? kRowF : 3 * rest_bases;
    float *gd = st.dc + 3 * lane, *gr = st.rest + rowf * lane;
    const float off = __uint_as_float(kInactive);
    gd[0] = gd[1] = gd[2] = off;
    for (int k = 0; k < rowf; k++) gr[k] = off;
}

// One view.  kRowF: floats per features_rest row when known at compile time
// (45 for SH degree 3), so the element -> (Gaussian, band, channel)
// arithmetic of the SH walk uses constant divisors; 0 reads it from the
// arguments.
template <int kRowF>
__global__ void __launch_bounds__(256, 4) k_project_bwd(ProjectBwdArgs a) {
    pdl_enter();
    const int n = a.vt.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const StepParams &sp = a.sp[0];
    const bool want_sh = a.do_optimizer || a.v_dc_out;
    float *vmean = a.v_mean + 3 * (size_t)i, *vscale = a.v_scale + 3 * (size_t)i, *vquat = a.v_quat + 4 * (size_t)i;
    if (a.v_opac_out) a.v_opac_out[i] = a.radii[i] > 0 ? a.grad[i].a.z : 0.f;
    if (a.gstats) {
        float4 st = a.gstats[i];
        st.z += 1.f;
        if (a.radii[i] > 0) {
            const float4 g0 = a.grad[i].a;
            st.x += sqrtf(g0.x * g0.x + g0.y * g0.y);
            st.y += 1.f;
        }
        a.gstats[i] = st;
    }
    float vm[3] = {0.f, 0.f, 0.f}, vsc[3] = {0.f, 0.f, 0.f}, vq[4] = {0.f, 0.f, 0.f, 0.f};
    float4 shin = make_float4(0.f, 0.f, 0.f, __int_as_float(0));   // colour gradient, w = 1 when it feeds SH
    // every input read before the visibility test, so the loads are in
    // flight together (a culled Gaussian's are not used)
    const int rad = a.radii[i];
    const GradRec gr = a.grad[i];
    const SplatRec rc = a.rec[i];
    const float mx = a.means[3 * i], my = a.means[3 * i + 1], mz = a.means[3 * i + 2];
    CovState cs;
    cov_state(a, i, cs);
    if (rad > 0) {
        const PixConicVjp pc = pix_conic_vjp(mx, my, mz, sp, (float)a.vt.width[0], (float)a.vt.height[0], gr, rc);
        cov_vjp(cs, sp, pc, vm, vsc, vq);
        if (want_sh) {
            if (!(finite_bits(gr.c.x) && finite_bits(gr.c.y) && finite_bits(gr.c.z))) {
                if (a.nan_counts) atomicAdd(a.nan_counts + kNanSH, 1u);
            } else {
                shin = make_float4(gr.c.x, gr.c.y, gr.c.z, __int_as_float(1));
            }
        }
    }
    vmean[0] = vm[0]; vmean[1] = vm[1]; vmean[2] = vm[2];
    vscale[0] = vsc[0]; vscale[1] = vsc[1]; vscale[2] = vsc[2];
    *reinterpret_cast<float4 *>(vquat) = make_float4(vq[0], vq[1], vq[2], vq[3]);
    if (want_sh) a.sh_in[i] = shin;
}

// The SH Adam (or the gradient export) of one view, after the projection
// VJP: each lane recomputes its Gaussian's SH basis from the mean and the
// camera, stages its gradient rows, and the warp walks the rows of its 32
// Gaussians.
template <int kRowF>
__global__ void __launch_bounds__(128) k_sh_walk(ProjectBwdArgs a) {
    pdl_enter();
    __shared__ __align__(16) ShFlat stage[4];
    const int n = a.vt.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int i0 = blockIdx.x * blockDim.x + wid * 32;
    if (i0 >= n) return;   // warp-uniform
    ShFlat &sh = stage[wid];
    const StepParams &sp = a.sp[0];
    if (i < n) {
        const float4 shin = a.sh_in[i];
        if (__float_as_int(shin.w)) {
            CovState cs;   // only the mean is used by the basis
            cs.px = a.means[3 * i]; cs.py = a.means[3 * i + 1]; cs.pz = a.means[3 * i + 2];
            float b[16];
            sh_basis(cs, sp, b);
            stage_sh_row<kRowF>(sh, lane, a.rest_bases, bands_in_use(sp, a.rest_bases), b, shin.x, shin.y, shin.z);
        } else {
            stage_sh_inactive<kRowF>(sh, lane, a.rest_bases);
        }
    }
    __syncwarp();
    sh_update<kRowF>(a, sp, sh, i0, min(32, n - i0), lane);
}

// Several views: the thread walks the Gaussian's record in every view of the
// step and sums; the SH gradients are summed in shared memory; v_opac gets the
// summed opacity-logit gradient.  A Gaussian visible in no view gets zero
// gradients and no SH update.
template <int kRowF>
__global__ void __launch_bounds__(128, 4) k_project_bwd_views(ProjectBwdArgs a) {
    pdl_enter();
    __shared__ __align__(16) ShFlat stage[4];
    const int n = a.vt.n, views = a.vt.count;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    ShFlat &sh = stage[wid];
    const StepParams &sp0 = a.sp[0];
    const int rowf = kRowF > 0 ? kRowF : 3 * a.rest_bases;
    const int nb = bands_in_use(sp0, a.rest_bases);
    float *gd = sh.dc + 3 * lane, *gr = sh.rest + rowf * lane;   // this lane's rows: summed over the views
    gd[0] = gd[1] = gd[2] = 0.f;
    for (int k = 0; k < rowf; k++) gr[k] = 0.f;
    bool sh_ok = false;
    if (i < n) {
        float vm[3] = {0.f, 0.f, 0.f}, vsc[3] = {0.f, 0.f, 0.f}, vq[4] = {0.f, 0.f, 0.f, 0.f};
        float vop = 0.f, act_xy = 0.f, act_vis = 0.f;
        bool any = false;
        CovState cs;
        for (int v = 0; v < views; v++) {
            const size_t u = (size_t)v * n + i;
            if (a.radii[u] <= 0) continue;
            if (!any) { cov_state(a, i, cs); any = true; }
            const GradRec g = a.grad[u];
            const StepParams &sp = a.sp[v];
            vop += g.a.z;
            act_xy += sqrtf(g.a.x * g.a.x + g.a.y * g.a.y);
            act_vis += 1.f;
            const ViewGeom vg = view_geom(a.vt, v);
            const PixConicVjp pc = pix_conic_vjp(cs.px, cs.py, cs.pz, sp, (float)vg.width, (float)vg.height, g, a.rec[u]);
            cov_vjp(cs, sp, pc, vm, vsc, vq);
            const float vc0 = g.c.x, vc1 = g.c.y, vc2 = g.c.z;
            if (!(finite_bits(vc0) && finite_bits(vc1) && finite_bits(vc2))) {
                if (a.nan_counts) atomicAdd(a.nan_counts + kNanSH, 1u);
                continue;
            }
            float b[16];
            sh_basis(cs, sp, b);
            gd[0] += b[15] * vc0; gd[1] += b[15] * vc1; gd[2] += b[15] * vc2;
            for (int k = 0; k < nb; k++) {
                gr[3 * k] += b[k] * vc0;
                gr[3 * k + 1] += b[k] * vc1;
                gr[3 * k + 2] += b[k] * vc2;
            }
            sh_ok = true;
        }
        float *vmean = a.v_mean + 3 * (size_t)i, *vscale = a.v_scale + 3 * (size_t)i, *vquat = a.v_quat + 4 * (size_t)i;
        vmean[0] = vm[0]; vmean[1] = vm[1]; vmean[2] = vm[2];
        vscale[0] = vsc[0]; vscale[1] = vsc[1]; vscale[2] = vsc[2];
        *reinterpret_cast<float4 *>(vquat) = make_float4(vq[0], vq[1], vq[2], vq[3]);
        a.v_opac[i] = vop;
        if (a.gstats) {
            float4 st = a.gstats[i];
            st.x += act_xy;
            st.y += act_vis;
            st.z += 1.f;
            a.gstats[i] = st;
        }
    }
    // slots Adam leaves alone: every slot without a finite visible view, and
    // the bands not in use
    const float off = __uint_as_float(kInactive);
    if (!sh_ok) {
        gd[0] = gd[1] = gd[2] = off;
        for (int k = 0; k < rowf; k++) gr[k] = off;
    } else {
        for (int k = 3 * nb; k < rowf; k++) gr[k] = off;
    }
    if (!a.do_optimizer) return;
    __syncwarp();
    const int i0 = (blockIdx.x * blockDim.x) + wid * 32;
    if (i0 >= n) return;
    sh_update<kRowF>(a, sp0, sh, i0, min(32, n - i0), lane);
}

void launch_project_bwd(const ProjectBwdArgs &a, cudaStream_t s) {
    const int n = a.vt.n;
    if (n <= 0) return;
    if (a.vt.count > 1) {
        if (a.rest_bases == 15) launch_pdl(k_project_bwd_views<45>, (n + 127) / 128, 128, 0, s, a);
        else launch_pdl(k_project_bwd_views<0>, (n + 127) / 128, 128, 0, s, a);
        return;
    }
    if (a.rest_bases == 15) launch_pdl(k_project_bwd<45>, (n + 255) / 256, 256, 0, s, a);
    else launch_pdl(k_project_bwd<0>, (n + 255) / 256, 256, 0, s, a);
    if (a.do_optimizer || a.v_dc_out) {
        if (a.rest_bases == 15) launch_pdl(k_sh_walk<45>, (n + 127) / 128, 128, 0, s, a);
        else launch_pdl(k_sh_walk<0>, (n + 127) / 128, 128, 0, s, a);
    }
}

}  // namespace msplat
