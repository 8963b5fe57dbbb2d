// Fused EWA projection + spherical-harmonics colour, one thread per
// (Gaussian, view): blockIdx.y is the view, records land at v * n + i.
// Follows project_and_sh_forward_kernel (msplat_metal.metal:1719-1834) and its
// helpers (:53-344, :620-687).  Built with --fmad=false: every float operation
// is rounded on its own, in the order the reference writes it, so radii, tile
// rectangles and depths (and therefore the tile lists) are bit-identical to
// the oracle's float path.
#include "common.cuh"
#include "kernels.h"
#include "tcgen05.cuh"

namespace msplat {

__constant__ float kShC0 = 0.28209479177387814f;
__constant__ float kShC1 = 0.4886025119029199f;
__constant__ float kShC2[5] = {1.0925484305920792f, -1.0925484305920792f, 0.31539156525252005f,
                               -1.0925484305920792f, 0.5462742152960396f};
__constant__ float kShC3[7] = {-0.5900435899266435f, 2.890611442640554f, -0.4570457994644658f,
                               0.3731763325901154f, -0.4570457994644658f, 1.445305721320277f,
                               -0.5900435899266435f};

// Reach of a splat, (hx, hy): the half-extents of a box around its centre
// outside which no pixel passes the rasterizers' tests sigma in [0, 5.55)
// and opacity * exp(-sigma) >= 1/255 (warp_reach turns it into the warps of
// a tile that the splat can touch).
//  - alpha >= 1/255 needs sigma <= ln(255 opacity); s = min(5.55, that)
//    + 1e-4 covers the rounding of the exponential, the product and the log.
//  - The rasterizers' rounded sigma is within 3.5 u (a dx^2 + c dy^2) of the
//    exact quadratic form (u = 2^-24; |b dx dy| <= (a dx^2 + c dy^2) / 2 for a
//    positive-definite conic), so rounded sigma <= s implies the exact form
//    of the conic with a and c shrunk by 1e-5 is <= s.  That ellipse's box is
//    sqrt(2 s c' / det'), sqrt(2 s a' / det'), det' by Kahan's fma
//    determinant (relative error 2 u), widened by 1e-5 for the rounding of
//    the box, of the rasterizers' dx, dy and of the shrink itself.
//  - Unbounded (+inf) unless the centre and conic are finite and moderate
//    (then no sigma can overflow, and every pair a warp skips had a finite
//    sigma); empty (-1) when s < 0.
__device__ __forceinline__ float2 reach_extent(float x, float y, float opac, float ca, float cb, float cc) {
    const float inf = __int_as_float(0x7f800000);
    const bool moderate = fabsf(x) <= 1e8f && fabsf(y) <= 1e8f && fabsf(ca) <= 1e20f && fabsf(cb) <= 1e20f &&
                          fabsf(cc) <= 1e20f;   // false for NaN
    if (!moderate) return make_float2(inf, inf);
    const float s = fminf(5.55f, logf(255.f * opac)) + 1e-4f;
    if (!(s >= 0.f)) return make_float2(-1.f, -1.f);
    const float a = ca * (1.f - 1e-5f), c = cc * (1.f - 1e-5f);
    if (!(a > 0.f && c > 0.f)) return make_float2(inf, inf);
    const float w = cb * cb;
    const float det = fmaf(a, c, -w) + fmaf(-cb, cb, w);
    if (!(det > 0.f)) return make_float2(inf, inf);
    const float k = 2.f * s / det;
    return make_float2(sqrtf(k * c) * (1.f + 1e-5f), sqrtf(k * a) * (1.f + 1e-5f));
}

// SH colour from the first deg bands (rest: the Gaussian's [15, 3] block, in
// shared or global memory), in the reference's operation order.
__device__ __forceinline__ void sh_colour(const float *dc, const float *rest, int deg, float vdx, float vdy,
                                          float vdz, float col[3]) {
    const float xx = vdx * vdx, xy = vdx * vdy, xz = vdx * vdz, yy = vdy * vdy, yz = vdy * vdz, zz = vdz * vdz;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float val = kShC0 * dc[c];
        if (deg >= 1) {
            val += kShC1 * (-vdy * rest[0 * 3 + c] + vdz * rest[1 * 3 + c] - vdx * rest[2 * 3 + c]);
            if (deg >= 2) {
                val += (kShC2[0] * xy * rest[3 * 3 + c] + kShC2[1] * yz * rest[4 * 3 + c] +
                        kShC2[2] * (2.f * zz - xx - yy) * rest[5 * 3 + c] + kShC2[3] * xz * rest[6 * 3 + c] +
                        kShC2[4] * (xx - yy) * rest[7 * 3 + c]);
                if (deg >= 3) {
                    val += (kShC3[0] * vdy * (3.f * xx - yy) * rest[8 * 3 + c] + kShC3[1] * xy * vdz * rest[9 * 3 + c] +
                            kShC3[2] * vdy * (4.f * zz - xx - yy) * rest[10 * 3 + c] +
                            kShC3[3] * vdz * (2.f * zz - 3.f * xx - 3.f * yy) * rest[11 * 3 + c] +
                            kShC3[4] * vdx * (4.f * zz - xx - yy) * rest[12 * 3 + c] +
                            kShC3[5] * vdz * (xx - yy) * rest[13 * 3 + c] +
                            kShC3[6] * vdx * (xx - 3.f * yy) * rest[14 * 3 + c]);
                }
            }
        }
        col[c] = val;
    }
}

constexpr int kStageFloats = 45;   // 15 SH bases x 3 channels per Gaussian

// One Gaussian's projection (the body of the kernel below).  rest: its SH
// row staged in shared memory when `staged`; with `bulk` the row arrives by
// the warp's bulk copy, which is waited for (bounded) before it is read.
template <bool kViews>
__device__ __forceinline__ void project_one(const ProjectArgs &a, int i, int view, bool staged, bool bulk,
                                            const float *rest, uint64_t *bar) {
    const ViewGeom vg = view_geom(a.vt, view);
    const size_t u = kViews ? (size_t)view * a.vt.n + i : (size_t)i;   // this view's record of Gaussian i
    const StepParams &sp = a.sp[view];
    const float Wf = (float)vg.width, Hf = (float)vg.height;
    // the rasterizer gradient record of every Gaussian starts the step at zero
    if (a.grad) {
        a.grad[u].a = make_float4(0.f, 0.f, 0.f, 0.f);
        a.grad[u].b = make_float4(0.f, 0.f, 0.f, 0.f);
        a.grad[u].c = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    a.radii[u] = 0;
    a.tiles_hit[u] = 0;

    const float px = a.means[3 * i], py = a.means[3 * i + 1], pz = a.means[3 * i + 2];
    // the Gaussian's other inputs, read with its centre (before the
    // near-plane test) so that all the loads are in flight together
    if (!MS_GUARD(((uintptr_t)a.quats & 15) == 0, 1, i, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) return;
    const float4 q = *reinterpret_cast<const float4 *>(a.quats + 4 * (size_t)i);
    const float sc0 = a.scales[3 * i], sc1 = a.scales[3 * i + 1], sc2 = a.scales[3 * i + 2];
    const float opl = a.opacities[i];
    const float dcv[3] = {a.features_dc[3 * (size_t)i], a.features_dc[3 * (size_t)i + 1],
                          a.features_dc[3 * (size_t)i + 2]};
    const float *v = sp.viewmat;
    // transform_4x3 + clip_near_plane
    const float vx = v[0] * px + v[1] * py + v[2] * pz + v[3];
    const float vy = v[4] * px + v[5] * py + v[6] * pz + v[7];
    const float vz = v[8] * px + v[9] * py + v[10] * pz + v[11];
    if (vz <= sp.clip_thresh) return;

    // exp_scale_clamped + quat_to_rotmat + scale_rot_to_cov3d (in registers)
    float s[3];
    s[0] = det_expf(fminf(fmaxf(sc0, -15.f), 15.f));
    s[1] = det_expf(fminf(fmaxf(sc1, -15.f), 15.f));
    s[2] = det_expf(fminf(fmaxf(sc2, -15.f), 15.f));
    const float qn = 1.0f / sqrtf(fmaxf(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z, 1e-8f));
    const float w = q.x * qn, x = q.y * qn, y = q.z * qn, z = q.w * qn;
    float R[3][3];
    R[0][0] = 1.f - 2.f * (y * y + z * z);
    R[1][0] = 2.f * (x * y + w * z);
    R[2][0] = 2.f * (x * z - w * y);
    R[0][1] = 2.f * (x * y - w * z);
    R[1][1] = 1.f - 2.f * (x * x + z * z);
    R[2][1] = 2.f * (y * z + w * x);
    R[0][2] = 2.f * (x * z + w * y);
    R[1][2] = 2.f * (y * z - w * x);
    R[2][2] = 1.f - 2.f * (x * x + y * y);
    float M[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) M[r][c] = R[r][c] * s[c];
    const float c00 = M[0][0] * M[0][0] + M[0][1] * M[0][1] + M[0][2] * M[0][2];
    const float c01 = M[0][0] * M[1][0] + M[0][1] * M[1][1] + M[0][2] * M[1][2];
    const float c02 = M[0][0] * M[2][0] + M[0][1] * M[2][1] + M[0][2] * M[2][2];
    const float c11 = M[1][0] * M[1][0] + M[1][1] * M[1][1] + M[1][2] * M[1][2];
    const float c12 = M[1][0] * M[2][0] + M[1][1] * M[2][1] + M[1][2] * M[2][2];
    const float c22 = M[2][0] * M[2][0] + M[2][1] * M[2][1] + M[2][2] * M[2][2];

    // project_cov3d_ewa
    const float lim_x = 1.3f * sp.tan_fovx, lim_y = 1.3f * sp.tan_fovy;
    const float cvx = vz * fminf(lim_x, fmaxf(-lim_x, vx / vz));
    const float cvy = vz * fminf(lim_y, fmaxf(-lim_y, vy / vz));
    const float rz = 1.f / vz, rz2 = rz * rz;
    const float j00 = sp.fx * rz, j11 = sp.fy * rz;
    const float j20 = -sp.fx * cvx * rz2, j21 = -sp.fy * cvy * rz2;
    const float t0x = j00 * v[0] + j20 * v[8], t0y = j00 * v[1] + j20 * v[9], t0z = j00 * v[2] + j20 * v[10];
    const float t1x = j11 * v[4] + j21 * v[8], t1y = j11 * v[5] + j21 * v[9], t1z = j11 * v[6] + j21 * v[10];
    const float tv0x = t0x * c00 + t0y * c01 + t0z * c02;
    const float tv0y = t0x * c01 + t0y * c11 + t0z * c12;
    const float tv0z = t0x * c02 + t0y * c12 + t0z * c22;
    const float tv1x = t1x * c00 + t1y * c01 + t1z * c02;
    const float tv1y = t1x * c01 + t1y * c11 + t1z * c12;
    const float tv1z = t1x * c02 + t1y * c12 + t1z * c22;
    const float a2 = (tv0x * t0x + tv0y * t0y + tv0z * t0z) + 0.3f;
    const float b2 = tv0x * t1x + tv0y * t1y + tv0z * t1z;
    const float d2 = (tv1x * t1x + tv1y * t1y + tv1z * t1z) + 0.3f;

    // compute_cov2d_bounds
    const float det = a2 * d2 - b2 * b2;
    if (!(det > 1e-6f)) return;
    const float inv_det = 1.f / det;
    const float ca = d2 * inv_det, cb = -b2 * inv_det, cc = a2 * inv_det;
    const float bm = 0.5f * (a2 + d2);
    const float disc = sqrtf(fmaxf(0.1f, bm * bm - det));
    const float radius = ceilf(3.f * sqrtf(bm + disc));

    // project_pix + ndc2pix
    const float *m = sp.projmat;
    const float hx = m[0] * px + m[1] * py + m[2] * pz + m[3];
    const float hy = m[4] * px + m[5] * py + m[6] * pz + m[7];
    const float hw = m[12] * px + m[13] * py + m[14] * pz + m[15];
    const float rw = 1.f / (hw + 1e-6f);
    const float ndx = hx * rw, ndy = hy * rw;
    const float cxp = 0.5f * Wf * ndx + sp.cx - 0.5f;
    const float cyp = 0.5f * Hf * ndy + sp.cy - 0.5f;
    const float ax = ceilf(3.f * sqrtf(a2)), ay = ceilf(3.f * sqrtf(d2));
    int x0, y0, x1, y1;
    tile_rect(cxp, cyp, ax, ay, vg.tiles_x, vg.tiles_y, x0, y0, x1, y1);
    const int area = (x1 - x0) * (y1 - y0);
    if (area <= 0) return;

    // SH colour (degrees_to_use bands) from the normalised view direction
    const float dx = px - sp.cam_pos[0], dy = py - sp.cam_pos[1], dz = pz - sp.cam_pos[2];
    const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
    const float vdx = dx * inv, vdy = dy * inv, vdz = dz * inv;
    const int deg = sp.degrees_to_use;
    const float *dc = dcv;
    float col[3];
    bool from_stage = staged;
    if (bulk && !tc::mbar_wait(bar, 0)) {   // the row did not arrive: read it from global memory
        record_fault(a.nan_counts ? a.nan_counts + kDbgSlot : nullptr, 40, i);
        from_stage = false;
    }
    if (from_stage) sh_colour(dc, rest, deg, vdx, vdy, vdz, col);
    else sh_colour(dc, a.features_rest + (size_t)a.rest_bases * 3 * i, deg, vdx, vdy, vdz, col);
    // sigmoid(opacity) once per Gaussian (the reference does it per
    // intersection at pack time; same input, same bits)
    const float opac = 1.f / (1.f + det_expf(-opl));

    // A non-finite opacity does not cull (the reference zeroes such a record
    // when it packs each intersection, hybrid_sort_pack_kernel): store 0,
    // which rasterizes the same way, and count the intersections.
    const bool oko = finite_bits(opac);
    const float op_rec = oko ? opac : 0.f;
    const float2 reach = reach_extent(cxp, cyp, op_rec, ca, cb, cc);
    SplatRec rec;
    rec.a = make_float4(cxp, cyp, op_rec, 0.f);
    rec.b = make_float4(ca, cb, cc, reach.x);
    rec.c = make_float4(col[0], col[1], col[2], reach.y);
    a.rec[u] = rec;
    a.depths[u] = vz;
    a.aabb[u] = make_float2(ax, ay);
    if (a.rect) a.rect[u] = make_ushort4((unsigned short)x0, (unsigned short)y0, (unsigned short)x1, (unsigned short)y1);

    // zombie gate: a non-finite projection output culls the Gaussian this step
    const bool okc = finite_bits(cxp) && finite_bits(cyp), okd = finite_bits(vz);
    const bool oka = finite_bits(ax) && finite_bits(ay);
    const bool okn = finite_bits(ca) && finite_bits(cb) && finite_bits(cc);
    const bool okr = finite_bits(col[0]) && finite_bits(col[1]) && finite_bits(col[2]);
    if (okc && okd && oka && okn && okr) {
        a.tiles_hit[u] = area;
        a.radii[u] = __float2int_rz(radius);
        if (!oko && a.nan_counts && area > 0) {
            atomicAdd(a.nan_counts + kNanPack, (unsigned)area);
            atomicAdd(a.nan_counts + kNanPackOpacity, (unsigned)area);
        }
    } else if (a.nan_counts) {
        atomicAdd(a.nan_counts + kNanProj, 1u);
        if (!okc) atomicAdd(a.nan_counts + kNanProjCenter, 1u);
        if (!okd) atomicAdd(a.nan_counts + kNanProjDepth, 1u);
        if (!oka) atomicAdd(a.nan_counts + kNanProjAabb, 1u);
        if (!okn) atomicAdd(a.nan_counts + kNanProjConic, 1u);
        if (!okr) atomicAdd(a.nan_counts + kNanProjRgb, 1u);
    }
}

// kViews: several views (blockIdx.y); false compiles the one-view step with
// the geometry read straight from the parameter bank.  At degree 3 with 15
// bases each warp stages its 32 Gaussians' SH rows (32 x 180 contiguous
// bytes) in shared memory: one bulk (TMA) copy issued by lane 0 when the rows
// are 16-byte aligned and whole 16-byte units, which lands while the warp
// computes the geometry; otherwise coalesced loads.  A lane's row there (45
// floats apart) is conflict-free.  Lane 0 waits for its copy before the warp
// leaves, so no copy outlives the CTA.
template <bool kViews>
__global__ void __launch_bounds__(256) k_project_fwd(ProjectArgs a) {
    pdl_enter();
    __shared__ __align__(16) float stage[8][32 * kStageFloats];
    __shared__ __align__(8) uint64_t bar[8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int view = kViews ? (int)blockIdx.y : 0;
    const bool staged = a.rest_bases == 15 && a.sp[view].degrees_to_use >= 3;   // uniform over the CTA
    bool bulk = false;
    if (staged) {
        const int i0 = i - lane;
        const int cnt = min(32, a.vt.n - i0);
        if (cnt > 0) {
            const float *src = a.features_rest + (size_t)i0 * kStageFloats;
            float *dst = stage[wid];
            const int nf = cnt * kStageFloats;
            bulk = (reinterpret_cast<uintptr_t>(src) & 15) == 0 && (nf & 3) == 0;   // uniform over the warp
            if (bulk) {
                if (lane == 0) {
                    tc::mbar_init(&bar[wid], 1);
                    tc::mbar_arrive_expect_tx(&bar[wid], (uint32_t)nf * 4u);
                    tc::bulk_g2s(dst, src, (uint32_t)nf * 4u, &bar[wid]);
                }
            } else {
                int done = 0;
                if ((reinterpret_cast<uintptr_t>(src) & 15) == 0) {
                    const int nv = nf >> 2;
                    const float4 *s4 = reinterpret_cast<const float4 *>(src);
                    float4 *d4 = reinterpret_cast<float4 *>(dst);
                    for (int k = lane; k < nv; k += 32) d4[k] = s4[k];
                    done = nv << 2;
                }
                for (int k = done + lane; k < nf; k += 32) dst[k] = src[k];
            }
        }
        __syncwarp();
    }
    if (i < a.vt.n) project_one<kViews>(a, i, view, staged, bulk, &stage[wid][lane * kStageFloats], &bar[wid]);
    if (bulk && lane == 0 && !tc::mbar_wait(&bar[wid], 0))
        record_fault(a.nan_counts ? a.nan_counts + kDbgSlot : nullptr, 41, i);
}

void launch_project_fwd(const ProjectArgs &a, cudaStream_t s) {
    if (a.vt.n <= 0) return;
    if (a.vt.count > 1) launch_pdl(k_project_fwd<true>, dim3((a.vt.n + 255) / 256, a.vt.count), 256, 0, s, a);
    else launch_pdl(k_project_fwd<false>, (a.vt.n + 255) / 256, 256, 0, s, a);
}

}  // namespace msplat
