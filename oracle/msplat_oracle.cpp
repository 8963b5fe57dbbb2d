// msplat CPU oracle — TEST INFRASTRUCTURE ONLY (see msplat_oracle.h).
//
// Scalar restatement of one msplat training step.  Every stage cites the
// reference lines it follows (paths relative to the semhfe/msplat tree).
// Compile with -ffp-contract=off: the float path must not be fused except
// where the reference writes fma().
#include "msplat_oracle.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Arithmetic primitives
// ---------------------------------------------------------------------------

// exp(x) for float: Cody-Waite reduction x = n*ln2 + r (ln2 split hi/lo so
// that n*ln2_hi is exact for |n| <= 256), then the degree-7 Taylor
// polynomial of e^r on |r| <= ln2/2 (truncation < 5e-9 relative) by Horner
// with fused multiply-adds, then an exact power-of-two scale.  Every
// operation is IEEE-rounded, so any conforming host or device gives the same
// bits.  Accuracy: within 2 ulp of the exact value (tests/test_oracle.py).
float det_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return std::numeric_limits<float>::infinity();
    if (x < -87.33654f) return 0.0f;
    const float n = std::rint(x * 1.44269504088896341f);
    float r = std::fma(n, -0.693145751953125f, x);
    r = std::fma(n, -1.42860676533018e-06f, r);
    float p = 1.0f / 5040.0f;
    p = std::fma(p, r, 1.0f / 720.0f);
    p = std::fma(p, r, 1.0f / 120.0f);
    p = std::fma(p, r, 1.0f / 24.0f);
    p = std::fma(p, r, 1.0f / 6.0f);
    p = std::fma(p, r, 0.5f);
    p = std::fma(p, r, 1.0f);
    p = std::fma(p, r, 1.0f);
    int ni = (int)n;
    float scale_lo = 1.0f;
    if (ni > 127) { scale_lo = 2.0f; ni -= 1; }
    if (ni < -126) { scale_lo = 0.5f; ni += 1; }
    uint32_t bits = (uint32_t)(ni + 127) << 23;
    float two_n;
    std::memcpy(&two_n, &bits, 4);
    return (p * two_n) * scale_lo;
}

template <class R> inline R EXP(R x);
template <> inline float EXP<float>(float x) { return det_expf(x); }
template <> inline double EXP<double>(double x) { return std::exp(x); }
template <class R> inline R FMA(R a, R b, R c) { return std::fma(a, b, c); }
template <class R> inline R SQRT(R x) { return std::sqrt(x); }
template <class R> inline R FMIN(R a, R b) { return std::fmin(a, b); }
template <class R> inline R FMAX(R a, R b) { return std::fmax(a, b); }

// core/metal/msplat_metal.metal:115-117: exponent-field test.
inline bool finite_bits(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return (b & 0x7F800000u) != 0x7F800000u;
}
inline bool finite_bits(double x) { return std::isfinite(x); }

// float -> int with truncation, saturating, NaN -> 0 (the conversion the
// GPU performs; C leaves out-of-range conversion undefined).
template <class R> inline int sat_f2i(R x) {
    if (x != x) return 0;
    if (x >= (R)2147483647.0) return INT_MAX;
    if (x <= (R)-2147483648.0) return INT_MIN;
    return (int)x;
}

// Spherical-harmonic constants (real SH normalisation, degrees 0-3).
const double SH_C0 = 0.28209479177387814;
const double SH_C1 = 0.4886025119029199;
const double SH_C2[5] = {1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                         -1.0925484305920792, 0.5462742152960396};
const double SH_C3[7] = {-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                         0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                         -0.5900435899266435};

template <class R> inline R CK(double v) { return (R)v; }
template <> inline float CK<float>(double v) { return (float)v; }

// 11-tap Gaussian window, sigma 1.5, normalised in double then rounded
// (equals the reference's GAUSS_1D table, .metal:3376-3380).
template <class R> void gauss_1d(R w[11]) {
    double g[11], s = 0;
    for (int i = 0; i < 11; i++) { g[i] = std::exp(-((i - 5) * (i - 5)) / (2.0 * 1.5 * 1.5)); s += g[i]; }
    for (int i = 0; i < 11; i++) w[i] = (R)(float)(g[i] / s);
}

// ---------------------------------------------------------------------------
// Per-Gaussian geometry (.metal:53-344)
// ---------------------------------------------------------------------------

template <class R> struct Mat3 { R m[3][3]; };  // m[row][col]

// .metal:134-156 (rsqrt restated as 1/sqrt; quats stored w,x,y,z)
template <class R> Mat3<R> quat_to_rotmat(const R q[4], R &w, R &x, R &y, R &z) {
    R s = R(1) / SQRT(FMAX(q[3] * q[3] + q[0] * q[0] + q[1] * q[1] + q[2] * q[2], CK<R>(1e-8f)));
    w = q[0] * s; x = q[1] * s; y = q[2] * s; z = q[3] * s;
    Mat3<R> M;
    M.m[0][0] = R(1) - R(2) * (y * y + z * z);
    M.m[1][0] = R(2) * (x * y + w * z);
    M.m[2][0] = R(2) * (x * z - w * y);
    M.m[0][1] = R(2) * (x * y - w * z);
    M.m[1][1] = R(1) - R(2) * (x * x + z * z);
    M.m[2][1] = R(2) * (y * z + w * x);
    M.m[0][2] = R(2) * (x * z + w * y);
    M.m[1][2] = R(2) * (y * z - w * x);
    M.m[2][2] = R(1) - R(2) * (x * x + y * y);
    return M;
}

// .metal:200-213: cov = (R S)(R S)^T, upper triangle
template <class R> void scale_rot_to_cov3d(const R s[3], const R q[4], R cov[6]) {
    R w, x, y, z;
    Mat3<R> Rm = quat_to_rotmat(q, w, x, y, z);
    R M[3][3];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) M[r][c] = Rm.m[r][c] * s[c];
    auto cv = [&](int r, int j) { return M[r][0] * M[j][0] + M[r][1] * M[j][1] + M[r][2] * M[j][2]; };
    cov[0] = cv(0, 0); cov[1] = cv(0, 1); cov[2] = cv(0, 2);
    cov[3] = cv(1, 1); cov[4] = cv(1, 2); cov[5] = cv(2, 2);
}

template <class R> struct Cam {
    R vm[16], pm[16], fx, fy, cx, cy, W, H, tan_fovx, tan_fovy, campos[3], bg[3], clip;
    int width, height, tiles_x, tiles_y;
};

// .metal:266-306
template <class R> void project_cov3d_ewa(const R cov[6], const Cam<R> &c, const R pv_in[3], R out[3]) {
    R lim_x = CK<R>(1.3f) * c.tan_fovx, lim_y = CK<R>(1.3f) * c.tan_fovy;
    R pz = pv_in[2];
    R px = pz * FMIN(lim_x, FMAX(-lim_x, pv_in[0] / pz));
    R py = pz * FMIN(lim_y, FMAX(-lim_y, pv_in[1] / pz));
    R rz = R(1) / pz, rz2 = rz * rz;
    R j00 = c.fx * rz, j11 = c.fy * rz;
    R j20 = -c.fx * px * rz2, j21 = -c.fy * py * rz2;
    const R *v = c.vm;
    R t0[3] = {j00 * v[0] + j20 * v[8], j00 * v[1] + j20 * v[9], j00 * v[2] + j20 * v[10]};
    R t1[3] = {j11 * v[4] + j21 * v[8], j11 * v[5] + j21 * v[9], j11 * v[6] + j21 * v[10]};
    R v00 = cov[0], v01 = cov[1], v02 = cov[2], v11 = cov[3], v12 = cov[4], v22 = cov[5];
    R tv0[3] = {t0[0] * v00 + t0[1] * v01 + t0[2] * v02, t0[0] * v01 + t0[1] * v11 + t0[2] * v12,
                t0[0] * v02 + t0[1] * v12 + t0[2] * v22};
    R tv1[3] = {t1[0] * v00 + t1[1] * v01 + t1[2] * v02, t1[0] * v01 + t1[1] * v11 + t1[2] * v12,
                t1[0] * v02 + t1[1] * v12 + t1[2] * v22};
    out[0] = (tv0[0] * t0[0] + tv0[1] * t0[1] + tv0[2] * t0[2]) + CK<R>(0.3f);
    out[1] = tv0[0] * t1[0] + tv0[1] * t1[1] + tv0[2] * t1[2];
    out[2] = (tv1[0] * t1[0] + tv1[1] * t1[1] + tv1[2] * t1[2]) + CK<R>(0.3f);
}

// .metal:57-87: tile rectangle of a splat (inclusive min, exclusive max)
template <class R> void tile_bbox(R cx_, R cy_, R ax, R ay, int tx, int ty, int &x0, int &y0, int &x1, int &y1) {
    R tcx = cx_ / R(16), tcy = cy_ / R(16), trx = ax / R(16), try_ = ay / R(16);
    x0 = std::min(std::max(0, sat_f2i(tcx - trx)), tx);
    x1 = std::min(std::max(0, sat_f2i(tcx + trx + R(1))), tx);
    y0 = std::min(std::max(0, sat_f2i(tcy - try_)), ty);
    y1 = std::min(std::max(0, sat_f2i(tcy + try_ + R(1))), ty);
}

// .metal:620-687 (degrees 0..3)
template <class R> void sh_to_color(int deg, const R d[3], const float *dc, const float *rest, R col[3]) {
    R x = d[0], y = d[1], z = d[2];
    R xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    for (int c = 0; c < 3; c++) {
        auto r = [&](int b) { return (R)rest[b * 3 + c]; };
        R v = CK<R>(SH_C0) * (R)dc[c];
        if (deg >= 1) {
            v += CK<R>(SH_C1) * (-y * r(0) + z * r(1) - x * r(2));
            if (deg >= 2) {
                v += (CK<R>(SH_C2[0]) * xy * r(3) + CK<R>(SH_C2[1]) * yz * r(4) +
                      CK<R>(SH_C2[2]) * (R(2) * zz - xx - yy) * r(5) + CK<R>(SH_C2[3]) * xz * r(6) +
                      CK<R>(SH_C2[4]) * (xx - yy) * r(7));
                if (deg >= 3) {
                    v += (CK<R>(SH_C3[0]) * y * (R(3) * xx - yy) * r(8) + CK<R>(SH_C3[1]) * xy * z * r(9) +
                          CK<R>(SH_C3[2]) * y * (R(4) * zz - xx - yy) * r(10) +
                          CK<R>(SH_C3[3]) * z * (R(2) * zz - R(3) * xx - R(3) * yy) * r(11) +
                          CK<R>(SH_C3[4]) * x * (R(4) * zz - xx - yy) * r(12) +
                          CK<R>(SH_C3[5]) * z * (xx - yy) * r(13) + CK<R>(SH_C3[6]) * x * (xx - R(3) * yy) * r(14));
                }
            }
        }
        col[c] = v;
    }
}

// SH basis values of bands 1..3 (the multipliers .metal:1993-2033 apply to v_colors)
template <class R> void sh_basis(const R d[3], R b[15]) {
    R x = d[0], y = d[1], z = d[2];
    R xx = x * x, xy = x * y, xz = x * z, yy = y * y, yz = y * z, zz = z * z;
    b[0] = -CK<R>(SH_C1) * y; b[1] = CK<R>(SH_C1) * z; b[2] = -CK<R>(SH_C1) * x;
    b[3] = CK<R>(SH_C2[0]) * xy; b[4] = CK<R>(SH_C2[1]) * yz; b[5] = CK<R>(SH_C2[2]) * (R(2) * zz - xx - yy);
    b[6] = CK<R>(SH_C2[3]) * xz; b[7] = CK<R>(SH_C2[4]) * (xx - yy);
    b[8] = CK<R>(SH_C3[0]) * y * (R(3) * xx - yy); b[9] = CK<R>(SH_C3[1]) * xy * z;
    b[10] = CK<R>(SH_C3[2]) * y * (R(4) * zz - xx - yy); b[11] = CK<R>(SH_C3[3]) * z * (R(2) * zz - R(3) * xx - R(3) * yy);
    b[12] = CK<R>(SH_C3[4]) * x * (R(4) * zz - xx - yy); b[13] = CK<R>(SH_C3[5]) * z * (xx - yy);
    b[14] = CK<R>(SH_C3[6]) * x * (xx - R(3) * yy);
}

template <class R> void viewdir(const float p[3], const Cam<R> &c, R d[3]) {
    R dx = (R)p[0] - c.campos[0], dy = (R)p[1] - c.campos[1], dz = (R)p[2] - c.campos[2];
    R inv = R(1) / SQRT(dx * dx + dy * dy + dz * dz);
    d[0] = dx * inv; d[1] = dy * inv; d[2] = dz * inv;
}

// ---------------------------------------------------------------------------
// State of one step
// ---------------------------------------------------------------------------

template <class R> struct Step {
    const OrStepIn &in;
    Cam<R> cam;
    int N, T, P;
    std::vector<R> xys, depths, conics, colors, aabb;
    std::vector<int> radii, tiles_hit;
    std::vector<int> tile_counts, tile_start;
    std::vector<int> ids;       // sorted tile lists, concatenated
    std::vector<R> pk;          // packed per isect: x y opac ca cb cc r g b
    std::vector<R> img, finalT;
    std::vector<int> final_idx;
    int K = 1;
    std::vector<R> chT, chC, preT, aftC;
    std::vector<int> chIdx;
    double loss_sum = 0;
    std::vector<R> v_rend;
    std::vector<R> v_xy, v_conic, v_col, v_op;
    std::vector<R> v_mean, v_scale, v_quat;
    uint32_t nan[16] = {0};
    long long pairs_fwd = 0, pairs_bwd = 0;

    explicit Step(const OrStepIn &i) : in(i) {}

    // the tile-row band of a restricted step (all rows when none is set)
    bool row_in_band(int ty) const {
        return in.tile_row_hi <= in.tile_row_lo || (ty >= in.tile_row_lo && ty < in.tile_row_hi);
    }

    void setup() {
        N = in.num_points;
        cam.width = in.width; cam.height = in.height;
        cam.tiles_x = (in.width + 15) / 16; cam.tiles_y = (in.height + 15) / 16;
        T = cam.tiles_x * cam.tiles_y;
        P = in.width * in.height;
        for (int k = 0; k < 16; k++) { cam.vm[k] = (R)in.viewmat[k]; cam.pm[k] = (R)in.projmat[k]; }
        cam.fx = in.fx; cam.fy = in.fy; cam.cx = in.cx; cam.cy = in.cy;
        cam.W = (R)(float)in.width; cam.H = (R)(float)in.height;
        cam.tan_fovx = CK<R>(0.5f) * cam.W / cam.fx;   // .metal:1771
        cam.tan_fovy = CK<R>(0.5f) * cam.H / cam.fy;
        for (int k = 0; k < 3; k++) { cam.campos[k] = (R)in.cam_pos[k]; cam.bg[k] = (R)in.background[k]; }
        cam.clip = (R)in.clip_thresh;
    }

    // project_and_sh_forward_kernel, .metal:1719-1834
    void project() {
        xys.assign(2 * (size_t)N, 0); depths.assign(N, 0); conics.assign(3 * (size_t)N, 0);
        colors.assign(3 * (size_t)N, 0); aabb.assign(2 * (size_t)N, 0);
        radii.assign(N, 0); tiles_hit.assign(N, 0);
        const int rb = in.rest_bases;
        uint32_t cnt[6] = {0};
#pragma omp parallel for schedule(static) reduction(+ : cnt[:6])
        for (int i = 0; i < N; i++) {
            const float *mp = in.means + 3 * (size_t)i;
            R p[3] = {(R)mp[0], (R)mp[1], (R)mp[2]};
            const R *v = cam.vm;
            R pv[3] = {v[0] * p[0] + v[1] * p[1] + v[2] * p[2] + v[3], v[4] * p[0] + v[5] * p[1] + v[6] * p[2] + v[7],
                       v[8] * p[0] + v[9] * p[1] + v[10] * p[2] + v[11]};
            if (pv[2] <= cam.clip) continue;
            R s[3], q[4], cov[6], c2[3];
            for (int k = 0; k < 3; k++)
                s[k] = EXP<R>(FMIN(FMAX((R)in.scales[3 * (size_t)i + k], CK<R>(-15.f)), CK<R>(15.f)));
            for (int k = 0; k < 4; k++) q[k] = (R)in.quats[4 * (size_t)i + k];
            scale_rot_to_cov3d(s, q, cov);
            project_cov3d_ewa(cov, cam, pv, c2);
            R det = c2[0] * c2[2] - c2[1] * c2[1];
            if (!(det > CK<R>(1e-6f))) continue;
            R inv_det = R(1) / det;
            R con[3] = {c2[2] * inv_det, -c2[1] * inv_det, c2[0] * inv_det};
            R b = CK<R>(0.5f) * (c2[0] + c2[2]);
            R disc = SQRT(FMAX(CK<R>(0.1f), b * b - det));
            R radius = std::ceil(R(3) * SQRT(b + disc));
            const R *m = cam.pm;
            R ph[4] = {m[0] * p[0] + m[1] * p[1] + m[2] * p[2] + m[3], m[4] * p[0] + m[5] * p[1] + m[6] * p[2] + m[7],
                       m[8] * p[0] + m[9] * p[1] + m[10] * p[2] + m[11],
                       m[12] * p[0] + m[13] * p[1] + m[14] * p[2] + m[15]};
            R rw = R(1) / (ph[3] + CK<R>(1e-6f));
            R ndx = ph[0] * rw, ndy = ph[1] * rw;
            R cxp = CK<R>(0.5f) * cam.W * ndx + cam.cx - CK<R>(0.5f);   // ndc2pix, .metal:53-55
            R cyp = CK<R>(0.5f) * cam.H * ndy + cam.cy - CK<R>(0.5f);
            R ax = std::ceil(R(3) * SQRT(c2[0])), ay = std::ceil(R(3) * SQRT(c2[2]));
            int x0, y0, x1, y1;
            tile_bbox(cxp, cyp, ax, ay, cam.tiles_x, cam.tiles_y, x0, y0, x1, y1);
            int area = (x1 - x0) * (y1 - y0);
            if (area <= 0) continue;
            tiles_hit[i] = area;
            depths[i] = pv[2];
            radii[i] = sat_f2i(radius);
            xys[2 * i] = cxp; xys[2 * i + 1] = cyp;
            aabb[2 * i] = ax; aabb[2 * i + 1] = ay;
            R d[3], col[3];
            viewdir(mp, cam, d);
            sh_to_color(in.degrees_to_use, d, in.features_dc + 3 * (size_t)i, in.features_rest + (size_t)rb * 3 * i, col);
            for (int k = 0; k < 3; k++) colors[3 * i + k] = col[k];
            for (int k = 0; k < 3; k++) conics[3 * i + k] = con[k];
            bool okc = finite_bits(cxp) && finite_bits(cyp), okd = finite_bits(pv[2]);
            bool oka = finite_bits(ax) && finite_bits(ay);
            bool okn = finite_bits(con[0]) && finite_bits(con[1]) && finite_bits(con[2]);
            bool okr = finite_bits(col[0]) && finite_bits(col[1]) && finite_bits(col[2]);
            if (!(okc && okd && oka && okn && okr)) {
                radii[i] = 0; tiles_hit[i] = 0;
                cnt[0]++; if (!okc) cnt[1]++; if (!okd) cnt[2]++; if (!oka) cnt[3]++;
                if (!okn) cnt[4]++;
                if (!okr) cnt[5]++;
            }
        }
        for (int k = 0; k < 6; k++) nan[7 + k] += cnt[k];
    }

    // count / prefix / scatter / sort+pack, .metal:2267-2627
    void build_tiles(long long capacity) {
        tile_counts.assign(T, 0);
        std::vector<std::vector<std::pair<R, int>>> lists(T);
        for (int i = 0; i < N; i++) {
            if (radii[i] <= 0) continue;
            R d = depths[i];
            if (!finite_bits(d) || d <= R(0)) continue;
            int x0, y0, x1, y1;
            tile_bbox(xys[2 * i], xys[2 * i + 1], aabb[2 * i], aabb[2 * i + 1], cam.tiles_x, cam.tiles_y, x0, y0, x1, y1);
            for (int y = y0; y < y1; y++) {
                if (!row_in_band(y)) continue;
                for (int x = x0; x < x1; x++) lists[(size_t)y * cam.tiles_x + x].push_back({d, i});
            }
        }
        tile_start.assign(T + 1, 0);
        for (int t = 0; t < T; t++) {
            tile_counts[t] = (int)lists[t].size();
            tile_start[t + 1] = tile_start[t] + tile_counts[t];
        }
        long long M = tile_start[T];
        ids.assign(M, 0);
        pk.assign(M * 9, 0);
        uint32_t gate = 0, gate_op = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : gate, gate_op)
        for (int t = 0; t < T; t++) {
            auto &L = lists[t];
            std::sort(L.begin(), L.end());   // ascending depth, ties by id (key = depth_bits<<32 | id)
            const long long s = tile_start[t];
            const bool fits = (long long)tile_start[t + 1] <= capacity;
            for (size_t j = 0; j < L.size(); j++) {
                const long long d = s + (long long)j;
                R *o = &pk[d * 9];
                if (!fits) { ids[d] = 0; for (int k = 0; k < 9; k++) o[k] = 0; continue; }
                int g = L[j].second;
                ids[d] = g;
                R op = R(1) / (R(1) + EXP<R>(-(R)in.opacities[g]));
                R x = xys[2 * g], y = xys[2 * g + 1];
                bool ok = finite_bits(x) && finite_bits(y) && finite_bits(op);
                for (int k = 0; k < 3; k++) ok = ok && finite_bits(conics[3 * g + k]) && finite_bits(colors[3 * g + k]);
                if (!ok) { gate++; if (!finite_bits(op)) gate_op++; for (int k = 0; k < 9; k++) o[k] = 0; continue; }
                o[0] = x; o[1] = y; o[2] = op;
                o[3] = conics[3 * g]; o[4] = conics[3 * g + 1]; o[5] = conics[3 * g + 2];
                o[6] = colors[3 * g]; o[7] = colors[3 * g + 1]; o[8] = colors[3 * g + 2];
            }
        }
        nan[13] += gate; nan[14] += gate_op;
    }

    // One pixel's front-to-back walk over [s, e) (.metal:545-606 / 3024-3066).
    // Returns T and accumulated colour; last = index of the last contributor.
    void composite(long long s, long long e, R px, R py, R &Tv, R C[3], long long &last, long long &pairs, uint32_t &nsig) {
        Tv = R(1); C[0] = C[1] = C[2] = R(0); last = s - 1;
        for (long long idx = s; idx < e; idx++) {
            const R *o = &pk[idx * 9];
            pairs++;
            R dx = o[0] - px, dy = o[1] - py;
            R sigma = FMA(CK<R>(0.5f), FMA(o[3], dx * dx, o[5] * dy * dy), o[4] * dx * dy);
            if (!finite_bits(sigma)) { nsig++; continue; }
            if (sigma < R(0) || (sigma >= CK<R>(5.55f) && !in.no_cutoff)) continue;
            R alpha = FMIN(CK<R>(0.999f), o[2] * EXP<R>(-sigma));
            if (alpha < CK<R>(1.f / 255.f) && !in.no_cutoff) continue;
            R nT = Tv * (R(1) - alpha);
            if (nT <= CK<R>(1e-4f)) { last = idx - 1; return; }
            R vis = alpha * Tv;
            for (int c = 0; c < 3; c++) C[c] = FMA(FMAX(o[6 + c] + CK<R>(0.5f), R(0)), vis, C[c]);
            Tv = nT;
            last = idx;
        }
    }

    static R sat(R x) { return FMIN(FMAX(x, R(0)), R(1)); }

    void raster_forward() {
        img.assign(3 * (size_t)P, 0); finalT.assign(P, 1); final_idx.assign(P, 0);
        const int W = in.width, H = in.height;
        long long pairs = 0;
        uint32_t nsig = 0;
        if (K <= 1) {
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : pairs, nsig)
            for (int t = 0; t < T; t++) {
                int tx = t % cam.tiles_x, ty = t / cam.tiles_x;
                if (!row_in_band(ty)) continue;
                for (int yy = 0; yy < 16; yy++)
                    for (int xx = 0; xx < 16; xx++) {
                        int x = tx * 16 + xx, y = ty * 16 + yy;
                        if (x >= W || y >= H) continue;
                        R Tv, C[3]; long long last;
                        uint32_t dummy = 0;
                        composite(tile_start[t], tile_start[t + 1], (R)x, (R)y, Tv, C, last, pairs, dummy);
                        size_t p = (size_t)y * W + x;
                        finalT[p] = Tv; final_idx[p] = (int)last;
                        for (int c = 0; c < 3; c++) img[3 * p + c] = sat(FMA(cam.bg[c], Tv, C[c]));
                    }
            }
        } else {
            chT.assign((size_t)K * P, 1); chC.assign((size_t)K * P * 3, 0); chIdx.assign((size_t)K * P, -1);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : pairs, nsig)
            for (int t = 0; t < T; t++) {
                int tx = t % cam.tiles_x, ty = t / cam.tiles_x;
                if (!row_in_band(ty)) continue;
                for (int k = 0; k < K; k++) {
                    long long cs = tile_start[t] + (long long)k * 512;
                    long long ce = std::min<long long>(tile_start[t] + (long long)(k + 1) * 512, tile_start[t + 1]);
                    for (int yy = 0; yy < 16; yy++)
                        for (int xx = 0; xx < 16; xx++) {
                            int x = tx * 16 + xx, y = ty * 16 + yy;
                            if (x >= W || y >= H) continue;
                            size_t o = (size_t)k * P + (size_t)y * W + x;
                            if (cs >= ce) { chT[o] = 1; chC[3 * o] = chC[3 * o + 1] = chC[3 * o + 2] = 0; chIdx[o] = -1; continue; }
                            R Tv, C[3]; long long last;
                            composite(cs, ce, (R)x, (R)y, Tv, C, last, pairs, nsig);
                            chT[o] = Tv; for (int c = 0; c < 3; c++) chC[3 * o + c] = C[c];
                            chIdx[o] = (int)last;
                        }
                }
            }
            // rasterize_forward_merge_kernel, .metal:3081-3134
#pragma omp parallel for schedule(static)
            for (int p = 0; p < P; p++) {
                R Tr = 1, Cr[3] = {0, 0, 0};
                int last = -1, cut = K;
                for (int k = 0; k < K; k++) {
                    size_t o = (size_t)k * P + p;
                    int cf = chIdx[o];
                    if (cf < 0 && k > 0) break;
                    for (int c = 0; c < 3; c++) Cr[c] = FMA(chC[3 * o + c], Tr, Cr[c]);
                    Tr *= chT[o];
                    if (cf >= 0) last = cf;
                    if (Tr <= CK<R>(1e-4f)) { cut = k + 1; break; }
                }
                for (int k = cut; k < K; k++) chIdx[(size_t)k * P + p] = -1;
                finalT[p] = Tr; final_idx[p] = last;
                for (int c = 0; c < 3; c++) img[3 * p + c] = sat(FMA(cam.bg[c], Tr, Cr[c]));
            }
        }
        pairs_fwd = pairs;
        nan[15] += nsig;
    }

    // ssim_h_fwd_kernel + ssim_fused_v_fwd_h_bwd_kernel + ssim_v_bwd_kernel (.metal:3388-3450, 3563-3681, 3764-3850)
    void loss() {
        const int W = in.width, H = in.height;
        R w[11];
        gauss_1d(w);
        const R inv255 = CK<R>(1.0f / 255.0f);
        const R C1 = CK<R>(0.0001f), C2 = CK<R>(0.0009f);
        const R sw = (R)in.ssim_weight, invn = (R)in.loss_inv_n;
        auto G = [&](int y, int x, int c) { return (R)in.gt[((size_t)y * W + x) * 3 + c] * inv255; };
        auto I = [&](int y, int x, int c) { return img[((size_t)y * W + x) * 3 + c]; };
        // pass 1: horizontal moments, zero padding
        std::vector<R> h((size_t)P * 15);
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                for (int c = 0; c < 3; c++) {
                    R mx = 0, my = 0, sx = 0, sy = 0, cr = 0;
                    for (int d = 0; d < 11; d++) {
                        int gx = x - 5 + d;
                        R gv = 0, rv = 0;
                        if (gx >= 0 && gx < W) { gv = G(y, gx, c); rv = I(y, gx, c); }
                        mx += w[d] * gv; my += w[d] * rv; sx += w[d] * gv * gv; sy += w[d] * rv * rv; cr += w[d] * gv * rv;
                    }
                    R *o = &h[((size_t)y * W + x) * 15 + c * 5];
                    o[0] = mx; o[1] = my; o[2] = sx; o[3] = sy; o[4] = cr;
                }
        // pass 2: derivative fields at every row and at columns -5..W+4 (the
        // reference also evaluates the out-of-image columns, from zero moments)
        const int FW = W + 10;
        std::vector<R> F((size_t)H * FW * 9);
        std::vector<R> pos_ssim((size_t)H * W, 0), pos_l1((size_t)H * W, 0);
        uint32_t nwin = 0;
#pragma omp parallel for schedule(static) reduction(+ : nwin)
        for (int y = 0; y < H; y++) {
            for (int fx = 0; fx < FW; fx++) {
                int gx = fx - 5;
                bool in_img = gx >= 0 && gx < W;
                R mval = 1;
                if (in.mask && in_img && in.mask[(size_t)y * W + gx] < 128) mval = 0;
                R ssim_c = 0, l1_c = 0;
                for (int c = 0; c < 3; c++) {
                    R m[5] = {0, 0, 0, 0, 0};
                    for (int k = 0; k < 11; k++) {
                        int gy = y - 5 + k;
                        if (gy < 0 || gy >= H || !in_img) continue;
                        const R *hp = &h[((size_t)gy * W + gx) * 15 + c * 5];
                        for (int f = 0; f < 5; f++) m[f] += w[k] * hp[f];
                    }
                    R *o = &F[(((size_t)y * FW + fx) * 3 + c) * 3];
                    bool fin = true;
                    for (int f = 0; f < 5; f++) fin = fin && finite_bits(m[f]);
                    if (!fin) { o[0] = o[1] = o[2] = 0; nwin++; continue; }
                    R mu_x = m[0], mu_y = m[1];
                    R sxq = FMAX(m[2] - mu_x * mu_x, R(0)), syq = FMAX(m[3] - mu_y * mu_y, R(0));
                    R sxy = m[4] - mu_x * mu_y;
                    R A = R(2) * mu_x * mu_y + C1, B = R(2) * sxy + C2;
                    R Cd = mu_x * mu_x + mu_y * mu_y + C1, D = sxq + syq + C2;
                    R iCD = R(1) / (Cd * D);
                    R dmu = R(2) * B * (mu_x * Cd - A * mu_y) / (Cd * Cd * D);
                    R dsyq = -A * B * iCD / D, dsxy = R(2) * A * iCD;
                    o[0] = mval * (dmu - R(2) * mu_y * dsyq - mu_x * dsxy);
                    o[1] = mval * (R(2) * dsyq);
                    o[2] = mval * dsxy;
                    if (in_img) {
                        ssim_c += mval * (A * B) / (Cd * D);
                        l1_c += mval * std::fabs(G(y, gx, c) - I(y, gx, c));
                    }
                }
                if (in_img) { pos_ssim[(size_t)y * W + gx] = ssim_c; pos_l1[(size_t)y * W + gx] = l1_c; }
            }
        }
        // The reference sums the loss per thread of a 16x16 tile: thread tr
        // evaluates window centres tr and tr+256 of the tile's 16 x 26 field
        // grid, and only a thread whose own pixel is in the image adds
        // w*(1 - s/3) + (1-w)*l/3 (.metal:3598-3671).
        double lsum = 0;
        const int tiles_x = (W + 15) / 16, tiles_y = (H + 15) / 16;
        for (int tyi = 0; tyi < tiles_y; tyi++)
            for (int txi = 0; txi < tiles_x; txi++)
                for (int tr = 0; tr < 256; tr++) {
                    int px = txi * 16 + (tr & 15), py = tyi * 16 + (tr >> 4);
                    if (px >= W || py >= H) continue;
                    R s = 0, l = 0;
                    for (int i = tr; i < 16 * 26; i += 256) {
                        int fy = i / 26, fxx = i % 26;
                        int gx = txi * 16 - 5 + fxx, gy = tyi * 16 + fy;
                        if (fxx < 5 || fxx >= 21 || gx < 0 || gx >= W || gy >= H) continue;
                        s += pos_ssim[(size_t)gy * W + gx];
                        l += pos_l1[(size_t)gy * W + gx];
                    }
                    lsum += (double)(sw * (R(1) - s / R(3)) + (R(1) - sw) * l / R(3));
                }
        loss_sum = lsum;
        nan[4] += nwin;
        // horizontal transpose convolution of the fields
        std::vector<R> dh((size_t)P * 9);
#pragma omp parallel for schedule(static)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++)
                for (int c = 0; c < 3; c++) {
                    R a[3] = {0, 0, 0};
                    for (int d = 0; d < 11; d++) {
                        const R *f = &F[(((size_t)y * FW + (x + d)) * 3 + c) * 3];
                        for (int k = 0; k < 3; k++) a[k] += w[10 - d] * f[k];
                    }
                    for (int k = 0; k < 3; k++) dh[((size_t)y * W + x) * 9 + c * 3 + k] = a[k];
                }
        // pass 3: vertical transpose convolution + combine
        v_rend.assign(3 * (size_t)P, 0);
        uint32_t nv = 0;
#pragma omp parallel for schedule(static) reduction(+ : nv)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                R mc = 1;
                if (in.mask && in.mask[(size_t)y * W + x] < 128) mc = 0;
                for (int c = 0; c < 3; c++) {
                    R a[3] = {0, 0, 0};
                    for (int d = 0; d < 11; d++) {
                        int gy = y - 5 + d;
                        if (gy < 0 || gy >= H) continue;
                        const R *f = &dh[((size_t)gy * W + x) * 9 + c * 3];
                        for (int k = 0; k < 3; k++) a[k] += w[10 - d] * f[k];
                    }
                    R r = I(y, x, c), g = G(y, x, c);
                    R vs = a[0] + r * a[1] + g * a[2];
                    R vl = mc * ((g > r) ? R(-1) : ((g < r) ? R(1) : R(0)));
                    R v = invn * (-sw * vs + (R(1) - sw) * vl);
                    if (!finite_bits(v)) { nv++; v = 0; }
                    v_rend[((size_t)y * W + x) * 3 + c] = v;
                }
            }
        nan[6] += nv;
    }

    // rasterize_backward_kernel / compute_chunk_prefix_suffix_kernel /
    // rasterize_backward_chunked_kernel (.metal:931-1135, 3139-3366).
    // One pixel's back-to-front walk over [s, min(e, bin_final + 1)).
    void pixel_backward(long long s, long long e, long long bin_final, R px, R py, R Tv, R buf[3], R Tfbg[3],
                        const R vo[3], R *contrib, long long &pairs) {
        long long hi = std::min(e - 1, bin_final);
        for (long long idx = hi; idx >= s; idx--) {
            const R *o = &pk[idx * 9];
            pairs++;
            R dx = o[0] - px, dy = o[1] - py;
            R sigma = FMA(CK<R>(0.5f), FMA(o[3], dx * dx, o[5] * dy * dy), o[4] * dx * dy);
            if (!finite_bits(sigma) || sigma < R(0) || (sigma >= CK<R>(5.55f) && !in.no_cutoff)) continue;
            R alpha = FMIN(CK<R>(0.999f), o[2] * EXP<R>(-sigma));
            if (alpha < CK<R>(1.f / 255.f) && !in.no_cutoff) continue;
            if (!(alpha < CK<R>(0.999f))) continue;   // clamped splats get no gradient (.metal:1085)
            R ra = R(1) / (R(1) - alpha);
            Tv *= ra;
            R fac = alpha * Tv;
            R rgb[3], tmp[3];
            for (int c = 0; c < 3; c++) {
                rgb[c] = FMAX(o[6 + c] + CK<R>(0.5f), R(0));
                tmp[c] = FMA(rgb[c], Tv, FMA(-buf[c], ra, -ra * Tfbg[c]));
            }
            R v_alpha = tmp[0] * vo[0] + tmp[1] * vo[1] + tmp[2] * vo[2];
            for (int c = 0; c < 3; c++) buf[c] = FMA(rgb[c], fac, buf[c]);
            R v_sigma = -alpha * v_alpha;
            R *g = &contrib[idx * 9];
            for (int c = 0; c < 3; c++)
                if (o[6 + c] + CK<R>(0.5f) >= R(0)) g[c] += fac * vo[c];
            R hv = CK<R>(0.5f) * v_sigma;
            g[3] += hv * (dx * dx); g[4] += hv * (dx * dy); g[5] += hv * (dy * dy);
            g[6] += v_sigma * FMA(o[3], dx, o[4] * dy);
            g[7] += v_sigma * FMA(o[4], dx, o[5] * dy);
            g[8] += -v_sigma * (R(1) - o[2]);
        }
    }

    void raster_backward() {
        const int W = in.width, H = in.height;
        const long long M = tile_start[T];
        std::vector<R> contrib((size_t)M * 9, R(0));
        long long pairs = 0;
        if (K > 1) {
            preT.assign((size_t)K * P, 0); aftC.assign((size_t)K * P * 3, 0);
#pragma omp parallel for schedule(static)
            for (int p = 0; p < P; p++) {
                R pT = 1;
                for (int k = 0; k < K; k++) { size_t o = (size_t)k * P + p; preT[o] = pT; pT *= chT[o]; }
                R aC[3] = {0, 0, 0};
                for (int k = K - 1; k >= 0; k--) {
                    size_t o = (size_t)k * P + p;
                    for (int c = 0; c < 3; c++) { aftC[3 * o + c] = aC[c]; aC[c] += preT[o] * chC[3 * o + c]; }
                }
            }
        }
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : pairs)
        for (int t = 0; t < T; t++) {
            int tx = t % cam.tiles_x, ty = t / cam.tiles_x;
            if (!row_in_band(ty)) continue;
            for (int yy = 0; yy < 16; yy++)
                for (int xx = 0; xx < 16; xx++) {
                    int x = tx * 16 + xx, y = ty * 16 + yy;
                    if (x >= W || y >= H) continue;
                    size_t p = (size_t)y * W + x;
                    R Tf = finalT[p];
                    R Tfbg[3] = {Tf * cam.bg[0], Tf * cam.bg[1], Tf * cam.bg[2]};
                    R vo[3] = {v_rend[3 * p], v_rend[3 * p + 1], v_rend[3 * p + 2]};
                    if (K <= 1) {
                        R buf[3] = {0, 0, 0};
                        pixel_backward(tile_start[t], tile_start[t + 1], final_idx[p], (R)x, (R)y, Tf, buf, Tfbg, vo,
                                       contrib.data(), pairs);
                    } else {
                        for (int k = 0; k < K; k++) {
                            long long cs = tile_start[t] + (long long)k * 512;
                            long long ce = std::min<long long>(tile_start[t] + (long long)(k + 1) * 512, tile_start[t + 1]);
                            size_t o = (size_t)k * P + p;
                            int bf = chIdx[o];
                            if (cs >= ce || bf < cs) continue;
                            R Tv = preT[o] * chT[o];
                            R buf[3] = {aftC[3 * o], aftC[3 * o + 1], aftC[3 * o + 2]};
                            pixel_backward(cs, ce, bf, (R)x, (R)y, Tv, buf, Tfbg, vo, contrib.data(), pairs);
                        }
                    }
                }
        }
        pairs_bwd = pairs;
        v_col.assign(3 * (size_t)N, 0); v_conic.assign(3 * (size_t)N, 0); v_xy.assign(2 * (size_t)N, 0); v_op.assign(N, 0);
        for (long long i = 0; i < M; i++) {
            int g = ids[i];
            const R *c = &contrib[i * 9];
            for (int k = 0; k < 3; k++) v_col[3 * g + k] += c[k];
            for (int k = 0; k < 3; k++) v_conic[3 * g + k] += c[3 + k];
            v_xy[2 * g] += c[6]; v_xy[2 * g + 1] += c[7];
            v_op[g] += c[8];
        }
    }

    // project_and_sh_backward_kernel, .metal:1860-2042 (+ VJPs .metal:1252-1569)
    void project_backward() {
        v_mean.assign(3 * (size_t)N, 0); v_scale.assign(3 * (size_t)N, 0); v_quat.assign(4 * (size_t)N, 0);
        const int rb = in.rest_bases;
        uint32_t nsh = 0;
#pragma omp parallel for schedule(static) reduction(+ : nsh)
        for (int i = 0; i < N; i++) {
            if (radii[i] <= 0) continue;
            const float *mp = in.means + 3 * (size_t)i;
            R p[3] = {(R)mp[0], (R)mp[1], (R)mp[2]};
            const R *m = cam.pm;
            // project_pix_vjp (.metal:1252-1270)
            R phw = m[12] * p[0] + m[13] * p[1] + m[14] * p[2] + m[15];
            R rw = R(1) / (phw + CK<R>(1e-6f));
            R vnx = CK<R>(0.5f) * cam.W * v_xy[2 * i], vny = CK<R>(0.5f) * cam.H * v_xy[2 * i + 1];
            R vp[4] = {vnx * rw, vny * rw, 0, -(vnx + vny) * rw * rw};
            R vm_[3];
            for (int c = 0; c < 3; c++) vm_[c] = m[c] * vp[0] + m[4 + c] * vp[1] + m[8 + c] * vp[2];
            // cov2d_to_conic_vjp (.metal:1289-1300): v_Sigma = -X G X
            R X[2][2] = {{conics[3 * i], conics[3 * i + 1]}, {conics[3 * i + 1], conics[3 * i + 2]}};
            R Gm[2][2] = {{v_conic[3 * i], v_conic[3 * i + 1]}, {v_conic[3 * i + 1], v_conic[3 * i + 2]}};
            R XG[2][2], VS[2][2];
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 2; c++) XG[r][c] = X[r][0] * Gm[0][c] + X[r][1] * Gm[1][c];
            for (int r = 0; r < 2; r++)
                for (int c = 0; c < 2; c++) VS[r][c] = -(XG[r][0] * X[0][c] + XG[r][1] * X[1][c]);
            R vc2[3] = {VS[0][0], VS[1][0] + VS[0][1], VS[1][1]};
            // recompute cov3d
            R s[3], q[4], cov[6];
            for (int k = 0; k < 3; k++)
                s[k] = EXP<R>(FMIN(FMAX((R)in.scales[3 * (size_t)i + k], CK<R>(-15.f)), CK<R>(15.f)));
            for (int k = 0; k < 4; k++) q[k] = (R)in.quats[4 * (size_t)i + k];
            scale_rot_to_cov3d(s, q, cov);
            // project_cov3d_ewa_vjp (.metal:1375-1443)
            const R *v = cam.vm;
            R pv[3] = {v[0] * p[0] + v[1] * p[1] + v[2] * p[2] + v[3], v[4] * p[0] + v[5] * p[1] + v[6] * p[2] + v[7],
                       v[8] * p[0] + v[9] * p[1] + v[10] * p[2] + v[11]};
            R lim_x = CK<R>(1.3f) * cam.tan_fovx, lim_y = CK<R>(1.3f) * cam.tan_fovy;
            R pz = pv[2];
            R px = pz * FMIN(lim_x, FMAX(-lim_x, pv[0] / pz));
            R py = pz * FMIN(lim_y, FMAX(-lim_y, pv[1] / pz));
            R rz = R(1) / pz, rz2 = rz * rz;
            R Wm[3][3], J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, V[3][3], vcov[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) Wm[r][c] = v[4 * r + c];
            J[0][0] = cam.fx * rz; J[1][1] = cam.fy * rz;
            J[0][2] = -cam.fx * px * rz2; J[1][2] = -cam.fy * py * rz2;
            V[0][0] = cov[0]; V[0][1] = V[1][0] = cov[1]; V[0][2] = V[2][0] = cov[2];
            V[1][1] = cov[3]; V[1][2] = V[2][1] = cov[4]; V[2][2] = cov[5];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) vcov[r][c] = 0;
            vcov[0][0] = vc2[0]; vcov[0][1] = vcov[1][0] = CK<R>(0.5f) * vc2[1]; vcov[1][1] = vc2[2];
            auto mul = [](const R A[3][3], const R B[3][3], R C[3][3]) {
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) C[r][c] = A[r][0] * B[0][c] + A[r][1] * B[1][c] + A[r][2] * B[2][c];
            };
            auto tr = [](const R A[3][3], R B[3][3]) {
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) B[r][c] = A[c][r];
            };
            R Tm[3][3], Tt[3][3], tmp[3][3], vV[3][3], vT[3][3], tmp2[3][3], Vt[3][3], vcovT[3][3];
            mul(J, Wm, Tm);
            tr(Tm, Tt);
            mul(Tt, vcov, tmp); mul(tmp, Tm, vV);                 // v_V = T^T v_cov T
            tr(V, Vt); tr(vcov, vcovT);
            mul(vcov, Tm, tmp); mul(tmp, Vt, vT);                 // v_cov T V^T
            mul(vcovT, Tm, tmp); mul(tmp, V, tmp2);               // + v_cov^T T V
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) vT[r][c] += tmp2[r][c];
            R vcov3[6] = {vV[0][0], vV[0][1] + vV[1][0], vV[0][2] + vV[2][0], vV[1][1], vV[1][2] + vV[2][1], vV[2][2]};
            R Wt[3][3], vJ[3][3];
            tr(Wm, Wt);
            mul(vT, Wt, vJ);
            R fxr = cam.fx * rz2, fyr = cam.fy * rz2, rz3 = rz2 * rz;
            R vt[3] = {-fxr * vJ[0][2], -fyr * vJ[1][2],
                       -fxr * vJ[0][0] + R(2) * cam.fx * px * rz3 * vJ[0][2] - fyr * vJ[1][1] +
                           R(2) * cam.fy * py * rz3 * vJ[1][2]};
            for (int c = 0; c < 3; c++) vm_[c] += vt[0] * Wm[0][c] + vt[1] * Wm[1][c] + vt[2] * Wm[2][c];
            for (int c = 0; c < 3; c++) v_mean[3 * i + c] = vm_[c];
            // scale_rot_to_cov3d_vjp (.metal:1536-1569) + quat_to_rotmat_vjp (.metal:1445-1490)
            R vVs[3][3] = {{vcov3[0], CK<R>(0.5f) * vcov3[1], CK<R>(0.5f) * vcov3[2]},
                           {CK<R>(0.5f) * vcov3[1], vcov3[3], CK<R>(0.5f) * vcov3[4]},
                           {CK<R>(0.5f) * vcov3[2], CK<R>(0.5f) * vcov3[4], vcov3[5]}};
            R w, x, y, z;
            Mat3<R> Rm = quat_to_rotmat(q, w, x, y, z);
            R Mm[3][3], vM[3][3], vR[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) Mm[r][c] = Rm.m[r][c] * s[c];
            mul(vVs, Mm, vM);
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) vM[r][c] = R(2) * vM[r][c];
            for (int c = 0; c < 3; c++)
                v_scale[3 * i + c] = (Rm.m[0][c] * vM[0][c] + Rm.m[1][c] * vM[1][c] + Rm.m[2][c] * vM[2][c]) * s[c];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) vR[r][c] = vM[r][c] * s[c];
            // Metal v_R[i][j] = column i, row j
            auto g = [&](int ci, int rj) { return vR[rj][ci]; };
            v_quat[4 * i + 0] = R(2) * (x * (g(1, 2) - g(2, 1)) + y * (g(2, 0) - g(0, 2)) + z * (g(0, 1) - g(1, 0)));
            v_quat[4 * i + 1] = R(2) * (-R(2) * x * (g(1, 1) + g(2, 2)) + y * (g(0, 1) + g(1, 0)) + z * (g(0, 2) + g(2, 0)) +
                                        w * (g(1, 2) - g(2, 1)));
            v_quat[4 * i + 2] = R(2) * (x * (g(0, 1) + g(1, 0)) - R(2) * y * (g(0, 0) + g(2, 2)) + z * (g(1, 2) + g(2, 1)) +
                                        w * (g(2, 0) - g(0, 2)));
            v_quat[4 * i + 3] = R(2) * (x * (g(0, 2) + g(2, 0)) + y * (g(1, 2) + g(2, 1)) - R(2) * z * (g(0, 0) + g(1, 1)) +
                                        w * (g(0, 1) - g(1, 0)));
            // fused SH backward + Adam (.metal:1960-2041)
            if (!in.do_optimizer) continue;
            R vc[3] = {v_col[3 * i], v_col[3 * i + 1], v_col[3 * i + 2]};
            if (!(finite_bits(vc[0]) && finite_bits(vc[1]) && finite_bits(vc[2]))) { nsh++; continue; }
            for (int c = 0; c < 3; c++)
                adam(in.features_dc + 3 * (size_t)i + c, in.exp_avg[3] + 3 * (size_t)i + c, in.exp_avg_sq[3] + 3 * (size_t)i + c,
                     CK<R>(SH_C0) * vc[c], 3);
            int nb = in.degrees_to_use >= 3 ? 15 : in.degrees_to_use == 2 ? 8 : in.degrees_to_use == 1 ? 3 : 0;
            if (nb > rb) nb = rb;
            if (nb == 0) continue;
            R d[3], bas[15];
            viewdir(mp, cam, d);
            sh_basis(d, bas);
            for (int b = 0; b < nb; b++)
                for (int c = 0; c < 3; c++) {
                    size_t k = (size_t)rb * 3 * i + b * 3 + c;
                    adam(in.features_rest + k, in.exp_avg[4] + k, in.exp_avg_sq[4] + k, bas[b] * vc[c], 4);
                }
        }
        nan[3] += nsh;
    }

    // adam_update_element (.metal:1838-1847) / fused_adam_kernel (.metal:1680-1713)
    void adam(float *p, float *ea, float *eas, R g, int grp) {
        R b1 = (R)in.beta1, b2 = (R)in.beta2;
        R m = FMA(b1, (R)*ea, (R(1) - b1) * g);
        R v = FMA(b2, (R)*eas, (R(1) - b2) * g * g);
        R np = (R)*p - (R)in.step_size[grp] * m / (SQRT(v) / (R)in.bc2_sqrt[grp] + (R)in.eps);
        *p = (float)np; *ea = (float)m; *eas = (float)v;
    }

    // mcmc_reg_grad_kernel (.metal:3987-4026) then fused_adam_kernel on groups 0,1,2,5
    void optimizer() {
        const bool reg = in.op_reg > 0.0f || in.sc_reg > 0.0f;
        std::vector<R> gs = v_scale, go = v_op;
        if (reg) {
            for (int i = 0; i < N; i++) {
                const float *dv = in.exp_avg_sq[3] + 3 * (size_t)i;
                R vdc = (R)dv[0] + (R)dv[1] + (R)dv[2];
                R duty = (vdc == R(0)) ? R(1) : (R)in.invis_scale;
                R invN = duty / (R)(float)N;
                R sig = R(1) / (R(1) + EXP<R>(-(R)in.opacities[i]));
                go[i] += (R)in.op_reg * sig * (R(1) - sig) * invN;
                R inv3N = invN * CK<R>(1.0f / 3.0f);
                for (int k = 0; k < 3; k++) {
                    R s = (R)in.scales[3 * (size_t)i + k];
                    gs[3 * i + k] += (R)in.sc_reg * EXP<R>(FMIN(FMAX(s, CK<R>(-15.f)), CK<R>(15.f))) * inv3N;
                }
            }
        }
        struct G { float *p, *m, *v; const R *g; size_t n; int idx; };
        G groups[4] = {{in.means, in.exp_avg[0], in.exp_avg_sq[0], v_mean.data(), 3 * (size_t)N, 0},
                       {in.scales, in.exp_avg[1], in.exp_avg_sq[1], gs.data(), 3 * (size_t)N, 1},
                       {in.quats, in.exp_avg[2], in.exp_avg_sq[2], v_quat.data(), 4 * (size_t)N, 2},
                       {in.opacities, in.exp_avg[5], in.exp_avg_sq[5], go.data(), (size_t)N, 5}};
        for (auto &gr : groups) {
            uint32_t bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
            for (long long e = 0; e < (long long)gr.n; e++) {
                R g = gr.g[e];
                if (!finite_bits(g)) { bad++; continue; }
                adam(gr.p + e, gr.m + e, gr.v + e, g, gr.idx);
            }
            nan[gr.idx] += bad;
        }
    }

    // sgld_noise_gen_kernel + sgld_noise_kernel (.metal:3862-3967)
    void sgld() {
        auto hash = [](uint32_t seed, uint32_t idx) {
            uint32_t x = seed * 747796405u + idx * 2891336453u;
            x = ((x >> ((x >> 28) + 4)) ^ x) * 277803737u;
            return (x >> 22) ^ x;
        };
        auto unit = [](uint32_t h) { return ((float)(h >> 9) + 0.5f) * (1.0f / (float)(1u << 23)); };
#pragma omp parallel for schedule(static)
        for (int i = 0; i < N; i++) {
            uint32_t base = (uint32_t)i * 4u;
            float u0 = unit(hash(in.seed, base)), u1 = unit(hash(in.seed, base + 1)), u2 = unit(hash(in.seed, base + 2)),
                  u3 = unit(hash(in.seed, base + 3));
            R r01 = SQRT(R(-2) * std::log((R)u0)), r23 = SQRT(R(-2) * std::log((R)u2));
            R a01 = CK<R>(6.283185307179586f) * (R)u1, a23 = CK<R>(6.283185307179586f) * (R)u3;
            R nz[3] = {r01 * std::cos(a01), r01 * std::sin(a01), r23 * std::cos(a23)};
            R op = R(1) / (R(1) + EXP<R>(-(R)in.opacities[i]));
            R wgt = R(1) / (R(1) + EXP<R>(CK<R>(-100.0f) * ((R(1) - op) - CK<R>(0.995f))));
            R ns = (R)in.noise_lr * (R)in.xyz_lr * wgt;
            R n0 = nz[0] * ns, n1 = nz[1] * ns, n2 = nz[2] * ns;
            const float *qp = in.quats + 4 * (size_t)i;
            R qw = qp[0], qx = qp[1], qy = qp[2], qz = qp[3];
            R ql = SQRT(FMAX(qw * qw + qx * qx + qy * qy + qz * qz, CK<R>(1e-8f)));
            qw /= ql; qx /= ql; qy /= ql; qz /= ql;
            R sc[3];
            for (int k = 0; k < 3; k++) sc[k] = EXP<R>(FMIN(FMAX((R)in.scales[3 * (size_t)i + k], CK<R>(-15.f)), CK<R>(15.f)));
            R rt0 = (R(1) - R(2) * (qy * qy + qz * qz)) * n0 + R(2) * (qx * qy + qw * qz) * n1 + R(2) * (qx * qz - qw * qy) * n2;
            R rt1 = R(2) * (qx * qy - qw * qz) * n0 + (R(1) - R(2) * (qx * qx + qz * qz)) * n1 + R(2) * (qy * qz + qw * qx) * n2;
            R rt2 = R(2) * (qx * qz + qw * qy) * n0 + R(2) * (qy * qz - qw * qx) * n1 + (R(1) - R(2) * (qx * qx + qy * qy)) * n2;
            rt0 *= sc[0] * sc[0]; rt1 *= sc[1] * sc[1]; rt2 *= sc[2] * sc[2];
            R v0 = (R(1) - R(2) * (qy * qy + qz * qz)) * rt0 + R(2) * (qx * qy - qw * qz) * rt1 + R(2) * (qx * qz + qw * qy) * rt2;
            R v1 = R(2) * (qx * qy + qw * qz) * rt0 + (R(1) - R(2) * (qx * qx + qz * qz)) * rt1 + R(2) * (qy * qz - qw * qx) * rt2;
            R v2 = R(2) * (qx * qz - qw * qy) * rt0 + R(2) * (qy * qz + qw * qx) * rt1 + (R(1) - R(2) * (qx * qx + qy * qy)) * rt2;
            if (!finite_bits(v0) || !finite_bits(v1) || !finite_bits(v2)) continue;
            R len2 = v0 * v0 + v1 * v1 + v2 * v2;
            if (!finite_bits(len2)) continue;
            R md = (R)in.max_disp;
            if (len2 > md * md) { R inv = md / SQRT(len2); v0 *= inv; v1 *= inv; v2 *= inv; }
            float *mp = in.means + 3 * (size_t)i;
            mp[0] = (float)((R)mp[0] + v0); mp[1] = (float)((R)mp[1] + v1); mp[2] = (float)((R)mp[2] + v2);
        }
    }

    // K_max rule, msplat_metal.mm:1204-1224
    int choose_k(long long capacity) const {
        int mode = in.raster_mode;
        if (mode == 1) return 1;
        if (mode == 0 && T >= 400) return 1;
        if (in.k_max > 0) return in.k_max;
        uint32_t avg = (uint32_t)(capacity / std::max(1, T));
        uint32_t cons = avg * 6;
        uint32_t k = (cons + 511) / 512;
        if (k < 2) k = 2;
        uint32_t am = (uint32_t)((capacity + 511) / 512);
        if (k > am) k = am;
        return (int)k;
    }

    template <class A, class B> static void put(B *dst, const std::vector<A> &src, size_t n) {
        if (!dst) return;
        for (size_t i = 0; i < n && i < src.size(); i++) dst[i] = (B)src[i];
    }

    int run(OrStepOut *out) {
        setup();
        long long cap = in.isect_capacity > 0 ? in.isect_capacity : 48LL * N;
        project();
        build_tiles(cap);
        K = choose_k(cap);
        raster_forward();
        const bool has_gt = in.gt != nullptr;
        if (has_gt) loss();
        double dot = 0;
        if (in.v_img_in) {
            v_rend.assign(in.v_img_in, in.v_img_in + 3 * (size_t)P);
            for (size_t k = 0; k < 3 * (size_t)P; k++) dot += (double)img[k] * (double)in.v_img_in[k];
        }
        if (in.do_backward && (has_gt || in.v_img_in || in.raster_grads_in)) {
            if (in.raster_grads_in) {
                v_xy.assign(2 * (size_t)N, 0); v_conic.assign(3 * (size_t)N, 0);
                v_col.assign(3 * (size_t)N, 0); v_op.assign(N, 0);
                for (int i = 0; i < N; i++) {
                    const float *g = in.raster_grads_in + 9 * (size_t)i;
                    v_xy[2 * i] = g[0]; v_xy[2 * i + 1] = g[1];
                    for (int k = 0; k < 3; k++) { v_conic[3 * i + k] = g[2 + k]; v_col[3 * i + k] = g[5 + k]; }
                    v_op[i] = g[8];
                }
            } else {
                raster_backward();
            }
            project_backward();
            if (in.do_optimizer) optimizer();
        }
        if (in.do_sgld) sgld();
        // outputs
        put(out->xys, xys, 2 * (size_t)N); put(out->depths, depths, N); put(out->conics, conics, 3 * (size_t)N);
        put(out->colors, colors, 3 * (size_t)N); put(out->aabb, aabb, 2 * (size_t)N);
        put(out->radii, radii, N); put(out->num_tiles_hit, tiles_hit, N);
        put(out->tile_counts, tile_counts, T);
        if (out->tile_bins)
            for (int t = 0; t < T; t++) { out->tile_bins[2 * t] = tile_start[t]; out->tile_bins[2 * t + 1] = tile_start[t + 1]; }
        out->num_isect = tile_start[T];
        if (out->gaussian_ids) put(out->gaussian_ids, ids, (size_t)std::min<long long>(out->ids_capacity, tile_start[T]));
        put(out->out_img, img, 3 * (size_t)P); put(out->final_Ts, finalT, P); put(out->final_idx, final_idx, P);
        out->loss = loss_sum / (double)P;
        put(out->v_rendered, v_rend, 3 * (size_t)P);
        put(out->v_xy, v_xy, 2 * (size_t)N); put(out->v_conic, v_conic, 3 * (size_t)N);
        put(out->v_colors, v_col, 3 * (size_t)N); put(out->v_opacity, v_op, N);
        put(out->v_mean3d, v_mean, 3 * (size_t)N); put(out->v_scale, v_scale, 3 * (size_t)N);
        put(out->v_quat, v_quat, 4 * (size_t)N);
        for (int k = 0; k < 16; k++) out->nan_counts[k] = nan[k];
        out->k_max_used = K;
        out->pairs_fwd = pairs_fwd; out->pairs_bwd = pairs_bwd;
        out->img_dot_v = dot;
        return 0;
    }
};

}  // namespace

extern "C" {

float or_det_expf(float x) { return det_expf(x); }

// The SSIM window the float path uses (.metal:3376-3380).
void or_gauss_1d(float out[11]) { gauss_1d<float>(out); }

int or_train_step(int prec, const OrStepIn *in, OrStepOut *out) {
    if (!in || !out || in->num_points < 0 || in->width <= 0 || in->height <= 0) return -1;
    if (prec == 64) { Step<double> s(*in); return s.run(out); }
    if (prec == 32) { Step<float> s(*in); return s.run(out); }
    return -2;
}

// model.cpp:311-332
void or_compute_relocation(float o_old, const float *s_old, int n, float *o_new_out, float *s_new) {
    if (n < 1) n = 1;
    if (n > 51) n = 51;
    float o_new = 1.0f - std::pow(1.0f - o_old, 1.0f / (float)n);
    const double on = (double)o_new;
    double denom = 0.0, binom = 1.0;
    for (int k = 1; k <= n; k++) {
        binom = binom * (double)(n - k + 1) / (double)k;
        const double term = binom * std::pow(on, (double)k) / std::sqrt((double)k);
        denom += (k % 2 == 1) ? term : -term;
    }
    double coeff = (denom > 1e-12) ? ((double)o_old / denom) : 1.0;
    if (!std::isfinite(coeff) || coeff <= 0.0) coeff = 1.0;
    for (int i = 0; i < 3; i++) s_new[i] = (float)((double)s_old[i] * coeff);
    *o_new_out = o_new;
}

// model.cpp:845-889
void or_prepare_cam(const float c2w[16], int width, int height, float fx, float fy, float vm[16], float pvm[16],
                    float campos[3]) {
    float fovX = 2.0f * std::atan(width / (2.0f * fx));
    float fovY = 2.0f * std::atan(height / (2.0f * fy));
    float R[3][3], Ri[3][3], T[3], Ti[3];
    for (int i = 0; i < 3; i++) { R[i][0] = c2w[i * 4 + 0]; R[i][1] = -c2w[i * 4 + 1]; R[i][2] = -c2w[i * 4 + 2]; T[i] = c2w[i * 4 + 3]; }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Ri[i][j] = R[j][i];
    for (int i = 0; i < 3; i++) Ti[i] = -(Ri[i][0] * T[0] + Ri[i][1] * T[1] + Ri[i][2] * T[2]);
    float v[16] = {Ri[0][0], Ri[0][1], Ri[0][2], Ti[0], Ri[1][0], Ri[1][1], Ri[1][2], Ti[1],
                   Ri[2][0], Ri[2][1], Ri[2][2], Ti[2], 0, 0, 0, 1};
    float t_p = 0.001f * std::tan(0.5f * fovY), r_p = 0.001f * std::tan(0.5f * fovX);
    float pm[16] = {0.001f / r_p, 0, 0, 0, 0, 0.001f / t_p, 0, 0, 0, 0, (1000.0f + 0.001f) / (1000.0f - 0.001f),
                    -1000.0f * 0.001f / (1000.0f - 0.001f), 0, 0, 1, 0};
    float out[16] = {};
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < 4; k++) out[i * 4 + j] += pm[i * 4 + k] * v[k * 4 + j];
    std::memcpy(vm, v, sizeof(v));
    std::memcpy(pvm, out, sizeof(out));
    for (int i = 0; i < 3; i++) campos[i] = T[i];
}

double or_psnr(const float *r, const float *g, long long n) {
    double mse = 0;
    for (long long i = 0; i < n; i++) { double d = r[i] - g[i]; mse += d * d; }
    mse /= n;
    return (float)(10.0f * std::log10(1.0 / mse));
}

double or_l1(const float *r, const float *g, long long n) {
    double s = 0;
    for (long long i = 0; i < n; i++) s += std::abs(r[i] - g[i]);
    return (float)(s / n);
}

// ssim.cpp:61-123 (replicate padding, float kernel from float exp)
double or_ssim_eval(const float *r, const float *g, int H, int W) {
    const int ks = 11, pad = 5;
    float kern[11], ksum = 0;
    for (int i = 0; i < ks; i++) { float x = (float)(i - ks / 2); kern[i] = std::exp(-(x * x) / (2.0f * 1.5f * 1.5f)); ksum += kern[i]; }
    for (int i = 0; i < ks; i++) kern[i] /= ksum;
    const size_t HW = (size_t)H * W;
    std::vector<float> rc(HW), gc(HW), rr(HW), gg(HW), rg(HW), m1(HW), m2(HW), srr(HW), sgg(HW), srg(HW), tmp(HW);
    auto blur = [&](const float *in, float *out) {
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                float s = 0;
                for (int k = 0; k < ks; k++) { int sx = std::min(std::max(x + k - pad, 0), W - 1); s += in[(size_t)y * W + sx] * kern[k]; }
                tmp[(size_t)y * W + x] = s;
            }
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                float s = 0;
                for (int k = 0; k < ks; k++) { int sy = std::min(std::max(y + k - pad, 0), H - 1); s += tmp[(size_t)sy * W + x] * kern[k]; }
                out[(size_t)y * W + x] = s;
            }
    };
    const float C1 = 0.01f * 0.01f, C2 = 0.03f * 0.03f;
    double sum = 0;
    long long cnt = 0;
    for (int c = 0; c < 3; c++) {
        for (size_t i = 0; i < HW; i++) {
            rc[i] = r[i * 3 + c]; gc[i] = g[i * 3 + c];
            rr[i] = rc[i] * rc[i]; gg[i] = gc[i] * gc[i]; rg[i] = rc[i] * gc[i];
        }
        blur(rc.data(), m1.data()); blur(gc.data(), m2.data());
        blur(rr.data(), srr.data()); blur(gg.data(), sgg.data()); blur(rg.data(), srg.data());
        for (size_t i = 0; i < HW; i++) {
            float a = m1[i] * m1[i], b = m2[i] * m2[i], ab = m1[i] * m2[i];
            float s1 = srr[i] - a, s2 = sgg[i] - b, s12 = srg[i] - ab;
            float num = (2.0f * ab + C1) * (2.0f * s12 + C2);
            float den = (a + b + C1) * (s1 + s2 + C2);
            sum += num / den;
            cnt++;
        }
    }
    return (float)(sum / cnt);
}

// model.cpp:497-566 (dead classification)
int or_mcmc_dead_mask(int n, int rs, const float *mn, const float *sc, const float *qt, const float *fdc,
                      const float *fr, const float *op, float cull_radius, uint8_t *dead) {
    const float r2 = cull_radius > 0.0f ? cull_radius * cull_radius : -1.0f;
    int cnt = 0;
    for (int i = 0; i < n; i++) {
        bool fin = std::isfinite(op[i]);
        for (int k = 0; k < 3; k++) fin = fin && std::isfinite(mn[3 * i + k]) && std::isfinite(sc[3 * i + k]) && std::isfinite(fdc[3 * i + k]);
        for (int k = 0; k < 4; k++) fin = fin && std::isfinite(qt[4 * i + k]);
        for (int k = 0; fin && k < rs; k++) fin = std::isfinite(fr[(size_t)i * rs + k]);
        float sig = 1.0f / (1.0f + std::exp(-op[i]));
        bool d = !fin || (sig <= 0.005f);
        if (!d && r2 > 0.0f) {
            float x = mn[3 * i], y = mn[3 * i + 1], z = mn[3 * i + 2];
            if (x * x + y * y + z * z > r2) d = true;
        }
        dead[i] = d ? 1 : 0;
        cnt += d;
    }
    return cnt;
}

// model.cpp:380-416 / 465-491 given the chosen sources
void or_mcmc_apply(int n_moves, const int *dst, const int *src, int rs, float *mn, float *sc, float *qt, float *fdc,
                   float *fr, float *op, float **ea, float **eas, const int *gstride) {
    std::vector<int> count;
    int maxs = 0;
    for (int i = 0; i < n_moves; i++) maxs = std::max(maxs, src[i] + 1);
    count.assign(maxs, 0);
    for (int i = 0; i < n_moves; i++) count[src[i]]++;
    auto zero = [&](int idx) {
        for (int g = 0; g < 6; g++) {
            std::memset(ea[g] + (size_t)idx * gstride[g], 0, sizeof(float) * gstride[g]);
            std::memset(eas[g] + (size_t)idx * gstride[g], 0, sizeof(float) * gstride[g]);
        }
    };
    for (int s = 0; s < maxs; s++) {
        if (count[s] == 0) continue;
        float o_old = 1.0f / (1.0f + std::exp(-op[s]));
        float s_old[3] = {std::exp(sc[3 * s]), std::exp(sc[3 * s + 1]), std::exp(sc[3 * s + 2])};
        float o_new, s_new[3];
        or_compute_relocation(o_old, s_old, count[s] + 1, &o_new, s_new);
        o_new = std::clamp(o_new, 1e-6f, 1.0f - 1e-6f);
        op[s] = std::log(o_new / (1.0f - o_new));
        for (int j = 0; j < 3; j++) sc[3 * s + j] = std::log(std::max(s_new[j], 1e-10f));
        zero(s);
    }
    for (int i = 0; i < n_moves; i++) {
        int d = dst[i], s = src[i];
        std::memcpy(mn + 3 * (size_t)d, mn + 3 * (size_t)s, 12);
        std::memcpy(qt + 4 * (size_t)d, qt + 4 * (size_t)s, 16);
        std::memcpy(fdc + 3 * (size_t)d, fdc + 3 * (size_t)s, 12);
        std::memcpy(fr + (size_t)rs * d, fr + (size_t)rs * s, sizeof(float) * rs);
        op[d] = op[s];
        std::memcpy(sc + 3 * (size_t)d, sc + 3 * (size_t)s, 12);
        zero(d);
    }
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
