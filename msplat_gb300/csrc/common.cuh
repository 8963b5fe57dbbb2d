// Shared device definitions of the msplat GB300 engine.
//
// Layouts (N = active Gaussians, P = H*W pixels, T = 16x16 tiles, M = tile
// intersections):
//   params      means[N,3] scales[N,3] (log) quats[N,4] (w,x,y,z)
//               features_dc[N,3] features_rest[N,B,3] opacities[N] (logit)
//   SplatRec    per Gaussian, 48 B: projected centre, sigmoid(opacity),
//               conic, raw SH colour, reach box (written by the projection)
//   isect_ids   per intersection, 4 B: the Gaussian (record) id, in per-tile
//               depth order (written by the sort)
//   GradRec     per Gaussian, 48 B: rasterizer gradients (xy, opacity logit;
//               conic; colour), accumulated with vector atomics
#pragma once

#include <mutex>
#include <cstdint>
#include <cuda_runtime.h>

namespace msplat {

constexpr int kTile = 16;           // tile edge (msplat.hpp BLOCK_X/BLOCK_Y)
constexpr int kTileThreads = 256;   // one thread per tile pixel
constexpr int kChunk = 512;         // depth-chunk length of the chunked raster (the reference's; tunable)

struct SplatRec {
    float4 a;   // x, y, opacity (sigmoid), unused
    float4 b;   // conic a, b, c, reach half-extent x (pixels)
    float4 c;   // raw SH colour r, g, b, reach half-extent y
};

struct GradRec {
    float4 a;   // v_x, v_y, v_opacity_logit, 0
    float4 b;   // v_conic a, b, c, 0
    float4 c;   // v_colour r, g, b, 0
};

// Per-step scalars, resident on the device so that a captured step can be
// replayed with new values (kernels take a pointer, not the values).
struct StepParams {
    float viewmat[16];
    float projmat[16];
    float fx, fy, cx, cy;
    float tan_fovx, tan_fovy;
    float cam_pos[3];
    float bg[3];
    float clip_thresh;
    int degrees_to_use;
    float ssim_weight, loss_inv_n;
    float step_size[6], bc2_sqrt[6];
    float beta1, beta2, eps;
    float op_reg, sc_reg, invis_scale;
    uint32_t seed;
    float noise_lr, xyz_lr, max_disp;
    int has_mask;
    int pad_[3];
    // target image and mask of this step (device; the mask may be null): read
    // from here, not from kernel arguments, so one captured step serves every
    // view of the same size
    const uint8_t *gt;
    const uint8_t *mask;
};

// Telemetry slots of the non-finite counters (same numbering as the
// reference's grad_nan_counts, msplat_metal.mm:535-543 and model.cpp:597-636).
enum NanSlot {
    kNanMean = 0, kNanScale = 1, kNanQuat = 2, kNanSH = 3, kNanSsimWin = 4, kNanOpacity = 5,
    kNanVRendered = 6, kNanProj = 7, kNanProjCenter = 8, kNanProjDepth = 9, kNanProjAabb = 10,
    kNanProjConic = 11, kNanProjRgb = 12, kNanPack = 13, kNanPackOpacity = 14, kNanRasterSigma = 15
};

// Programmatic dependent launch.  The step's kernels are launched with
// launch_pdl, so a kernel's launch is prepared while its predecessor in the
// stream drains; every such kernel starts with pdl_enter, which waits for
// the predecessor grid to complete with its memory visible (before any
// global load or store).  The predecessor lets it go when its blocks exit
// (no early trigger: successor blocks parked on SMs during the predecessor's
// last wave made the captured step slower, 1.392 -> 1.456 ms, against
// 1.377 ms this way).  A kernel after a non-kernel stream operation, or
// launched plainly, behaves as usual.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Runs set_up once per device (kernel attributes and constant banks belong
// to the device current at the call), under a lock.  A device is marked done
// only when set_up returned cudaSuccess, so a failed first call is retried
// by the next one; the error is returned.
template <class F> inline cudaError_t once_per_device(std::mutex &mu, bool (&done)[64], F &&set_up) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return set_up();
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return cudaSuccess;
    e = set_up();
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

__device__ __forceinline__ bool finite_bits(float x) {
    return (__float_as_uint(x) & 0x7F800000u) != 0x7F800000u;
}

// Deterministic exp: Cody-Waite reduction x = n*ln2 + r with ln2 split
// hi/lo, degree-7 Taylor polynomial of e^r (|r| <= ln2/2) in Horner form with
// fused multiply-adds, exact power-of-two scaling.  Only IEEE-rounded
// operations, so the host oracle's copy of this algorithm gives the same bits.
__device__ __forceinline__ float det_expf(float x) {
    if (x != x) return x;
    if (x > 88.72283f) return __int_as_float(0x7f800000);
    if (x < -87.33654f) return 0.0f;
    const float n = rintf(__fmul_rn(x, 1.44269504088896341f));
    float r = __fmaf_rn(n, -0.693145751953125f, x);
    r = __fmaf_rn(n, -1.42860676533018e-06f, r);
    float p = 1.0f / 5040.0f;
    p = __fmaf_rn(p, r, 1.0f / 720.0f);
    p = __fmaf_rn(p, r, 1.0f / 120.0f);
    p = __fmaf_rn(p, r, 1.0f / 24.0f);
    p = __fmaf_rn(p, r, 1.0f / 6.0f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    int ni = (int)n;
    float scale_lo = 1.0f;
    if (ni > 127) { scale_lo = 2.0f; ni -= 1; }
    if (ni < -126) { scale_lo = 0.5f; ni += 1; }
    const float two_n = __uint_as_float((uint32_t)(ni + 127) << 23);
    return __fmul_rn(__fmul_rn(p, two_n), scale_lo);
}

// Adam's parameter step st * m / (sqrt(v) / bc + eps) (fused_adam_kernel,
// msplat_metal.metal:1680-1713), both divisions by the fast reciprocal
// (within 2 ulp, as the reference's fast-math division): the IEEE divisions
// were most of the optimizer kernels' instructions.
__device__ __forceinline__ float adam_delta(float st, float m, float v, float bc, float eps) {
    return __fdividef(st * m, __fdividef(sqrtf(v), bc) + eps);
}

// det_expf for x in [-87, 0] (the rasterizers' -sigma, sigma in [0, 5.55)):
// the same operations without the NaN, overflow and subnormal branches, which
// cannot trigger there, so the same bits.
__device__ __forceinline__ float det_expf_neg(float x) {
    const float n = rintf(__fmul_rn(x, 1.44269504088896341f));
    float r = __fmaf_rn(n, -0.693145751953125f, x);
    r = __fmaf_rn(n, -1.42860676533018e-06f, r);
    float p = 1.0f / 5040.0f;
    p = __fmaf_rn(p, r, 1.0f / 720.0f);
    p = __fmaf_rn(p, r, 1.0f / 120.0f);
    p = __fmaf_rn(p, r, 1.0f / 24.0f);
    p = __fmaf_rn(p, r, 1.0f / 6.0f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    const float two_n = __uint_as_float((uint32_t)((int)n + 127) << 23);
    return __fmul_rn(p, two_n);
}

// A sigma beyond which a splat of opacity op composites nothing: alpha =
// op * exp(-sigma) < 1/255 for every sigma > ln(255 op), and the margin of
// 1e-4 (a factor e^-1e-4 on alpha) covers the rounding of the exponential,
// of the product and of this logarithm (each within a few 1e-7 relative), so
// the rasterizers may skip such a pair without evaluating alpha: its alpha
// test fails either way.  +inf (nothing skipped) for a NaN opacity, whose
// alpha the reference's fmin turns into 0.999; -inf for a zero opacity.
__device__ __forceinline__ float sigma_cut(float op) {
    if (!(op >= 0.f)) return __int_as_float(0x7f800000);
    return op > 0.f ? logf(255.f * op) + 1e-4f : __int_as_float(0xff800000);
}

// Tile rectangle of a splat, inclusive min / exclusive max (get_tile_bbox,
// msplat_metal.metal:57-87).  Truncating, saturating float->int conversion.
// The divisions by 16 are exact scalings: multiplying by 1/16 gives the same
// bits as the IEEE division.
__device__ __forceinline__ void tile_rect(float cx, float cy, float ax, float ay, int tiles_x, int tiles_y,
                                          int &x0, int &y0, int &x1, int &y1) {
    const float tcx = __fmul_rn(cx, 0.0625f), tcy = __fmul_rn(cy, 0.0625f);
    const float trx = __fmul_rn(ax, 0.0625f), try_ = __fmul_rn(ay, 0.0625f);
    x0 = min(max(0, __float2int_rz(__fsub_rn(tcx, trx))), tiles_x);
    x1 = min(max(0, __float2int_rz(__fadd_rn(__fadd_rn(tcx, trx), 1.0f))), tiles_x);
    y0 = min(max(0, __float2int_rz(__fsub_rn(tcy, try_))), tiles_y);
    y1 = min(max(0, __float2int_rz(__fadd_rn(__fadd_rn(tcy, try_), 1.0f))), tiles_y);
}

// Pixel of thread tid in its 16x16 tile: each warp covers an 8x4 block (two
// warps across, four down), a squarer footprint than two 16-pixel rows, so a
// small splat misses more warps entirely.
__device__ __forceinline__ int tile_px(int tid) { return (tid & 7) | ((tid >> 2) & 8); }
__device__ __forceinline__ int tile_py(int tid) { return ((tid >> 3) & 3) | ((tid >> 4) & 12); }

// Warps of a tile that a splat can reach: bit w is set when the 8x4 block of
// warp w (tile-local x in [8(w&1), 8(w&1)+7], y in [4(w>>1), 4(w>>1)+3])
// meets the box centre +- (hx, hy), the splat's reach from the projection
// (outside it no pixel passes the rasterizers' sigma and alpha tests).
// (ox, oy) is the tile's first pixel.  Non-finite extents reach every warp,
// negative ones none; the box edges get a margin well above the rounding of
// the tile-local offsets.  A warp whose bit is clear skips the splat: every
// one of its pixels would have rejected it, so nothing changes.
__device__ __forceinline__ uint32_t warp_reach(float x, float y, float hx, float hy, float ox, float oy) {
    if (!(hx <= 3.0e38f && hy <= 3.0e38f)) return 0xFFu;
    if (hx < 0.f || hy < 0.f) return 0u;
    const float lx = x - ox, ly = y - oy;
    const float rx = hx + 0.02f + 1e-6f * (fabsf(lx) + hx + fabsf(ox));
    const float ry = hy + 0.02f + 1e-6f * (fabsf(ly) + hy + fabsf(oy));
    const float x0 = lx - rx, x1 = lx + rx, y0 = ly - ry, y1 = ly + ry;
    const uint32_t cols = (x1 >= 0.f && x0 <= 7.f ? 0x55u : 0u) | (x1 >= 8.f && x0 <= 15.f ? 0xAAu : 0u);
    const uint32_t rows = (y1 >= 0.f && y0 <= 3.f ? 0x03u : 0u) | (y1 >= 4.f && y0 <= 7.f ? 0x0Cu : 0u) |
                          (y1 >= 8.f && y0 <= 11.f ? 0x30u : 0u) | (y1 >= 12.f && y0 <= 15.f ? 0xC0u : 0u);
    return cols & rows;
}

// Tile list bound as a slot of the intersection buffer, which holds the
// global slots [lo, lo + cap) (lo = 0 unless a tile group is being rastered),
// clamped to the buffer.
__device__ __forceinline__ int clamp_off(uint32_t off, long long lo, long long cap) {
    const long long r = (long long)off - lo;
    return (int)(r < 0 ? 0 : (r < cap ? r : cap));
}

// Checked builds (-DMSPLAT_CHECKED): an index that fails its bound is
// recorded in dbg[0..2] (code, index, aux) and the access is skipped.  In the
// normal build the guard is the constant true and compiles away.
#ifdef MSPLAT_CHECKED
__device__ __forceinline__ bool ms_guard(bool ok, unsigned code, long long idx, unsigned *dbg) {
    if (!ok && dbg) {
        if (atomicCAS(dbg, 0u, code) == 0u) {
            dbg[1] = (unsigned)idx;
            dbg[2] = (unsigned)(idx >> 32);
        }
    }
    return ok;
}
#define MS_GUARD(ok, code, idx, dbg) ms_guard((ok), (code), (long long)(idx), (dbg))
#else
#define MS_GUARD(ok, code, idx, dbg) (true)
#endif
constexpr int kDbgSlot = 16;   // nan_counts[16..18]: checked-build violation record

// A fault a kernel detected and survived (a bounded wait that ran out), in
// every build: the first one is recorded in the same slots as a checked-build
// violation, which the engine's stats report (check_record).
__device__ __forceinline__ void record_fault(unsigned *dbg, unsigned code, long long idx) {
    if (dbg && atomicCAS(dbg, 0u, code) == 0u) {
        dbg[1] = (unsigned)idx;
        dbg[2] = (unsigned)(idx >> 32);
    }
}

// Splat record behind intersection slot idx.  Tile lists hold Gaussian ids;
// an id past n (the slots of a tile that overflowed the buffer) reads as a
// transparent record.  The id rides in a.w.
__device__ __forceinline__ SplatRec isect_record(const uint32_t *ids, const SplatRec *rec, uint32_t n, int idx) {
    const uint32_t g = ids[idx];
    SplatRec r;
    if (g < n) {
        r = rec[g];
        r.a.w = __int_as_float((int)g);
    } else {
        r.a = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
        r.b = make_float4(0.f, 0.f, 0.f, 0.f);
        r.c = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    return r;
}

__device__ __forceinline__ void atomic_add_f4(float4 *addr, float4 v) {
    atomicAdd(addr, v);   // sm_90+: one vector reduction in L2
}

// ---------------------------------------------------------------------------
// Views of one step.  Every stage covers all views of the step in one launch:
// record u = v * n + i is Gaussian i seen from view v (projection records,
// depths, radii and rasterizer gradients are [views, n]); the tiles of all
// views form one global tile range, view v owning [tile_base[v],
// tile_base[v+1]); the images are concatenated, view v's pixel (x, y) at
// pix_base[v] + y * width[v] + x; StepParams are one per view.  A plain step
// is a table of one view.
// ---------------------------------------------------------------------------
constexpr int kMaxViews = 16;

struct ViewTable {
    int count;                         // views (1..kMaxViews)
    int n;                             // Gaussians per view
    int tiles;                         // tiles of all views (= tile_base[count])
    long long pixels;                  // pixels of all views (= pix_base[count])
    int tile_base[kMaxViews + 1];
    int tiles_x[kMaxViews], tiles_y[kMaxViews];
    int width[kMaxViews], height[kMaxViews];
    long long pix_base[kMaxViews + 1];
};

// Geometry of one view, selected with constant indices only (the table stays
// in the kernel's parameter bank; no local copy).
struct ViewGeom {
    int tile_base, tiles_x, tiles_y, width, height;
    long long pix_base;
};

__host__ __device__ __forceinline__ ViewGeom view_geom(const ViewTable &vt, int v) {
    ViewGeom g{vt.tile_base[0], vt.tiles_x[0], vt.tiles_y[0], vt.width[0], vt.height[0], vt.pix_base[0]};
#pragma unroll
    for (int k = 1; k < kMaxViews; k++)
        if (k == v) {
            g.tile_base = vt.tile_base[k];
            g.tiles_x = vt.tiles_x[k];
            g.tiles_y = vt.tiles_y[k];
            g.width = vt.width[k];
            g.height = vt.height[k];
            g.pix_base = vt.pix_base[k];
        }
    return g;
}

// view owning global tile t / global pixel p
__host__ __device__ __forceinline__ int view_of_tile(const ViewTable &vt, int t) {
    int v = 0;
#pragma unroll
    for (int k = 1; k < kMaxViews; k++) v += (k < vt.count && t >= vt.tile_base[k]) ? 1 : 0;
    return v;
}
__host__ __device__ __forceinline__ int view_of_pixel(const ViewTable &vt, long long p) {
    int v = 0;
#pragma unroll
    for (int k = 1; k < kMaxViews; k++) v += (k < vt.count && p >= vt.pix_base[k]) ? 1 : 0;
    return v;
}

}  // namespace msplat
