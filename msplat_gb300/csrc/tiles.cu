// Tile-intersection mapping: count -> exclusive scan -> scatter -> per-tile
// sort + pack.  Follows count_intersections_kernel, prefix_sum_tiles_kernel,
// scatter_intersections_kernel and hybrid_sort_pack_kernel
// (msplat_metal.metal:2248-2627) with the same keys (depth bits << 32 | id,
// ascending) and therefore the same per-tile order.  Differences of layout:
// buckets sit at exact (not power-of-two padded) offsets, and each tile is
// sorted by one CTA with a stable LSD radix sort (8-bit digits, constant
// digits skipped) in shared memory, or in global memory for heavy tiles.
// All views of a step are mapped together: the count and scatter grids have
// one row (blockIdx.y) per view, the scan and the sorts run over the global
// tile range, and the ids in the keys are record ids v * n + i.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace msplat {

// per-tile sort classes (by key count): 0 up to kSortSmallKeys (256-thread
// CTAs, when the sort width chosen is 256; else class 0 stays empty), 1 up
// to kSortLightKeys (512-thread CTAs), 2 up to kSortHeavyKeys (1024-thread
// CTAs), 3 above (global-memory sort)
constexpr int kSortItems = 8;                      // keys per thread in the shared-memory sorts
constexpr int kSortSmallKeys = 256 * kSortItems;   // 2048
constexpr int kSortLightKeys = 512 * kSortItems;   // 4096: 512-thread CTA, two per SM
constexpr int kSortHeavyKeys = 1024 * kSortItems;  // 8192: 1024-thread CTA, one per SM
constexpr int kSortClasses = 4;

__device__ __forceinline__ bool splat_active(size_t u, const int *radii, const float *depths) {
    if (radii[u] <= 0) return false;
    const float d = depths[u];
    return finite_bits(d) && d > 0.0f;
}

template <bool kViews>
__global__ void __launch_bounds__(256) k_count(TileArgs a) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int view = kViews ? (int)blockIdx.y : 0;
    const size_t u = kViews ? (size_t)view * a.vt.n + i : (size_t)i;
    if (i >= a.vt.n || !splat_active(u, a.radii, a.depths)) return;
    const ViewGeom vg = view_geom(a.vt, view);
    const float4 ra = a.rec[u].a;
    const float2 ab = a.aabb[u];
    int x0, y0, x1, y1;
    tile_rect(ra.x, ra.y, ab.x, ab.y, vg.tiles_x, vg.tiles_y, x0, y0, x1, y1);
    for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++) {
            const int t = vg.tile_base + y * vg.tiles_x + x;
            if (MS_GUARD(t < a.num_tiles && t >= 0, 2, t, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr))
                atomicAdd(a.tile_counts + t, 1u);
        }
}

// Exclusive scan of the tile counts by one CTA of 1024 threads, in chunks of
// 4096 tiles: each thread takes four consecutive tiles of the chunk (one
// 16-byte load; a warp reads 512 contiguous bytes), the thread sums are
// scanned across the CTA, and a carry runs from chunk to chunk.  Each tile
// with intersections is filed into its sort class.
__global__ void __launch_bounds__(1024) k_scan(TileArgs a) {
    pdl_enter();
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t max_warp[32];
    __shared__ uint32_t class_n[kSortClasses];
    __shared__ uint32_t carry;
    const int T = a.num_tiles;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t small_keys = a.sort_width == 256 ? (uint32_t)kSortSmallKeys : 0u;
    if (tid < kSortClasses) class_n[tid] = 0;
    if (tid == 0) carry = 0;
    uint32_t mx = 0;
    for (int base = 0; base < T; base += 4096) {
        const int t0 = base + 4 * tid;
        uint32_t c[4] = {0u, 0u, 0u, 0u};
        if (t0 + 3 < T) {
            const uint4 q = *reinterpret_cast<const uint4 *>(a.tile_counts + t0);
            c[0] = q.x; c[1] = q.y; c[2] = q.z; c[3] = q.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) c[k] = t0 + k < T ? a.tile_counts[t0 + k] : 0u;
        }
        const uint32_t sum = c[0] + c[1] + c[2] + c[3];
        mx = max(mx, max(max(c[0], c[1]), max(c[2], c[3])));
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();   // warp totals written; carry and class counts settled
        if (wid == 0) {
            const uint32_t v = warp_tot[lane];
            uint32_t inc = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += u;
            }
            warp_tot[lane] = inc - v;
        }
        __syncthreads();
        uint32_t run = carry + warp_tot[wid] + incl - sum;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int t = t0 + k;
            if (t >= T) break;
            a.tile_offsets[t] = run;
            run += c[k];
            // sort class of the tile: shared-memory sort by a 256-, 512- or
            // 1024-thread CTA, or the global-memory sort above kSortHeavyKeys
            if (c[k] > 0) {
                const int cls = c[k] <= small_keys ? 0
                                : c[k] <= (uint32_t)kSortLightKeys ? 1
                                : c[k] <= (uint32_t)kSortHeavyKeys ? 2 : 3;
                const uint32_t pos = atomicAdd(&class_n[cls], 1u);
                a.tile_lists[(size_t)cls * T + pos] = (uint32_t)t;
            }
        }
        __syncthreads();   // every thread has read carry and warp_tot
        if (tid == 1023) carry = run;   // the last thread's run ends the chunk
    }
    const uint32_t wmax = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 0) max_warp[wid] = wmax;
    __syncthreads();
    if (tid == 0) {
        uint32_t m = 0;
        for (int k = 0; k < 32; k++) m = max(m, max_warp[k]);
        a.max_tile_count[0] = m;
        a.tile_offsets[T] = carry;
    }
    if (tid < kSortClasses) {
        a.tile_class[tid] = class_n[tid];                  // list lengths
        a.tile_class[kSortClasses + tid] = 0;              // work counters of the sort kernels
    }
}

// kGroup: a tile group of a fixed intersection budget is being built (tiles
// outside [tile_lo, tile_hi) skipped, slots from isect_lo); false: all tiles
template <bool kViews, bool kGroup>
__global__ void __launch_bounds__(256) k_scatter(TileArgs a) {
    pdl_enter();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int view = kViews ? (int)blockIdx.y : 0;
    const size_t u = kViews ? (size_t)view * a.vt.n + i : (size_t)i;
    if (i >= a.vt.n || !splat_active(u, a.radii, a.depths)) return;
    const ViewGeom vg = view_geom(a.vt, view);
    const float4 ra = a.rec[u].a;
    const float2 ab = a.aabb[u];
    int x0, y0, x1, y1;
    tile_rect(ra.x, ra.y, ab.x, ab.y, vg.tiles_x, vg.tiles_y, x0, y0, x1, y1);
    const uint64_t key = ((uint64_t)__float_as_uint(a.depths[u]) << 32) | (uint32_t)u;
    for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++) {
            const int t = vg.tile_base + y * vg.tiles_x + x;
            if (!MS_GUARD(t >= 0 && t < a.num_tiles, 3, t, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) continue;
            if (kGroup && (t < a.tile_lo || t >= a.tile_hi)) continue;   // another tile group
            const uint32_t pos = atomicAdd(a.tile_write + t, 1u);
            const uint64_t dst = (uint64_t)a.tile_offsets[t] + pos - (kGroup ? (uint64_t)a.isect_lo : 0ull);
            if (dst < (uint64_t)a.capacity) a.keys[dst] = key;   // overflow is dropped, never written
        }
}

// Block-aggregated count and scatter.  A CTA of kAggThreads covers
// kAggPerCta Gaussians of one view and keeps a shared-memory histogram over
// that view's tiles.  Count stores the CTA's histogram row to cta_bins (view
// v's rows [ctas, T_v] start at ctas * tile_base[v]); a column scan turns the
// rows into per-(CTA, tile) start offsets and the tile totals; the scatter
// CTA loads its row, adds the tile offsets, and hands out slots with
// shared-memory atomics.  No global atomics, and each tile's bucket is
// filled CTA by CTA.  Used while every view's histogram fits (kAggMaxTiles).

__device__ __forceinline__ void agg_rect(const TileArgs &a, const ViewGeom &vg, size_t u, int &x0, int &y0, int &x1,
                                         int &y1) {
    const float4 ra = a.rec[u].a;
    const float2 ab = a.aabb[u];
    tile_rect(ra.x, ra.y, ab.x, ab.y, vg.tiles_x, vg.tiles_y, x0, y0, x1, y1);
}

template <bool kViews>
__global__ void __launch_bounds__(kAggThreads) k_count_agg(TileArgs a) {
    pdl_enter();
    extern __shared__ uint32_t bins[];
    const int view = kViews ? (int)blockIdx.y : 0;
    const ViewGeom vg = view_geom(a.vt, view);
    const int T = vg.tiles_x * vg.tiles_y;
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = 0;
    __syncthreads();
    const size_t ubase = kViews ? (size_t)view * a.vt.n : 0;
    const int g0 = blockIdx.x * kAggPerCta, g1 = min(a.vt.n, g0 + kAggPerCta);
    for (int i = g0 + threadIdx.x; i < g1; i += blockDim.x) {
        if (!splat_active(ubase + i, a.radii, a.depths)) continue;
        int x0, y0, x1, y1;
        agg_rect(a, vg, ubase + i, x0, y0, x1, y1);
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) atomicAdd(&bins[y * vg.tiles_x + x], 1u);
    }
    __syncthreads();
    uint32_t *row = a.cta_bins + (size_t)gridDim.x * vg.tile_base + (size_t)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) row[t] = bins[t];
}

// Exclusive scan down each tile's column of CTA rows; the column total is the
// tile's count.  A CTA covers 32 global tiles (one per lane, so each row
// access is a 128-byte line while the lanes share a view) and splits the
// rows over its 32 warps: row sums (the rows held in registers when a warp
// has at most 16), a scan of the 32 partial sums per tile in shared memory,
// then the rows rewritten.
template <bool kViews>
__global__ void __launch_bounds__(1024) k_cta_scan(TileArgs a, int ctas) {
    pdl_enter();
    __shared__ uint32_t part[32][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int t = blockIdx.x * 32 + lane;
    const int tc = min(t, a.num_tiles - 1);
    const ViewGeom vg = view_geom(a.vt, kViews ? view_of_tile(a.vt, tc) : 0);
    const int Tv = vg.tiles_x * vg.tiles_y;
    uint32_t *col = a.cta_bins + (size_t)ctas * vg.tile_base + (tc - vg.tile_base);
    const int per = (ctas + 31) / 32;
    const int c0 = min(ctas, w * per), c1 = min(ctas, c0 + per);
    const bool in = t < a.num_tiles;
    // up to kHeld rows per warp (2^20 Gaussians per view): all loads issued
    // at once and kept in registers for the rewrite; more rows loop
    constexpr int kHeld = 32;
    const bool held_rows = per <= kHeld;   // CTA-uniform
    uint32_t held[kHeld];
    uint32_t sum = 0;
    if (held_rows) {
#pragma unroll
        for (int k = 0; k < kHeld; k++) {
            const int c = c0 + k;
            held[k] = (in && c < c1) ? col[(size_t)c * Tv] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kHeld; k++) sum += held[k];
    } else if (in) {
        for (int c = c0; c < c1; c++) sum += col[(size_t)c * Tv];
    }
    part[w][lane] = sum;
    __syncthreads();
    uint32_t run = 0, total = 0;
    for (int k = 0; k < 32; k++) {
        const uint32_t v = part[k][lane];
        if (k < w) run += v;
        total += v;
    }
    if (in) {
        if (held_rows) {
#pragma unroll
            for (int k = 0; k < kHeld; k++) {
                const int c = c0 + k;
                if (c < c1) {
                    col[(size_t)c * Tv] = run;
                    run += held[k];
                }
            }
        } else {
            for (int c = c0; c < c1; c++) {
                const uint32_t v = col[(size_t)c * Tv];
                col[(size_t)c * Tv] = run;
                run += v;
            }
        }
        if (w == 0) a.tile_counts[t] = total;
    }
}

template <bool kViews, bool kGroup>
__global__ void __launch_bounds__(kAggThreads) k_scatter_agg(TileArgs a) {
    pdl_enter();
    extern __shared__ uint32_t bins[];
    const int view = kViews ? (int)blockIdx.y : 0;
    const ViewGeom vg = view_geom(a.vt, view);
    const int T = vg.tiles_x * vg.tiles_y;
    const uint32_t *row = a.cta_bins + (size_t)gridDim.x * vg.tile_base + (size_t)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = a.tile_offsets[vg.tile_base + t] + row[t];
    __syncthreads();
    const size_t ubase = kViews ? (size_t)view * a.vt.n : 0;
    const int g0 = blockIdx.x * kAggPerCta, g1 = min(a.vt.n, g0 + kAggPerCta);
    for (int i = g0 + threadIdx.x; i < g1; i += blockDim.x) {
        const size_t u = ubase + i;
        if (!splat_active(u, a.radii, a.depths)) continue;
        int x0, y0, x1, y1;
        agg_rect(a, vg, u, x0, y0, x1, y1);
        const uint64_t key = ((uint64_t)__float_as_uint(a.depths[u]) << 32) | (uint32_t)u;
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) {
                const int lt = y * vg.tiles_x + x;
                if (kGroup && (vg.tile_base + lt < a.tile_lo || vg.tile_base + lt >= a.tile_hi)) continue;
                const uint64_t dst = (uint64_t)atomicAdd(&bins[lt], 1u) - (kGroup ? (uint64_t)a.isect_lo : 0ull);
                if (dst < (uint64_t)a.capacity) a.keys[dst] = key;   // overflow is dropped, never written
            }
    }
}


size_t tile_cta_bins_bytes(const ViewTable &vt) {
    if (max_view_tiles(vt) > kAggMaxTiles || vt.n <= 0) return 0;
    return (size_t)((vt.n + kAggPerCta - 1) / kAggPerCta) * (size_t)vt.tile_base[vt.count] * sizeof(uint32_t);
}

// ---------------------------------------------------------------------------
// Per-tile sort + pack.  Keys are (depth bits << 32 | id); the reference
// orders each tile by (depth, id) ascending.
//
// Tiles up to kSortHeavyKeys sort in shared memory: the 32-bit depth keys with
// a 16-bit local index as payload go through a stable LSD radix sort on 8-bit
// digits (bytes above the highest bit that differs within the tile are
// skipped, and so is any byte that turns out constant), then runs of equal
// depth (exact clones) are put in id order.  A 512-thread CTA takes tiles up
// to 4096 keys, a 1024-thread CTA tiles up to 8192; larger tiles sort their
// 64-bit keys in global memory in chunks.  Each class runs as a persistent
// grid that takes tiles from its list (built by k_scan) through an atomic
// work counter.  The output is the sorted Gaussian ids; the rasterizers
// gather each splat's record by id (the records of all Gaussians stay in L2
// at 1M), instead of reading a 48-byte record per intersection written here.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t digit_of(uint64_t key, int shift) { return (uint32_t)(key >> shift) & 255u; }

// A tile whose bucket does not fit the buffer is emitted transparent
// (hybrid_sort_pack_kernel's region guard, msplat_metal.metal:2523-2535): its
// slots that exist get an id no Gaussian has.  Returns true when it did so.
template <int THREADS> __device__ bool emit_if_overflow(const TileArgs &a, uint32_t start, int count) {
    if ((uint64_t)start + (uint64_t)count <= (uint64_t)a.capacity) return false;
    for (int j = threadIdx.x; j < count; j += THREADS) {
        const uint64_t d = (uint64_t)start + j;
        if (d < (uint64_t)a.capacity) a.isect_ids[d] = 0xffffffffu;
    }
    return true;
}

// next tile of class `cls` for this CTA, or -1; ends with a barrier
__device__ __forceinline__ int next_tile(const TileArgs &a, int cls, int *slot) {
    if (threadIdx.x == 0) {
        const uint32_t k = atomicAdd(a.tile_class + kSortClasses + cls, 1u);
        *slot = k < a.tile_class[cls] ? (int)a.tile_lists[(size_t)cls * a.num_tiles + k] : -1;
    }
    __syncthreads();
    return *slot;
}

// ---- shared-memory pair sort (tiles up to THREADS * kSortItems keys) ----

template <int THREADS> struct PairSmem {
    static constexpr int kWarps = THREADS / 32;
    static constexpr int kCap = THREADS * kSortItems;
    uint32_t key[2][kCap];        // depth bits
    uint32_t id[kCap];            // Gaussian id of local index i
    uint16_t idx[2][kCap];        // local index riding with the key
    uint16_t wcnt[kWarps][256];   // per-warp digit counts
    uint16_t woff[kWarps][256];   // per-warp offsets inside a digit
    uint32_t base[256];
    uint32_t dsum[8];
    uint32_t dlo, dhi;
    int skip_shift;
    int slot;
};

// One LSD pass over n keys, buffer b -> 1 - b.  The keys are spread over the
// warps in contiguous segments of 32 * ipt (ipt = ceil(n / THREADS)), so small
// tiles keep few warps busy for few rounds.  Expects wcnt == 0 for the warps
// holding keys and leaves it so.  Returns false (nothing moved) when one digit
// holds every key.
template <int THREADS>
__device__ bool pair_pass(PairSmem<THREADS> &sm, int b, int n, int shift, unsigned *dbg) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int ipt = (n + THREADS - 1) / THREADS;   // 1..kSortItems
    const int seg = 32 * ipt;
    const int nw = (n + seg - 1) / seg;
    uint32_t kv[kSortItems], rank[kSortItems];
    uint16_t iv[kSortItems];
    const uint32_t lt = (1u << lane) - 1u;
    if (wid < nw) {
#pragma unroll
        for (int j = 0; j < kSortItems; j++) {
            if (j >= ipt) continue;
            const int i = wid * seg + j * 32 + lane;
            const bool valid = i < n;
            kv[j] = valid ? sm.key[b][i] : 0u;
            iv[j] = valid ? sm.idx[b][i] : (uint16_t)0;
            const uint32_t d = valid ? ((kv[j] >> shift) & 255u) : 256u;
            // lanes holding the same digit: eight ballots, one per digit bit
            uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
            for (int bit = 0; bit < 8; bit++) {
                const uint32_t m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
                peers &= ((d >> bit) & 1u) ? m : ~m;
            }
            uint32_t old = 0;
            if (valid) old = sm.wcnt[wid][d];
            __syncwarp();
            rank[j] = valid ? old + __popc(peers & lt) : 0xffffffffu;
            if (valid && (peers & lt) == 0) sm.wcnt[wid][d] = (uint16_t)(old + __popc(peers));
            __syncwarp();
        }
    }
    __syncthreads();
    uint32_t total = 0, incl = 0;
    if (tid < 256) {
        for (int w = 0; w < nw; w++) {
            const uint32_t c = sm.wcnt[w][tid];
            sm.woff[w][tid] = (uint16_t)total;
            sm.wcnt[w][tid] = 0;
            total += c;
        }
        incl = total;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) sm.dsum[wid] = incl;
        if (total == (uint32_t)n) sm.skip_shift = shift;
    }
    __syncthreads();
    if (sm.skip_shift == shift) return false;   // uniform
    if (tid < 256) {
        uint32_t add = 0;
        for (int w = 0; w < wid; w++) add += sm.dsum[w];
        sm.base[tid] = add + incl - total;
    }
    __syncthreads();
    if (wid < nw) {
#pragma unroll
        for (int j = 0; j < kSortItems; j++) {
            if (j >= ipt || rank[j] == 0xffffffffu) continue;
            const uint32_t d = (kv[j] >> shift) & 255u;
            const uint32_t pos = sm.base[d] + sm.woff[wid][d] + rank[j];
            if (MS_GUARD(pos < (uint32_t)n, 4, pos, dbg)) {
                sm.key[1 - b][pos] = kv[j];
                sm.idx[1 - b][pos] = iv[j];
            }
        }
    }
    __syncthreads();
    return true;
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) k_sort_pack_smem(TileArgs a, int cls) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PairSmem<THREADS> &sm = *reinterpret_cast<PairSmem<THREADS> *>(smem_raw);
    const int tid = threadIdx.x;
    unsigned *dbg = a.nan_counts ? a.nan_counts + kDbgSlot : nullptr;
    // shared memory starts stale: the passes expect zero digit counts
    for (int i = tid; i < PairSmem<THREADS>::kWarps * 256; i += THREADS) (&sm.wcnt[0][0])[i] = 0;
    for (;;) {
        const int t = next_tile(a, cls, &sm.slot);   // barrier inside
        if (t < 0) break;
        if (t < a.tile_lo || t >= a.tile_hi) {   // another tile group (t is CTA-uniform)
            __syncthreads();                      // every thread has read the slot before it is reused
            continue;
        }
        const int count = (int)a.tile_counts[t];
        const uint32_t start = a.tile_offsets[t] - (uint32_t)a.isect_lo;   // offsets and isect_lo are below 2^32
        if (!MS_GUARD(count <= PairSmem<THREADS>::kCap, 5, count, dbg) || emit_if_overflow<THREADS>(a, start, count)) {
            __syncthreads();
            continue;
        }
        if (tid == 0) { sm.dlo = 0xffffffffu; sm.dhi = 0u; sm.skip_shift = -1; }
        __syncthreads();
        uint32_t lo = 0xffffffffu, hi = 0u;
        for (int j = tid; j < count; j += THREADS) {
            const uint64_t k = a.keys[start + j];
            const uint32_t d = (uint32_t)(k >> 32);
            sm.key[0][j] = d;
            sm.idx[0][j] = (uint16_t)j;
            sm.id[j] = (uint32_t)k;
            lo = min(lo, d);
            hi = max(hi, d);
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if ((tid & 31) == 0) { atomicMin(&sm.dlo, lo); atomicMax(&sm.dhi, hi); }
        __syncthreads();
        const uint32_t diff = sm.dlo ^ sm.dhi;
        int b = 0;
        for (int shift = 0; shift < 32; shift += 8) {
            if ((diff >> shift) == 0u) break;   // this byte and all above are equal in every key
            if (pair_pass<THREADS>(sm, b, count, shift, dbg)) b ^= 1;
        }
        // equal depths (exact clones): order the run by id
        for (int j = tid; j < count; j += THREADS) {
            const uint32_t dj = sm.key[b][j];
            if (j > 0 && sm.key[b][j - 1] == dj) continue;
            if (j + 1 >= count || sm.key[b][j + 1] != dj) continue;
            int e = j + 1;
            while (e < count && sm.key[b][e] == dj) e++;
            for (int u = j + 1; u < e; u++) {
                const uint16_t v = sm.idx[b][u];
                const uint32_t vid = sm.id[v];
                int w = u - 1;
                while (w >= j && sm.id[sm.idx[b][w]] > vid) { sm.idx[b][w + 1] = sm.idx[b][w]; w--; }
                sm.idx[b][w + 1] = v;
            }
        }
        __syncthreads();
        for (int j = tid; j < count; j += THREADS) a.isect_ids[start + j] = sm.id[sm.idx[b][j]];
        __syncthreads();
    }
}

template <int THREADS> constexpr size_t pair_smem_bytes() { return sizeof(PairSmem<THREADS>); }

// ---- global-memory sort for tiles above kSortHeavyKeys ----

constexpr int kGlobThreads = 512;
constexpr int kGlobWarps = kGlobThreads / 32;

struct GlobSmem {
    uint32_t hist[256];
    uint32_t base[256];
    uint16_t wcnt[kGlobWarps][256];
    uint32_t woff[kGlobWarps][256];
    uint32_t dlo, dhi;
    int skip;
    int slot;
};

// Exclusive scan of sm.hist into sm.base by the first 256 threads; sets
// sm.skip when one digit holds all n keys.  Ends with a barrier.
__device__ void digit_scan(GlobSmem &sm, int n) {
    const int tid = threadIdx.x;
    if (tid < 256) {
        const uint32_t h = sm.hist[tid];
        const int lane = tid & 31, w = tid >> 5;
        uint32_t inc = h;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        sm.base[tid] = inc - h;   // warp-local exclusive
        if (lane == 31) sm.woff[0][w] = inc;
        if (h == (uint32_t)n) sm.skip = 1;
    }
    __syncthreads();
    if (tid < 256) {
        uint32_t add = 0;
        for (int w = 0; w < (tid >> 5); w++) add += sm.woff[0][w];
        sm.base[tid] += add;
    }
    __syncthreads();
}

// One stable pass on n keys in chunks of kGlobThreads: src -> dst.
__device__ bool radix_pass_chunked(const uint64_t *src, uint64_t *dst, int n, int shift, GlobSmem &sm, unsigned *dbg) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int d = tid; d < 256; d += kGlobThreads) sm.hist[d] = 0;
    if (tid == 0) sm.skip = 0;
    __syncthreads();
    for (int i = tid; i < n; i += kGlobThreads) atomicAdd(&sm.hist[digit_of(src[i], shift)], 1u);
    __syncthreads();
    digit_scan(sm, n);
    if (sm.skip) return false;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int c0 = 0; c0 < n; c0 += kGlobThreads) {
        const int i = c0 + tid;
        const bool valid = i < n;
        const uint64_t key = valid ? src[i] : 0ull;
        const uint32_t d = valid ? digit_of(key, shift) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) sm.wcnt[wid][d] = (uint16_t)__popc(peers);
        __syncthreads();
        for (int dd = tid; dd < 256; dd += kGlobThreads) {
            uint32_t acc = sm.base[dd];
#pragma unroll 4
            for (int w = 0; w < kGlobWarps; w++) {
                const uint32_t cnt = sm.wcnt[w][dd];
                sm.woff[w][dd] = acc;
                sm.wcnt[w][dd] = 0;
                acc += cnt;
            }
            sm.base[dd] = acc;
        }
        __syncthreads();
        if (valid && MS_GUARD(sm.woff[wid][d] + rank < (uint32_t)n, 4, sm.woff[wid][d] + rank, dbg))
            dst[sm.woff[wid][d] + rank] = key;
        __syncthreads();
    }
    return true;
}

// Keys sorted by depth: order each run of equal depth by id.
__device__ void order_ties(uint64_t *a, int n) {
    for (int j = threadIdx.x; j < n; j += kGlobThreads) {
        const uint32_t dj = (uint32_t)(a[j] >> 32);
        if (j > 0 && (uint32_t)(a[j - 1] >> 32) == dj) continue;          // not a run start
        if (j + 1 >= n || (uint32_t)(a[j + 1] >> 32) != dj) continue;      // run of one
        int e = j + 1;
        while (e < n && (uint32_t)(a[e] >> 32) == dj) e++;
        for (int u = j + 1; u < e; u++) {                                  // insertion sort by id
            const uint64_t v = a[u];
            int w = u - 1;
            while (w >= j && (uint32_t)a[w] > (uint32_t)v) { a[w + 1] = a[w]; w--; }
            a[w + 1] = v;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kGlobThreads) k_sort_pack_global(TileArgs a, int cls) {
    pdl_enter();
    __shared__ GlobSmem sm;
    const int tid = threadIdx.x;
    unsigned *dbg = a.nan_counts ? a.nan_counts + kDbgSlot : nullptr;
    for (int i = tid; i < kGlobWarps * 256; i += kGlobThreads) (&sm.wcnt[0][0])[i] = 0;
    for (;;) {
        const int t = next_tile(a, cls, &sm.slot);
        if (t < 0) break;
        if (t < a.tile_lo || t >= a.tile_hi) {   // another tile group (t is CTA-uniform)
            __syncthreads();                      // every thread has read the slot before it is reused
            continue;
        }
        const int count = (int)a.tile_counts[t];
        const uint32_t start = a.tile_offsets[t] - (uint32_t)a.isect_lo;   // offsets and isect_lo are below 2^32
        if (emit_if_overflow<kGlobThreads>(a, start, count)) {
            __syncthreads();
            continue;
        }
        if (tid == 0) { sm.dlo = 0xffffffffu; sm.dhi = 0u; }
        __syncthreads();
        uint32_t lo = 0xffffffffu, hi = 0u;
        for (int j = tid; j < count; j += kGlobThreads) {
            const uint32_t d = (uint32_t)(a.keys[start + j] >> 32);
            lo = min(lo, d);
            hi = max(hi, d);
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if ((tid & 31) == 0) { atomicMin(&sm.dlo, lo); atomicMax(&sm.dhi, hi); }
        __syncthreads();
        const uint32_t diff = sm.dlo ^ sm.dhi;
        uint64_t *src = a.keys + start, *alt = a.keys_alt + start;
        for (int shift = 32; shift < 64; shift += 8) {
            if ((diff >> (shift - 32)) == 0u) break;
            if (radix_pass_chunked(src, alt, count, shift, sm, dbg)) { uint64_t *tmp = src; src = alt; alt = tmp; }
            __syncthreads();
        }
        order_ties(src, count);
        for (int j = tid; j < count; j += kGlobThreads) a.isect_ids[start + j] = (uint32_t)src[j];
        __syncthreads();
    }
}

size_t sort_pack_smem_bytes() { return pair_smem_bytes<1024>(); }

// The kernels' shared-memory limits, set once on each device (function
// attributes belong to the device the call is made on).  A failure is left
// in cudaGetLastError for the caller's launch check.
static void tile_attrs() {
    static bool done[64] = {false};
    static std::mutex mu;
    once_per_device(mu, done, []() {
        cudaError_t e = cudaSuccess;
        auto set = [&](const void *k, int bytes) {
            const cudaError_t r = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e == cudaSuccess) e = r;
        };
        set((const void *)k_sort_pack_smem<256>, (int)pair_smem_bytes<256>());
        set((const void *)k_sort_pack_smem<512>, (int)pair_smem_bytes<512>());
        set((const void *)k_sort_pack_smem<1024>, (int)pair_smem_bytes<1024>());
        set((const void *)k_count_agg<false>, kAggMaxTiles * 4);
        set((const void *)k_count_agg<true>, kAggMaxTiles * 4);
        set((const void *)k_scatter_agg<false, false>, kAggMaxTiles * 4);
        set((const void *)k_scatter_agg<true, false>, kAggMaxTiles * 4);
        set((const void *)k_scatter_agg<false, true>, kAggMaxTiles * 4);
        set((const void *)k_scatter_agg<true, true>, kAggMaxTiles * 4);
        return e;
    });
}

static bool presorted_path(const TileArgs &a) {
    return a.presorted && a.vt.n > 0 && max_view_tiles(a.vt) <= kAggMaxTiles && a.cta_bins != nullptr;
}

// the column scan of the per-CTA histograms and the tile scan
int launch_tile_scans(const TileArgs &a, cudaStream_t s) {
    const int agg_blocks = (a.vt.n + kAggPerCta - 1) / kAggPerCta;
    if (a.vt.count > 1) launch_pdl(k_cta_scan<true>, (a.num_tiles + 31) / 32, 1024, 0, s, a, agg_blocks);
    else launch_pdl(k_cta_scan<false>, (a.num_tiles + 31) / 32, 1024, 0, s, a, agg_blocks);
    debug_sync(s, "cta_scan");
    launch_pdl(k_scan, 1, 1024, 0, s, a);
    debug_sync(s, "scan");
    return 2;
}

int launch_tile_count(const TileArgs &a, cudaStream_t s) {
    tile_attrs();
    if (presorted_path(a)) return launch_presorted_count(a, s) + launch_tile_scans(a, s);
    int launches = 0;
    const int n = a.vt.n, views = a.vt.count, maxT = max_view_tiles(a.vt);
    const bool agg = maxT <= kAggMaxTiles && a.cta_bins != nullptr;
    const int agg_blocks = (n + kAggPerCta - 1) / kAggPerCta;
    const size_t agg_smem = (size_t)maxT * sizeof(uint32_t);
    const bool mv = views > 1;
    if (n > 0 && agg) {
        if (mv) launch_pdl(k_count_agg<true>, dim3(agg_blocks, views), kAggThreads, agg_smem, s, a);
        else launch_pdl(k_count_agg<false>, agg_blocks, kAggThreads, agg_smem, s, a);
        debug_sync(s, "count");
        if (mv) launch_pdl(k_cta_scan<true>, (a.num_tiles + 31) / 32, 1024, 0, s, a, agg_blocks);
        else launch_pdl(k_cta_scan<false>, (a.num_tiles + 31) / 32, 1024, 0, s, a, agg_blocks);
        debug_sync(s, "cta_scan");
        launches += 2;
    } else if (n > 0) {
        if (mv) launch_pdl(k_count<true>, dim3((n + 255) / 256, views), 256, 0, s, a);
        else launch_pdl(k_count<false>, (n + 255) / 256, 256, 0, s, a);
        debug_sync(s, "count");
        launches += 1;
    }
    launch_pdl(k_scan, 1, 1024, 0, s, a);
    debug_sync(s, "scan");
    launches += 1;
    return launches;
}

int launch_tile_build(const TileArgs &a, int num_sms, cudaStream_t s) {
    tile_attrs();
    if (presorted_path(a)) return launch_presorted_build(a, s);
    int launches = 0;
    const int n = a.vt.n, views = a.vt.count, maxT = max_view_tiles(a.vt);
    const bool agg = maxT <= kAggMaxTiles && a.cta_bins != nullptr;
    const int agg_blocks = (n + kAggPerCta - 1) / kAggPerCta;
    const size_t agg_smem = (size_t)maxT * sizeof(uint32_t);
    const bool mv = views > 1;
    const bool grp = a.tile_lo > 0 || a.tile_hi < a.num_tiles || a.isect_lo > 0;
    if (n > 0) {
        const dim3 ga(agg_blocks, views), gs((n + 255) / 256, views);
        if (agg) {
            if (grp) {
                if (mv) launch_pdl(k_scatter_agg<true, true>, ga, kAggThreads, agg_smem, s, a);
                else launch_pdl(k_scatter_agg<false, true>, ga, kAggThreads, agg_smem, s, a);
            } else {
                if (mv) launch_pdl(k_scatter_agg<true, false>, ga, kAggThreads, agg_smem, s, a);
                else launch_pdl(k_scatter_agg<false, false>, ga, kAggThreads, agg_smem, s, a);
            }
        } else {
            if (grp) {
                if (mv) launch_pdl(k_scatter<true, true>, gs, 256, 0, s, a);
                else launch_pdl(k_scatter<false, true>, gs, 256, 0, s, a);
            } else {
                if (mv) launch_pdl(k_scatter<true, false>, gs, 256, 0, s, a);
                else launch_pdl(k_scatter<false, false>, gs, 256, 0, s, a);
            }
        }
        debug_sync(s, "scatter");
        launches += 1;
    }
    // persistent sort grids, one per class; idle classes exit at once
    if (a.sort_width == 256) {
        launch_pdl(k_sort_pack_smem<256>, 4 * num_sms, 256, pair_smem_bytes<256>(), s, a, 0);
        debug_sync(s, "sort_pack_256");
        launches += 1;
    }
    launch_pdl(k_sort_pack_smem<512>, 2 * num_sms, 512, pair_smem_bytes<512>(), s, a, 1);
    debug_sync(s, "sort_pack_512");
    launch_pdl(k_sort_pack_smem<1024>, num_sms, 1024, pair_smem_bytes<1024>(), s, a, 2);
    debug_sync(s, "sort_pack_1024");
    launch_pdl(k_sort_pack_global, num_sms, kGlobThreads, 0, s, a, 3);
    debug_sync(s, "sort_pack_global");
    return launches + 3;
}

int launch_tiles(const TileArgs &a, int num_sms, cudaStream_t s) {
    return launch_tile_count(a, s) + launch_tile_build(a, num_sms, s);
}

}  // namespace msplat
