// Tile-intersection mapping: count -> exclusive scan -> scatter -> per-tile
// sort + pack.  Follows count_intersections_kernel, prefix_sum_tiles_kernel,
// scatter_intersections_kernel and hybrid_sort_pack_kernel
// (msplat_metal.metal:2248-2627) with the same keys (depth bits << 32 | id,
// ascending) and therefore the same per-tile order.  Differences of layout:
// buckets sit at exact (not power-of-two padded) offsets, and each tile is
// sorted by one CTA with a stable LSD radix sort (8-bit digits, constant
// digits skipped) in shared memory, or in global memory for heavy tiles.
#include "common.cuh"
#include "kernels.h"

namespace msplat {

__device__ __forceinline__ bool splat_active(int i, const int *radii, const float *depths) {
    if (radii[i] <= 0) return false;
    const float d = depths[i];
    return finite_bits(d) && d > 0.0f;
}

__global__ void __launch_bounds__(256) k_count(TileArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !splat_active(i, a.radii, a.depths)) return;
    const float4 ra = a.rec[i].a;
    const float2 ab = a.aabb[i];
    int x0, y0, x1, y1;
    tile_rect(ra.x, ra.y, ab.x, ab.y, a.tiles_x, a.tiles_y, x0, y0, x1, y1);
    for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++)
            if (MS_GUARD(y * a.tiles_x + x < a.num_tiles && y * a.tiles_x + x >= 0, 2, y * a.tiles_x + x,
                         a.nan_counts ? a.nan_counts + kDbgSlot : nullptr))
                atomicAdd(a.tile_counts + y * a.tiles_x + x, 1u);
}

// Exclusive scan of the tile counts by one CTA of 1024 threads: each thread
// scans a contiguous run, the run totals are scanned across the CTA.
__global__ void __launch_bounds__(1024) k_scan(TileArgs a) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t max_warp[32];
    const int T = a.num_tiles;
    const int per = (T + 1023) / 1024;
    const int lo = min(T, (int)threadIdx.x * per), hi = min(T, lo + per);
    uint32_t sum = 0, mx = 0;
    for (int t = lo; t < hi; t++) { const uint32_t c = a.tile_counts[t]; sum += c; mx = max(mx, c); }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    const uint32_t wmax = __reduce_max_sync(0xffffffffu, mx);
    if (lane == 31) warp_tot[wid] = incl;
    if (lane == 0) max_warp[wid] = wmax;
    __syncthreads();
    if (wid == 0) {
        uint32_t v = warp_tot[lane], inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        warp_tot[lane] = inc - v;
        const uint32_t m = __reduce_max_sync(0xffffffffu, max_warp[lane]);
        if (lane == 0) max_warp[0] = m;
    }
    __syncthreads();
    uint32_t run = warp_tot[wid] + incl - sum;
    for (int t = lo; t < hi; t++) {
        a.tile_offsets[t] = run;
        run += a.tile_counts[t];
    }
    if (threadIdx.x == 1023) a.tile_offsets[T] = run;
    if (threadIdx.x == 0) a.max_tile_count[0] = max_warp[0];
}

__global__ void __launch_bounds__(256) k_scatter(TileArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !splat_active(i, a.radii, a.depths)) return;
    const float4 ra = a.rec[i].a;
    const float2 ab = a.aabb[i];
    int x0, y0, x1, y1;
    tile_rect(ra.x, ra.y, ab.x, ab.y, a.tiles_x, a.tiles_y, x0, y0, x1, y1);
    const uint64_t key = ((uint64_t)__float_as_uint(a.depths[i]) << 32) | (uint32_t)i;
    for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++) {
            const int t = y * a.tiles_x + x;
            if (!MS_GUARD(t >= 0 && t < a.num_tiles, 3, t, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) continue;
            const uint32_t pos = atomicAdd(a.tile_write + t, 1u);
            const uint64_t dst = (uint64_t)a.tile_offsets[t] + pos;
            if (dst < (uint64_t)a.capacity) a.keys[dst] = key;   // overflow is dropped, never written
        }
}

// Block-aggregated count and scatter: a CTA covers kAggPerCta Gaussians and
// keeps a shared-memory histogram over all tiles, so the global atomics fall
// from one per intersection to one per (CTA, touched tile).  Scatter reserves
// each tile's slot range with that one atomic and hands out slots inside it
// with shared-memory atomics.  Used while the histogram fits (kAggMaxTiles).
constexpr int kAggPerCta = 4096;
constexpr int kAggMaxTiles = 12288;

__global__ void __launch_bounds__(256) k_count_agg(TileArgs a) {
    extern __shared__ uint32_t bins[];
    const int T = a.num_tiles;
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = 0;
    __syncthreads();
    const int g0 = blockIdx.x * kAggPerCta, g1 = min(a.n, g0 + kAggPerCta);
    for (int i = g0 + threadIdx.x; i < g1; i += blockDim.x) {
        if (!splat_active(i, a.radii, a.depths)) continue;
        const float4 ra = a.rec[i].a;
        const float2 ab = a.aabb[i];
        int x0, y0, x1, y1;
        tile_rect(ra.x, ra.y, ab.x, ab.y, a.tiles_x, a.tiles_y, x0, y0, x1, y1);
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) atomicAdd(&bins[y * a.tiles_x + x], 1u);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < T; t += blockDim.x)
        if (bins[t]) atomicAdd(a.tile_counts + t, bins[t]);
}

__global__ void __launch_bounds__(256) k_scatter_agg(TileArgs a) {
    extern __shared__ uint32_t bins[];
    const int T = a.num_tiles;
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = 0;
    __syncthreads();
    const int g0 = blockIdx.x * kAggPerCta, g1 = min(a.n, g0 + kAggPerCta);
    for (int i = g0 + threadIdx.x; i < g1; i += blockDim.x) {
        if (!splat_active(i, a.radii, a.depths)) continue;
        const float4 ra = a.rec[i].a;
        const float2 ab = a.aabb[i];
        int x0, y0, x1, y1;
        tile_rect(ra.x, ra.y, ab.x, ab.y, a.tiles_x, a.tiles_y, x0, y0, x1, y1);
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) atomicAdd(&bins[y * a.tiles_x + x], 1u);
    }
    __syncthreads();
    // reserve each touched tile's slots; bins[t] becomes the next free slot
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
        const uint32_t c = bins[t];
        if (c) bins[t] = a.tile_offsets[t] + atomicAdd(a.tile_write + t, c);
    }
    __syncthreads();
    for (int i = g0 + threadIdx.x; i < g1; i += blockDim.x) {
        if (!splat_active(i, a.radii, a.depths)) continue;
        const float4 ra = a.rec[i].a;
        const float2 ab = a.aabb[i];
        int x0, y0, x1, y1;
        tile_rect(ra.x, ra.y, ab.x, ab.y, a.tiles_x, a.tiles_y, x0, y0, x1, y1);
        const uint64_t key = ((uint64_t)__float_as_uint(a.depths[i]) << 32) | (uint32_t)i;
        for (int y = y0; y < y1; y++)
            for (int x = x0; x < x1; x++) {
                const uint64_t dst = atomicAdd(&bins[y * a.tiles_x + x], 1u);
                if (dst < (uint64_t)a.capacity) a.keys[dst] = key;   // overflow is dropped, never written
            }
    }
}

// ---------------------------------------------------------------------------
// Per-tile sort by one CTA.  Keys are (depth bits << 32 | id).  A stable LSD
// radix sort on the four depth bytes (a byte equal in every key is skipped)
// orders the tile by depth; runs of equal depth (exact clones) are then put
// in id order, which gives the reference's (depth, id) order.
// Tiles up to kSortSmemKeys keys sort in shared memory in one chunk, 8 keys
// per thread; larger tiles run chunked passes in global memory.
// ---------------------------------------------------------------------------
constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kItems = 8;
constexpr int kSortSmemKeys = kSortThreads * kItems;   // 4096

struct SortSmem {
    uint32_t hist[256];
    uint32_t base[256];
    uint16_t wcnt[kSortWarps][256];
    uint32_t woff[kSortWarps][256];
    int skip;
};

__device__ __forceinline__ uint32_t digit_of(uint64_t key, int shift) { return (uint32_t)(key >> shift) & 255u; }

// Exclusive scan of sm.hist into sm.base by the first 256 threads; sets
// sm.skip when one digit holds all n keys.  Ends with a barrier.
__device__ void digit_scan(SortSmem &sm, int n) {
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

// One pass on n <= kSortSmemKeys keys, all in one chunk: src -> dst.
// Returns false (and writes nothing) when the digit is constant.
__device__ bool radix_pass_1chunk(const uint64_t *src, uint64_t *dst, int n, int shift, SortSmem &sm, unsigned *dbg) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int k = tid; k < kSortWarps * 256; k += kSortThreads) (&sm.wcnt[0][0])[k] = 0;
    if (tid == 0) sm.skip = 0;
    __syncthreads();
    uint64_t key[kItems];
    uint32_t dig[kItems], rank[kItems];
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        const int idx = wid * (32 * kItems) + j * 32 + lane;
        const bool valid = idx < n;
        key[j] = valid ? src[idx] : 0ull;
        dig[j] = valid ? digit_of(key[j], shift) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, dig[j]);
        uint32_t old = 0;
        if (valid) old = sm.wcnt[wid][dig[j]];
        __syncwarp();
        rank[j] = old + __popc(peers & lt);
        if (valid && (peers & lt) == 0) sm.wcnt[wid][dig[j]] = (uint16_t)(old + __popc(peers));
        __syncwarp();
    }
    __syncthreads();
    // per digit: offsets of each warp, totals -> hist
    if (tid < 256) {
        uint32_t run = 0;
#pragma unroll 4
        for (int w = 0; w < kSortWarps; w++) {
            sm.woff[w][tid] = run;
            run += sm.wcnt[w][tid];
        }
        sm.hist[tid] = run;
    }
    __syncthreads();
    // exclusive scan of the totals (hist -> base); woff[0] is reused as warp
    // sums only after every thread has read its offsets, so keep a copy
    uint32_t my_off[kItems];
#pragma unroll
    for (int j = 0; j < kItems; j++) my_off[j] = (dig[j] < 256u) ? sm.woff[wid][dig[j]] : 0u;
    __syncthreads();
    digit_scan(sm, n);
    if (sm.skip) return false;
#pragma unroll
    for (int j = 0; j < kItems; j++) {
        if (dig[j] >= 256u) continue;
        const uint32_t pos = sm.base[dig[j]] + my_off[j] + rank[j];
        if (MS_GUARD(pos < (uint32_t)n, 4, pos, dbg)) dst[pos] = key[j];
    }
    __syncthreads();
    return true;
}

// One pass on any n in chunks of kSortThreads keys (global-memory tiles).
__device__ bool radix_pass_chunked(const uint64_t *src, uint64_t *dst, int n, int shift, SortSmem &sm, unsigned *dbg) {
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int d = tid; d < 256; d += kSortThreads) sm.hist[d] = 0;
    if (tid == 0) sm.skip = 0;
    __syncthreads();
    for (int i = tid; i < n; i += kSortThreads) atomicAdd(&sm.hist[digit_of(src[i], shift)], 1u);
    __syncthreads();
    digit_scan(sm, n);
    if (sm.skip) return false;
    const uint32_t lt_mask = (1u << lane) - 1u;
    for (int c0 = 0; c0 < n; c0 += kSortThreads) {
        const int i = c0 + tid;
        const bool valid = i < n;
        const uint64_t key = valid ? src[i] : 0ull;
        const uint32_t d = valid ? digit_of(key, shift) : 256u;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const uint32_t rank = __popc(peers & lt_mask);
        if (valid && rank == 0) sm.wcnt[wid][d] = (uint16_t)__popc(peers);
        __syncthreads();
        for (int dd = tid; dd < 256; dd += kSortThreads) {
            uint32_t acc = sm.base[dd];
#pragma unroll 4
            for (int w = 0; w < kSortWarps; w++) {
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
    for (int j = threadIdx.x; j < n; j += kSortThreads) {
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

__global__ void __launch_bounds__(kSortThreads) k_sort_pack(TileArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SortSmem &sm = *reinterpret_cast<SortSmem *>(smem_raw);
    uint64_t *sk0 = reinterpret_cast<uint64_t *>(smem_raw + ((sizeof(SortSmem) + 15) & ~size_t(15)));
    uint64_t *sk1 = sk0 + kSortSmemKeys;
    const int t = blockIdx.x;
    const int count = (int)a.tile_counts[t];
    if (count == 0) return;
    const uint32_t start = a.tile_offsets[t];
    const int tid = threadIdx.x;
    unsigned *dbg = a.nan_counts ? a.nan_counts + kDbgSlot : nullptr;
    // a tile whose bucket does not fit the buffer is emitted transparent
    // (hybrid_sort_pack_kernel's region guard, msplat_metal.metal:2523-2535)
    if ((uint64_t)start + (uint64_t)count > (uint64_t)a.capacity) {
        for (int j = tid; j < count; j += kSortThreads) {
            const uint64_t d = (uint64_t)start + j;
            if (d < (uint64_t)a.capacity) {
                SplatRec z;
                z.a = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
                z.b = make_float4(0.f, 0.f, 0.f, 0.f);
                z.c = make_float4(0.f, 0.f, 0.f, 0.f);
                a.packed[d] = z;
            }
        }
        return;
    }
    // shared memory starts with stale contents: the chunked pass expects its
    // per-warp digit counts at zero (each chunk clears what it used)
    for (int i = tid; i < kSortWarps * 256; i += kSortThreads) (&sm.wcnt[0][0])[i] = 0;
    uint64_t *src, *alt;
    const bool in_smem = count <= kSortSmemKeys;
    if (in_smem) {
        for (int j = tid; j < count; j += kSortThreads) sk0[j] = a.keys[start + j];
        src = sk0; alt = sk1;
    } else {
        src = a.keys + start; alt = a.keys_alt + start;
    }
    __syncthreads();
    for (int shift = 32; shift < 64; shift += 8) {
        const bool moved = in_smem ? radix_pass_1chunk(src, alt, count, shift, sm, dbg)
                                   : radix_pass_chunked(src, alt, count, shift, sm, dbg);
        if (moved) { uint64_t *tmp = src; src = alt; alt = tmp; }
        __syncthreads();
    }
    order_ties(src, count);
    // pack: gather the splat records in sorted order
    for (int j = tid; j < count; j += kSortThreads) {
        const uint64_t key = src[j];
        const uint32_t g = (uint32_t)key;
        SplatRec r;
        if (g >= (uint32_t)a.n) {
            r.a = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
            r.b = make_float4(0.f, 0.f, 0.f, 0.f);
            r.c = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            r = a.rec[g];
            const bool ok = finite_bits(r.a.x) && finite_bits(r.a.y) && finite_bits(r.a.z) && finite_bits(r.b.x) &&
                            finite_bits(r.b.y) && finite_bits(r.b.z) && finite_bits(r.c.x) && finite_bits(r.c.y) &&
                            finite_bits(r.c.z);
            if (!ok) {
                if (a.nan_counts) {
                    atomicAdd(a.nan_counts + kNanPack, 1u);
                    if (!finite_bits(r.a.z)) atomicAdd(a.nan_counts + kNanPackOpacity, 1u);
                }
                r.a = make_float4(0.f, 0.f, 0.f, 0.f);
                r.b = make_float4(0.f, 0.f, 0.f, 0.f);
                r.c = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            r.a.w = __int_as_float((int)g);
        }
        a.packed[start + j] = r;
    }
}

size_t sort_pack_smem_bytes() {
    return ((sizeof(SortSmem) + 15) & ~size_t(15)) + 2 * kSortSmemKeys * sizeof(uint64_t);
}

void launch_tiles(const TileArgs &a, cudaStream_t s) {
    static bool attr_set = false;
    const size_t smem = sort_pack_smem_bytes();
    if (!attr_set) {
        cudaFuncSetAttribute(k_sort_pack, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_count_agg, cudaFuncAttributeMaxDynamicSharedMemorySize, kAggMaxTiles * 4);
        cudaFuncSetAttribute(k_scatter_agg, cudaFuncAttributeMaxDynamicSharedMemorySize, kAggMaxTiles * 4);
        attr_set = true;
    }
    const bool agg = a.num_tiles <= kAggMaxTiles;
    const int agg_blocks = (a.n + kAggPerCta - 1) / kAggPerCta;
    const size_t agg_smem = (size_t)a.num_tiles * sizeof(uint32_t);
    if (a.n > 0) {
        if (agg) k_count_agg<<<agg_blocks, 256, agg_smem, s>>>(a);
        else k_count<<<(a.n + 255) / 256, 256, 0, s>>>(a);
    }
    debug_sync(s, "count");
    k_scan<<<1, 1024, 0, s>>>(a);
    debug_sync(s, "scan");
    if (a.n > 0) {
        if (agg) k_scatter_agg<<<agg_blocks, 256, agg_smem, s>>>(a);
        else k_scatter<<<(a.n + 255) / 256, 256, 0, s>>>(a);
    }
    debug_sync(s, "scatter");
    k_sort_pack<<<a.num_tiles, kSortThreads, smem, s>>>(a);
    debug_sync(s, "sort_pack");
}

}  // namespace msplat
