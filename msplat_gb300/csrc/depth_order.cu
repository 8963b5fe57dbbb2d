// Depth-presorted tile ordering: the per-tile lists come out in (depth, id)
// order without a per-tile sort.
//
//   1. Each view's Gaussians are sorted once by depth: a stable LSD radix sort
//      of (depth bits, Gaussian id) on 8-bit digits, four passes of
//      histogram -> scan -> scatter; inactive Gaussians (culled, or depth not
//      finite and positive) carry the key 0xffffffff and sort last.  Stability
//      puts equal depths in id order, the reference's tie rule.
//   2. Their tile rectangles (computed by the projection) are written in that
//      order by the last sort pass (8 bytes each).
//   3. The block-aggregated count and scatter of the other path run over the
//      sorted positions p: CTA c covers p in [1024 c, 1024 c + 1024), so each
//      tile's bucket is a sequence of per-CTA runs in increasing depth, and
//      the key stored is p itself.
//   4. Inside a run the scatter's shared-memory slot order is arbitrary: each
//      key's place is the run's start plus the number of smaller keys in the
//      run (positions are unique), and the id written there is the Gaussian at
//      position p.  Runs are short (a CTA's 1024 Gaussians are a thin depth
//      slab spread over the image); the count is quadratic in a run's length,
//      which stays within 1024 (1024 Gaussians per CTA rather than 2048 or
//      512: shorter runs against a larger count table).
// The lists are the same as the per-tile radix sort's (same keys, same
// order); the scan and the class lists of tiles.cu are shared.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"

namespace msplat {

constexpr int kGsThreads = 256;
constexpr int kGsItems = kGsPerCta / kGsThreads;   // keys per thread of a radix-sort CTA
static_assert(kGsItems * kGsThreads == kGsPerCta, "whole rounds of 32 keys per warp");
static_assert(kAggPerCta == 1 << kAggShift, "a run is the positions p with equal p >> kAggShift");

// (radius and depth are loaded together: a culled record's depth is read
// but not used)
__device__ __forceinline__ uint32_t gs_key0(const TileArgs &a, size_t u) {
    const int r = a.radii[u];
    const float d = a.depths[u];
    return (r > 0 && finite_bits(d) && d > 0.0f) ? __float_as_uint(d) : 0xffffffffu;
}

constexpr uint32_t kGsMask = kGsDigits - 1;
constexpr int kGsDigitsPerThread = kGsDigits / kGsThreads;   // digits each thread of a block handles
static_assert(kGsDigitsPerThread * kGsThreads == kGsDigits, "whole digits per thread");

// Digit counts of one kGsPerCta-key block: hist[view][digit][block].
template <bool kFirst>
__global__ void __launch_bounds__(kGsThreads) k_gs_hist(TileArgs a, int shift, const uint32_t *key_in) {
    pdl_enter();
    __shared__ uint32_t h[kGsDigits];
    const int view = blockIdx.y, n = a.vt.n, nb = gridDim.x;
    const size_t vb = (size_t)view * n;
    const int e0 = blockIdx.x * kGsPerCta;
    uint32_t key[kGsItems];   // all of the thread's keys, loaded while the counts are cleared
#pragma unroll
    for (int j = 0; j < kGsItems; j++) {
        const int e = e0 + j * kGsThreads + (int)threadIdx.x;
        key[j] = e < n ? (kFirst ? gs_key0(a, vb + e) : key_in[vb + e]) : 0u;
    }
    for (int d = threadIdx.x; d < kGsDigits; d += kGsThreads) h[d] = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kGsItems; j++)
        if (e0 + j * kGsThreads + (int)threadIdx.x < n) atomicAdd(&h[(key[j] >> shift) & kGsMask], 1u);
    __syncthreads();
    for (int d = threadIdx.x; d < kGsDigits; d += kGsThreads)
        a.gs_hist[(size_t)view * kGsDigits * nb + (size_t)d * nb + blockIdx.x] = h[d];
}

// Per digit (one warp each), the exclusive scan of its blocks' counts in
// place, and the digit's total to dtot[view][digit].  In rounds of 1024
// blocks: the warp loads the round's counts at once (coalesced) into its
// shared buffer, each lane sums a contiguous run of 32, a warp scan of the
// run sums gives each run's offset, and the lane rewrites its run as
// offsets; the buffer is padded by a word per 32 (no bank conflicts either
// way).
constexpr int kDsPer = 32;                       // counts per lane per round
constexpr int kDsRound = 32 * kDsPer;            // counts per warp per round
__device__ __forceinline__ int ds_pad(int i) { return i + (i >> 5); }

__global__ void __launch_bounds__(256) k_gs_digit_scan(TileArgs a, int nb) {
    pdl_enter();
    __shared__ uint32_t buf[8][kDsRound + kDsRound / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int d = blockIdx.x * 8 + w, view = blockIdx.y;
    uint32_t *h = a.gs_hist + (size_t)view * kGsDigits * nb + (size_t)d * nb;
    uint32_t *sb = buf[w];
    uint32_t carry = 0;
    for (int b0 = 0; b0 < nb; b0 += kDsRound) {
        const int m = min(nb - b0, kDsRound);
        uint32_t v[kDsPer];
#pragma unroll
        for (int k = 0; k < kDsPer; k++) {
            const int b = 32 * k + lane;
            v[k] = b < m ? h[b0 + b] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kDsPer; k++) sb[ds_pad(32 * k + lane)] = v[k];
        __syncwarp();
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kDsPer; j++) sum += sb[ds_pad(lane * kDsPer + j)];
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        uint32_t run = carry + inc - sum;
#pragma unroll
        for (int j = 0; j < kDsPer; j++) {
            const int i = ds_pad(lane * kDsPer + j);
            const uint32_t x = sb[i];
            sb[i] = run;
            run += x;
        }
        carry += __shfl_sync(0xffffffffu, inc, 31);
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kDsPer; k++) {
            const int b = 32 * k + lane;
            if (b < m) h[b0 + b] = sb[ds_pad(b)];
        }
        __syncwarp();   // the buffer is refilled by the next round
    }
    if (lane == 0) a.gs_dtot[(size_t)view * kGsDigits + d] = carry;
}

// Stable scatter of one kGsPerCta-key block: warp w holds keys
// [32 kGsItems w, 32 kGsItems (w + 1)) of the block in kGsItems rounds of 32;
// a key's place is its digit's offset for
// the block + the same digit's keys in earlier warps + in earlier rounds of
// its warp + in lower lanes of its round (peers found with eight ballots).
// The last pass also writes each sorted position's tile rectangle (srect,
// gathered from the projection's; empty for inactive keys).
template <bool kFirst>
__global__ void __launch_bounds__(kGsThreads) k_gs_scatter(TileArgs a, int shift, const uint32_t *key_in,
                                                           const uint32_t *val_in, uint32_t *key_out,
                                                           uint32_t *val_out, ushort4 *srect_out) {
    pdl_enter();
    // wcnt: per warp and digit the keys counted so far, then (in place) the
    // earlier warps' keys of the digit
    __shared__ uint16_t wcnt[kGsThreads / 32][kGsDigits];
    __shared__ uint32_t base[kGsDigits];
    __shared__ uint32_t wsum[kGsThreads / 32];
    const int view = blockIdx.y, n = a.vt.n, nb = gridDim.x;
    const size_t vb = (size_t)view * n;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // the warp's keys, ids and (last pass) tile rectangles, all loaded before
    // the block's digit starts are computed
    const int e0 = blockIdx.x * kGsPerCta + wid * (32 * kGsItems);
    uint32_t kv[kGsItems], vv[kGsItems], rank[kGsItems];
    ushort4 rc[kGsItems];
#pragma unroll
    for (int j = 0; j < kGsItems; j++) {
        const int e = e0 + j * 32 + lane;
        const bool valid = e < n;
        kv[j] = valid ? (kFirst ? gs_key0(a, vb + e) : key_in[vb + e]) : 0u;
        vv[j] = valid ? (kFirst ? (uint32_t)e : val_in[vb + e]) : 0u;
    }
    if (srect_out) {
#pragma unroll
        for (int j = 0; j < kGsItems; j++)
            rc[j] = (e0 + j * 32 + lane < n && kv[j] != 0xffffffffu) ? a.rect[vb + vv[j]] : make_ushort4(0, 0, 0, 0);
    }
    for (int k = tid; k < (kGsThreads / 32) * kGsDigits; k += kGsThreads) (&wcnt[0][0])[k] = 0;
    {   // this block's start for digits kGsDigitsPerThread tid ..: the digit's
        // start (exclusive scan of the digit totals) + the earlier blocks' keys
        // of that digit
        const uint32_t *dt = a.gs_dtot + (size_t)view * kGsDigits + kGsDigitsPerThread * tid;
        uint32_t tot = 0;
#pragma unroll
        for (int q = 0; q < kGsDigitsPerThread; q++) tot += dt[q];
        uint32_t inc = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) wsum[wid] = inc;
        __syncthreads();
        uint32_t run = inc - tot;
        for (int w = 0; w < wid; w++) run += wsum[w];
        const uint32_t *hb = a.gs_hist + (size_t)view * kGsDigits * nb + blockIdx.x;
#pragma unroll
        for (int q = 0; q < kGsDigitsPerThread; q++) {
            const int d = kGsDigitsPerThread * tid + q;
            base[d] = run + hb[(size_t)d * nb];
            run += dt[q];
        }
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int j = 0; j < kGsItems; j++) {
        const int e = e0 + j * 32 + lane;
        const bool valid = e < n;
        const uint32_t d = valid ? ((kv[j] >> shift) & kGsMask) : (uint32_t)kGsDigits;
        uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int bit = 0; bit < kGsBits; bit++) {
            const uint32_t m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
            peers &= ((d >> bit) & 1u) ? m : ~m;
        }
        uint32_t old = 0;
        if (valid) old = wcnt[wid][d];
        __syncwarp();
        rank[j] = valid ? old + __popc(peers & lt) : 0xffffffffu;
        if (valid && (peers & lt) == 0) wcnt[wid][d] = (uint16_t)(old + __popc(peers));
        __syncwarp();
    }
    __syncthreads();
    // per digit, the counts of the earlier warps (in place)
    for (int d = tid; d < kGsDigits; d += kGsThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kGsThreads / 32; w++) {
            const uint32_t c = wcnt[w][d];
            wcnt[w][d] = (uint16_t)run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kGsItems; j++) {
        if (rank[j] == 0xffffffffu) continue;
        const uint32_t d = (kv[j] >> shift) & kGsMask;
        const uint32_t pos = base[d] + wcnt[wid][d] + rank[j];
        if (MS_GUARD(pos < (uint32_t)n, 7, pos, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr)) {
            key_out[vb + pos] = kv[j];
            val_out[vb + pos] = vv[j];
            if (srect_out) srect_out[vb + pos] = rc[j];
        }
    }
}

// The tile rectangles of this thread's sorted positions g0 + threadIdx.x +
// u kAggThreads (empty past the view's last Gaussian).
constexpr int kAggPerThread = kAggPerCta / kAggThreads;
static_assert(kAggPerThread * kAggThreads == kAggPerCta, "whole positions per thread");
__device__ __forceinline__ void srect_rows(const TileArgs &a, size_t vb, int g0, ushort4 (&r)[kAggPerThread]) {
#pragma unroll
    for (int u = 0; u < kAggPerThread; u++) {
        const int p = g0 + (int)threadIdx.x + u * kAggThreads;
        r[u] = p < a.vt.n ? a.srect[vb + p] : make_ushort4(0, 0, 0, 0);
    }
}

// Block-aggregated count over sorted positions (k_count_agg's rows).
__global__ void __launch_bounds__(kAggThreads) k_count_agg_sorted(TileArgs a) {
    pdl_enter();
    extern __shared__ uint32_t bins[];
    const int view = blockIdx.y;
    const ViewGeom vg = view_geom(a.vt, view);
    const int T = vg.tiles_x * vg.tiles_y;
    ushort4 r[kAggPerThread];   // this thread's rectangles, loaded while the histogram is cleared
    srect_rows(a, (size_t)view * a.vt.n, blockIdx.x * kAggPerCta, r);
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = 0;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kAggPerThread; u++)
        for (int y = r[u].y; y < r[u].w; y++)
            for (int x = r[u].x; x < r[u].z; x++) atomicAdd(&bins[y * vg.tiles_x + x], 1u);
    __syncthreads();
    uint32_t *row = a.cta_bins + (size_t)gridDim.x * vg.tile_base + (size_t)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) row[t] = bins[t];
}

// Block-aggregated scatter over sorted positions: the key is the position p.
template <bool kGroup>
__global__ void __launch_bounds__(kAggThreads) k_scatter_agg_sorted(TileArgs a) {
    pdl_enter();
    extern __shared__ uint32_t bins[];
    const int view = blockIdx.y;
    const ViewGeom vg = view_geom(a.vt, view);
    const int T = vg.tiles_x * vg.tiles_y;
    const int g0 = blockIdx.x * kAggPerCta;
    ushort4 r[kAggPerThread];   // this thread's rectangles, loaded while the slot table is filled
    srect_rows(a, (size_t)view * a.vt.n, g0, r);
    const uint32_t *row = a.cta_bins + (size_t)gridDim.x * vg.tile_base + (size_t)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) bins[t] = a.tile_offsets[vg.tile_base + t] + row[t];
    __syncthreads();
    uint32_t *keys = reinterpret_cast<uint32_t *>(a.keys);
#pragma unroll
    for (int u = 0; u < kAggPerThread; u++) {
        const uint32_t p = (uint32_t)(g0 + threadIdx.x + u * kAggThreads);
        for (int y = r[u].y; y < r[u].w; y++)
            for (int x = r[u].x; x < r[u].z; x++) {
                const int lt = y * vg.tiles_x + x;
                if (kGroup && (vg.tile_base + lt < a.tile_lo || vg.tile_base + lt >= a.tile_hi)) continue;
                const uint64_t dst = (uint64_t)atomicAdd(&bins[lt], 1u) - (kGroup ? (uint64_t)a.isect_lo : 0ull);
                if (dst < (uint64_t)a.capacity) keys[dst] = p;   // overflow is dropped, never written
            }
    }
}

// Each tile's runs in order: the key at slot j (a sorted position p) goes to
// its run's start + the number of smaller keys in the run; the record id of
// the Gaussian at p is written there.  The run's bounds are two entries of
// the tile's column of cta_bins; keys and bounds are read through L1 (staging
// them in shared memory measured slower at 1M Gaussians, 1297x840: 1.354 ms
// per step with up to 4096 staged keys, 1.369 with 8192, 1.343 without); the
// id gather is issued before the count.  A tile whose bucket does not fit the
// buffer is emitted transparent.
constexpr int kOrderThreads = 512;   // 1M, 1297x840: 1.331 ms per step; 256: 1.336-1.338, 1024: 1.343, 128: 1.361

__global__ void __launch_bounds__(kOrderThreads) k_tile_order(TileArgs a, int ctas) {
    pdl_enter();
    const int t = a.tile_lo + blockIdx.x;
    if (t >= a.tile_hi) return;
    const int count = (int)a.tile_counts[t];
    if (count == 0) return;
    const uint64_t start = (uint64_t)a.tile_offsets[t] - (uint64_t)a.isect_lo;
    if (start + (uint64_t)count > (uint64_t)a.capacity) {
        for (int j = threadIdx.x; j < count; j += blockDim.x)
            if (start + j < (uint64_t)a.capacity) a.isect_ids[start + j] = 0xffffffffu;
        return;
    }
    const int view = view_of_tile(a.vt, t);
    const ViewGeom vg = view_geom(a.vt, view);
    const int Tv = vg.tiles_x * vg.tiles_y;
    const uint32_t *col = a.cta_bins + (size_t)ctas * vg.tile_base + (t - vg.tile_base);   // run starts: col[c * Tv]
    const uint32_t *keys = reinterpret_cast<const uint32_t *>(a.keys) + start;
    const size_t vb = (size_t)view * a.vt.n;
    for (int j = threadIdx.x; j < count; j += blockDim.x) {
        const uint32_t p = keys[j];
        const uint32_t gid = a.gs_val[kGsPasses & 1][vb + p];
        const int c = (int)(p >> kAggShift);
        const uint32_t rs = col[(size_t)c * Tv];
        const uint32_t re = c + 1 < ctas ? col[(size_t)(c + 1) * Tv] : (uint32_t)count;
        uint32_t below = 0;
        for (uint32_t q = rs; q < re; q++) below += keys[q] < p ? 1u : 0u;
        const uint32_t dst = rs + below;
        if (MS_GUARD(dst < (uint32_t)count, 8, dst, a.nan_counts ? a.nan_counts + kDbgSlot : nullptr))
            a.isect_ids[start + dst] = (uint32_t)(vb + gid);
    }
}

int launch_presorted_count(const TileArgs &a, cudaStream_t s) {
    const int n = a.vt.n, views = a.vt.count;
    const int nb = (n + kGsPerCta - 1) / kGsPerCta;
    const dim3 g(nb, views);
    // pass 0 reads the keys from the projection; passes alternate buffers 1, 0, 1, ...
    const dim3 gd(kGsDigits / 8, views);   // one warp per digit, 8 per CTA
    launch_pdl(k_gs_hist<true>, g, kGsThreads, 0, s, a, 0, nullptr);
    launch_pdl(k_gs_digit_scan, gd, 256, 0, s, a, nb);
    launch_pdl(k_gs_scatter<true>, g, kGsThreads, 0, s, a, 0, nullptr, nullptr, a.gs_key[1], a.gs_val[1],
               kGsPasses == 1 ? a.srect : (ushort4 *)nullptr);
    for (int pass = 1; pass < kGsPasses; pass++) {
        const int src = pass & 1, dst = src ^ 1;
        launch_pdl(k_gs_hist<false>, g, kGsThreads, 0, s, a, kGsBits * pass, a.gs_key[src]);
        launch_pdl(k_gs_digit_scan, gd, 256, 0, s, a, nb);
        launch_pdl(k_gs_scatter<false>, g, kGsThreads, 0, s, a, kGsBits * pass, a.gs_key[src], a.gs_val[src],
                   a.gs_key[dst], a.gs_val[dst], pass == kGsPasses - 1 ? a.srect : (ushort4 *)nullptr);
    }
    debug_sync(s, "depth_sort");
    const int agg_blocks = (n + kAggPerCta - 1) / kAggPerCta;
    const size_t smem = (size_t)max_view_tiles(a.vt) * sizeof(uint32_t);
    static bool done[64] = {false};
    static std::mutex mu;
    once_per_device(mu, done, []() {   // (a failure stays in cudaGetLastError for the launch check)
        cudaError_t e = cudaFuncSetAttribute(k_count_agg_sorted, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kAggMaxTiles * 4);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_scatter_agg_sorted<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kAggMaxTiles * 4);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_scatter_agg_sorted<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     kAggMaxTiles * 4);
        return e;
    });
    launch_pdl(k_count_agg_sorted, dim3(agg_blocks, views), kAggThreads, smem, s, a);
    debug_sync(s, "count_sorted");
    return 3 * kGsPasses + 1;
}

int launch_presorted_build(const TileArgs &a, cudaStream_t s) {
    const int n = a.vt.n, views = a.vt.count;
    const int agg_blocks = (n + kAggPerCta - 1) / kAggPerCta;
    const size_t smem = (size_t)max_view_tiles(a.vt) * sizeof(uint32_t);
    const bool grp = a.tile_lo > 0 || a.tile_hi < a.num_tiles || a.isect_lo > 0;
    if (grp) launch_pdl(k_scatter_agg_sorted<true>, dim3(agg_blocks, views), kAggThreads, smem, s, a);
    else launch_pdl(k_scatter_agg_sorted<false>, dim3(agg_blocks, views), kAggThreads, smem, s, a);
    debug_sync(s, "scatter_sorted");
    if (a.tile_hi > a.tile_lo) launch_pdl(k_tile_order, a.tile_hi - a.tile_lo, kOrderThreads, 0, s, a, agg_blocks);
    debug_sync(s, "tile_order");
    return 2;
}

}  // namespace msplat
