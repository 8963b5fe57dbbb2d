// GPU-resident MCMC relocation and growth (Model::mcmcAfterTrain,
// core/src/model.cpp:497-660, with relocate :336-416, addNewGaussians
// :419-495 and computeRelocation :311-332), which the reference runs on the
// CPU after a full device drain every 100 steps.
//
//  1. classify: dead = non-finite parameter, sigmoid(opacity) <= 0.005, or
//     |mean|^2 > cull_radius^2; weight = sigmoid(opacity) of the living;
//  2. device scans: compacted dead list, FP64 cumulative weights;
//  3. every dead slot draws a source with probability proportional to its
//     weight (counter-based uniform + binary search in the cumulative
//     weights; the reference's std::discrete_distribution over mt19937 is
//     the same distribution, not the same stream).  The weight is
//     sigmoid(opacity), or, with the learned proposal, the MLP's score;
//  4. each drawn source with c copies is rescaled by Eq. 9 with n = c + 1
//     and its Adam moments zeroed; then every dead slot copies its source
//     and has its moments zeroed;
//  5. growth: min(cap, 1.05 N) - N new slots drawn the same way over all N.
#include <cstdio>
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "kernels.h"

namespace msplat {

__device__ __forceinline__ uint32_t mix32(uint32_t seed, uint32_t idx) {
    uint32_t x = seed * 747796405u + idx * 2891336453u;
    x = ((x >> ((x >> 28) + 4)) ^ x) * 277803737u;
    return (x >> 22) ^ x;
}

// uniform in [0, 1) with 53 random bits
__device__ __forceinline__ double unit53(uint32_t seed, uint32_t j) {
    const uint64_t hi = mix32(seed, 2u * j), lo = mix32(seed ^ 0x85EBCA6Bu, 2u * j + 1u);
    const uint64_t bits = ((hi << 32) | lo) >> 11;
    return (double)bits * (1.0 / 9007199254740992.0);
}

__device__ __forceinline__ bool all_finite(const float *p, int n) {
    bool ok = true;
    for (int k = 0; k < n; k++) ok = ok && finite_bits(p[k]);
    return ok;
}

__global__ void k_mcmc_classify(McmcArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const int rs = 3 * a.rest_bases;
    const bool fin = finite_bits(a.opacities[i]) && all_finite(a.means + 3 * (size_t)i, 3) &&
                     all_finite(a.scales + 3 * (size_t)i, 3) && all_finite(a.quats + 4 * (size_t)i, 4) &&
                     all_finite(a.features_dc + 3 * (size_t)i, 3) && all_finite(a.features_rest + (size_t)rs * i, rs);
    const float sig = 1.0f / (1.0f + expf(-a.opacities[i]));
    bool dead = !fin || (sig <= 0.005f);
    bool culled = false;
    if (!dead && a.cull_r2 > 0.0f) {
        const float x = a.means[3 * i], y = a.means[3 * i + 1], z = a.means[3 * i + 2];
        if (x * x + y * y + z * z > a.cull_r2) { dead = true; culled = true; }
    }
    a.flags[i] = dead ? 1u : 0u;
    const float w = a.score ? a.score[i] : sig;
    a.weights[i] = dead ? 0.0 : ((finite_bits(w) && w > 0.f) ? (double)w : 0.0);
    if (!fin) atomicAdd(a.counters + 0, 1u);
    if (culled) atomicAdd(a.counters + 1, 1u);
}

// weights over all n Gaussians for growth (no one is dead at that point)
__global__ void k_mcmc_weights(McmcArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const float sig = 1.0f / (1.0f + expf(-a.opacities[i]));
    const float w = a.score ? a.score[i] : sig;
    a.weights[i] = (finite_bits(w) && w > 0.f) ? (double)w : 0.0;
}

// ---- block scans (one level per launch; the partials are scanned by one CTA) ----
constexpr int kScanT = 512, kScanPer = 4, kScanTile = kScanT * kScanPer;

template <class T> __device__ T block_excl_scan(T v, T *warp_sums, T &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) warp_sums[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        T s = (lane < kScanT / 32) ? warp_sums[lane] : T(0), si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const T u = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += u;
        }
        if (lane < kScanT / 32) warp_sums[lane] = si - s;
        if (lane == 31) warp_sums[32] = si;
    }
    __syncthreads();
    const T r = warp_sums[wid] + inc - v;
    total = warp_sums[32];
    __syncthreads();
    return r;
}

// in[i] -> out[i] exclusive (inclusive if incl) within tiles of kScanTile; tile totals -> part
template <class T> __global__ void k_scan_tiles(const T *in, T *out, T *part, int n, int incl) {
    __shared__ T ws[33];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
    T v[kScanPer], s = T(0);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        v[k] = (base + k < n) ? in[base + k] : T(0);
        s += v[k];
    }
    T total;
    T run = block_excl_scan<T>(s, ws, total);
#pragma unroll
    for (int k = 0; k < kScanPer; k++) {
        if (base + k < n) out[base + k] = incl ? run + v[k] : run;
        run += v[k];
    }
    if (threadIdx.x == 0) part[blockIdx.x] = total;
}

// one CTA: exclusive scan of the tile totals (any count), in place; total -> part[m]
template <class T> __global__ void k_scan_parts(T *part, int m) {
    __shared__ T ws[33];
    T carry = T(0);
    for (int c0 = 0; c0 < m; c0 += kScanT) {
        const int i = c0 + threadIdx.x;
        const T v = i < m ? part[i] : T(0);
        T total;
        const T r = block_excl_scan<T>(v, ws, total);
        if (i < m) part[i] = carry + r;
        carry += total;
    }
    if (threadIdx.x == 0) part[m] = carry;
}

template <class T> __global__ void k_scan_add(T *out, const T *part, int n) {
    const int i = blockIdx.x * kScanTile + threadIdx.x;
    const T add = part[blockIdx.x];
    for (int k = 0; k < kScanPer; k++) {
        const int j = i + k * kScanT;
        if (j < n) out[j] += add;
    }
}

template <class T> void device_scan(const T *in, T *out, T *part, int n, bool inclusive, cudaStream_t s) {
    const int tiles = (n + kScanTile - 1) / kScanTile;
    k_scan_tiles<T><<<tiles, kScanT, 0, s>>>(in, out, part, n, inclusive ? 1 : 0);
    k_scan_parts<T><<<1, kScanT, 0, s>>>(part, tiles);
    k_scan_add<T><<<tiles, kScanT, 0, s>>>(out, part, n);
}

__global__ void k_mcmc_dead_list(McmcArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || !a.flags[i]) return;
    a.dead_list[a.flag_pos[i]] = i;
}

// move j draws its source; dst = dead_list[j] (relocation) or n + j (growth)
__global__ void k_mcmc_draw(McmcArgs a, int moves, int growth, uint32_t seed) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= moves) return;
    const double total = a.cumw[a.n - 1];
    const double target = unit53(seed, (uint32_t)j) * total;
    int lo = 0, hi = a.n - 1;   // first i with cumw[i] > target
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a.cumw[mid] > target) hi = mid; else lo = mid + 1;
    }
    const int dst = growth ? a.n + j : a.dead_list[j];
    a.moves[2 * j] = dst;
    a.moves[2 * j + 1] = lo;
    atomicAdd(a.copies + lo, 1u);
}

__device__ void eq9(float o_old, const float s_old[3], int n, float &o_new, float s_new[3]) {
    if (n < 1) n = 1;
    if (n > 51) n = 51;
    o_new = 1.0f - powf(1.0f - o_old, 1.0f / (float)n);
    const double on = (double)o_new;
    double denom = 0.0, binom = 1.0;
    for (int k = 1; k <= n; k++) {
        binom = binom * (double)(n - k + 1) / (double)k;
        const double term = binom * pow(on, (double)k) / sqrt((double)k);
        denom += (k & 1) ? term : -term;
    }
    double coeff = (denom > 1e-12) ? ((double)o_old / denom) : 1.0;
    if (!isfinite(coeff) || coeff <= 0.0) coeff = 1.0;
    for (int i = 0; i < 3; i++) s_new[i] = (float)((double)s_old[i] * coeff);
}

__device__ void zero_moments(const McmcArgs &a, int idx) {
    const int rs = 3 * a.rest_bases;
    const int stride[6] = {3, 3, 4, 3, rs, 1};
    for (int g = 0; g < 6; g++) {
        float *m = a.exp_avg[g] + (size_t)stride[g] * idx, *v = a.exp_avg_sq[g] + (size_t)stride[g] * idx;
        for (int k = 0; k < stride[g]; k++) { m[k] = 0.f; v[k] = 0.f; }
    }
}

// sources with c > 0 copies: Eq. 9 with n = c + 1, moments zeroed
__global__ void k_mcmc_rescale(McmcArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint32_t c = a.copies[i];
    if (c == 0) return;
    const float o_old = 1.0f / (1.0f + expf(-a.opacities[i]));
    const float s_old[3] = {expf(a.scales[3 * i]), expf(a.scales[3 * i + 1]), expf(a.scales[3 * i + 2])};
    float o_new, s_new[3];
    eq9(o_old, s_old, (int)c + 1, o_new, s_new);
    o_new = fminf(fmaxf(o_new, 1e-6f), 1.0f - 1e-6f);
    a.opacities[i] = logf(o_new / (1.0f - o_new));
    for (int j = 0; j < 3; j++) a.scales[3 * i + j] = logf(fmaxf(s_new[j], 1e-10f));
    zero_moments(a, i);
    a.copies[i] = 0;   // ready for the next round of draws
}

__global__ void k_mcmc_copy(McmcArgs a, int moves) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= moves) return;
    const int dst = a.moves[2 * j], src = a.moves[2 * j + 1];
    const int rs = 3 * a.rest_bases;
    for (int k = 0; k < 3; k++) a.means[3 * (size_t)dst + k] = a.means[3 * (size_t)src + k];
    for (int k = 0; k < 4; k++) a.quats[4 * (size_t)dst + k] = a.quats[4 * (size_t)src + k];
    for (int k = 0; k < 3; k++) a.features_dc[3 * (size_t)dst + k] = a.features_dc[3 * (size_t)src + k];
    for (int k = 0; k < rs; k++) a.features_rest[(size_t)rs * dst + k] = a.features_rest[(size_t)rs * src + k];
    a.opacities[dst] = a.opacities[src];
    for (int k = 0; k < 3; k++) a.scales[3 * (size_t)dst + k] = a.scales[3 * (size_t)src + k];
    zero_moments(a, dst);
    if (a.gstats) a.gstats[dst] = make_float4(0.f, 0.f, 0.f, 0.f);
}

static void ck(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("mcmc ") + what + ": " + cudaGetErrorString(e));
}

// One relocation + growth round.  Host control needs the dead count and the
// total weight, read back once each (the reference drains the device here).
void run_mcmc(McmcArgs a, int cap_max, int &relocation_count, McmcResult &res, cudaStream_t s) {
    res = McmcResult{};
    const int N = a.n;
    const int B = 256;
    res.num_active = N;
    if (N <= 0) return;
    ck(cudaMemsetAsync(a.counters, 0, 4 * sizeof(unsigned), s), "memset");
    ck(cudaMemsetAsync(a.copies, 0, sizeof(unsigned) * (size_t)cap_max, s), "memset");
    k_mcmc_classify<<<(N + B - 1) / B, B, 0, s>>>(a);
    device_scan<uint32_t>(a.flags, a.flag_pos, a.upart, N, false, s);
    device_scan<double>(a.weights, a.cumw, a.dpart, N, true, s);
    k_mcmc_dead_list<<<(N + B - 1) / B, B, 0, s>>>(a);
    unsigned cnt[4];
    ck(cudaMemcpyAsync(cnt, a.counters, sizeof(cnt), cudaMemcpyDeviceToHost, s), "readback");
    uint32_t last_pos = 0, last_flag = 0;
    double total = 0;
    ck(cudaMemcpyAsync(&last_pos, a.flag_pos + N - 1, 4, cudaMemcpyDeviceToHost, s), "readback");
    ck(cudaMemcpyAsync(&last_flag, a.flags + N - 1, 4, cudaMemcpyDeviceToHost, s), "readback");
    ck(cudaMemcpyAsync(&total, a.cumw + N - 1, 8, cudaMemcpyDeviceToHost, s), "readback");
    ck(cudaStreamSynchronize(s), "sync");
    const int dead = (int)(last_pos + last_flag);
    res.num_dead = dead;
    res.num_nonfinite = (int)cnt[0];
    res.num_culled = (int)cnt[1];
    // relocation: dead slots draw living sources (skipped without dead or weight)
    if (dead > 0 && dead < N && total > 0.0) {
        const uint32_t seed = 0x9E3779B9u ^ (uint32_t)(++relocation_count);
        k_mcmc_draw<<<(dead + B - 1) / B, B, 0, s>>>(a, dead, 0, seed);
        k_mcmc_rescale<<<(N + B - 1) / B, B, 0, s>>>(a);
        k_mcmc_copy<<<(dead + B - 1) / B, B, 0, s>>>(a, dead);
        res.num_relocated = dead;
    }
    // growth toward the cap by 5 %
    const int target = (int)(1.05f * (float)N) < cap_max ? (int)(1.05f * (float)N) : cap_max;
    const int num_new = target - N;
    if (num_new > 0) {
        k_mcmc_weights<<<(N + B - 1) / B, B, 0, s>>>(a);
        device_scan<double>(a.weights, a.cumw, a.dpart, N, true, s);
        ck(cudaMemcpyAsync(&total, a.cumw + N - 1, 8, cudaMemcpyDeviceToHost, s), "readback");
        ck(cudaStreamSynchronize(s), "sync");
        if (total > 0.0) {
            const uint32_t seed = 0xA24BAED4u ^ (uint32_t)(++relocation_count);
            McmcArgs g = a;
            g.moves = a.moves + 2 * (size_t)res.num_relocated;   // keep the relocation moves readable
            k_mcmc_draw<<<(num_new + B - 1) / B, B, 0, s>>>(g, num_new, 1, seed);
            k_mcmc_rescale<<<(N + B - 1) / B, B, 0, s>>>(g);
            k_mcmc_copy<<<(num_new + B - 1) / B, B, 0, s>>>(g, num_new);
            res.num_grown = num_new;
            res.num_active = N + num_new;
        }
    }
    ck(cudaGetLastError(), "launch");
}

}  // namespace msplat
