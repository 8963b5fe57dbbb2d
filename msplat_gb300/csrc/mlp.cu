// Learned relocation proposal: a 22 -> 64 -> 64 -> 2 MLP (SiLU) evaluated
// with tcgen05 tensor-core MMAs, BF16 operands and F32 accumulators in tensor
// memory (tcgen05.cuh).  One CTA of 128 threads takes 128 rows: the layer
// input sits in shared memory in the K-major core-matrix layout, one thread
// issues the MMAs of a layer, the four warps read the accumulator rows back
// (warp w owns TMEM lanes 32w..32w+31 = rows), add the bias, apply SiLU and
// write the next layer's BF16 input.
#include <cstdio>
#include <stdexcept>
#include <string>

#include "common.cuh"
#include "kernels.h"
#include "tcgen05.cuh"

namespace msplat {

// ---------------------------------------------------------------------------
// Probe of the MMA path: D[128 x N] = A[128 x K] * B[N x K]^T from row-major
// BF16 in global memory, F32 out.  Used by the library self-test.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_tc_gemm_probe(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D,
                                                      int N, int K, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    uint8_t *As = smem;                          // 128 x K
    uint8_t *Bs = smem + 128 * K * 2;            // N x K
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid == 0) tc::mbar_init(&bar, 1);
    if (warp == 0) tc::tmem_alloc(&tmem_base, 64);
    // stage: row r of A (K bf16) into its core matrices
    for (int e = tid; e < 128 * K; e += 128) {
        const int r = e / K, k = e % K;
        *reinterpret_cast<__nv_bfloat16 *>(As + tc::kmajor_off(r, k, K)) = A[e];
    }
    for (int e = tid; e < N * K; e += 128) {
        const int r = e / K, k = e % K;
        *reinterpret_cast<__nv_bfloat16 *>(Bs + tc::kmajor_off(r, k, K)) = B[e];
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t d = tmem_base;
    if (tid == 0) {
        const uint32_t id = tc::idesc_bf16(128, N);
        for (int s = 0; s < K / 16; s++) {
            const uint64_t ad = tc::smem_desc(tc::smem_u32(As) + 256 * s, 128, (K / 8) * 128);
            const uint64_t bd = tc::smem_desc(tc::smem_u32(Bs) + 256 * s, 128, (K / 8) * 128);
            tc::mma_bf16(d, ad, bd, id, s > 0);
        }
        tc::mma_commit(&bar);
    }
    __syncwarp();
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar, 0) ? 1 : 0) != 0;
    if (!ok) {
        if (tid == 0) atomicExch(err, 1u);
        tc::mbar_wait(&bar, 0);   // give an MMA still in flight a second bounded wait before freeing
    }
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + (tid & 31);
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(d + ((uint32_t)(warp * 32) << 16) + c0, v);
            for (int k = 0; k < 16; k++) D[row * N + c0 + k] = v[k];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem_base, 64);
}

int tc_gemm_probe(const void *A, const void *B, float *D, int N, int K, unsigned *err, cudaStream_t s) {
    if (N != 16 && N != 32 && N != 64) return -1;
    if (K != 16 && K != 32 && K != 64) return -1;
    const size_t smem = (size_t)(128 + N) * K * 2;
    k_tc_gemm_probe<<<1, 128, smem, s>>>(static_cast<const __nv_bfloat16 *>(A), static_cast<const __nv_bfloat16 *>(B),
                                         D, N, K, err);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

// ---------------------------------------------------------------------------
// The MLP: x[32] (22 features, zero padded) -> 64 -> 64 -> 2 (padded to 16).
// Weights live as FP32 master copies; k_mlp_pack writes their BF16 operand
// images (K-major core-matrix tiles, flat-copied into shared memory):
//   forward B operands  W1t [64 x 32], W2t [64 x 64], W3t [16 x 64]  (rows = out)
//   backward B operands W2b [64 x 64], W3b [64 x 16]                 (rows = in)
// ---------------------------------------------------------------------------

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z) {
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}

// pack 8 floats as bf16 into one 16-byte core-matrix row segment
__device__ __forceinline__ uint4 pack8(const float *v) {
    uint4 u;
    uint32_t *w = &u.x;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
        w[k] = *reinterpret_cast<const uint32_t *>(&h);
    }
    return u;
}

__device__ __forceinline__ float bf16_at(const uint8_t *tile, int r, int k, int K) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(tile + tc::kmajor_off(r, k, K)));
}

__global__ void k_mlp_pack(const float *P, uint8_t *img) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const float *W1 = P + kMlpW1, *W2 = P + kMlpW2, *W3 = P + kMlpW3;
    // W1t[o][i] = W1[i][o]   (64 x 32)
    if (t < 64 * 32) {
        const int o = t / 32, i = t % 32;
        *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1t + tc::kmajor_off(o, i, 32)) = __float2bfloat16_rn(W1[i * 64 + o]);
    }
    // W2t[o][i] = W2[i][o]; W2b[i][o] = W2[i][o]   (64 x 64)
    if (t < 64 * 64) {
        const int a = t / 64, b = t % 64;
        *reinterpret_cast<__nv_bfloat16 *>(img + kImgW2t + tc::kmajor_off(a, b, 64)) = __float2bfloat16_rn(W2[b * 64 + a]);
        *reinterpret_cast<__nv_bfloat16 *>(img + kImgW2b + tc::kmajor_off(a, b, 64)) = __float2bfloat16_rn(W2[a * 64 + b]);
    }
    // W3t[o][i] = W3[i][o] (16 x 64); W3b[i][o] = W3[i][o] (64 x 16)
    if (t < 16 * 64) {
        const int o = t / 64, i = t % 64;
        *reinterpret_cast<__nv_bfloat16 *>(img + kImgW3t + tc::kmajor_off(o, i, 64)) = __float2bfloat16_rn(W3[i * 16 + o]);
        *reinterpret_cast<__nv_bfloat16 *>(img + kImgW3b + tc::kmajor_off(i, o, 16)) = __float2bfloat16_rn(W3[i * 16 + o]);
    }
}

// shared-memory map of the MLP kernels (bytes)
constexpr int kSmX = 0, kSmW1t = 8192, kSmW2t = 12288, kSmW3t = 20480, kSmW2b = 22528, kSmW3b = 30720;
constexpr int kSmH1 = 32768, kSmH2 = 49152;                  // forward ends at 65536
constexpr int kSmDY = 65536, kSmDZ = 69632, kSmFDZ = 86016, kSmFDY = 118784, kSmTrainEnd = 126976;
constexpr uint32_t kTmemCols = 512;   // Z1 0..63, Z2 64..127, Y 128..143, dH2 144..207, dH1 208..271

struct MlpCtx {
    uint8_t *sm;
    uint32_t tmem;
    uint64_t *bar;
    uint32_t phase;
    bool ok;
};

// one MMA chain into TMEM columns [dcol, dcol + N), then every thread waits
__device__ __forceinline__ void mlp_gemm(MlpCtx &c, int a_off, int b_off, int K, int N, uint32_t dcol) {
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (threadIdx.x == 0 && c.ok) {
        const uint32_t id = tc::idesc_bf16(128, N);
        const uint32_t sbo = (uint32_t)(K / 8) * 128;
        for (int s = 0; s < K / 16; s++) {
            const uint64_t ad = tc::smem_desc(tc::smem_u32(c.sm + a_off) + 256 * s, 128, sbo);
            const uint64_t bd = tc::smem_desc(tc::smem_u32(c.sm + b_off) + 256 * s, 128, sbo);
            tc::mma_bf16(c.tmem + dcol, ad, bd, id, s > 0);
        }
        tc::mma_commit(c.bar);
    }
    __syncwarp();
    bool done = c.ok ? tc::mbar_wait(c.bar, c.phase) : true;
    done = __syncthreads_and(done ? 1 : 0) != 0;
    if (c.ok && !done) tc::mbar_wait(c.bar, c.phase);   // second bounded wait for an MMA still in flight
    c.ok = c.ok && done;
    c.phase ^= 1u;
    tc::fence_after_sync();
}

// TMEM columns of this thread's row
__device__ __forceinline__ uint32_t row_taddr(const MlpCtx &c, uint32_t col) {
    return c.tmem + ((uint32_t)((threadIdx.x >> 5) * 32) << 16) + col;
}

// forward epilogue of a hidden layer: SiLU(acc + bias) -> BF16 tile [128 x 64]
__device__ __forceinline__ void mlp_hidden_epilogue(MlpCtx &c, uint32_t col, const float *bias, int out_off) {
    const int r = threadIdx.x;
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        if (c.ok) tc::tmem_ld16(row_taddr(c, col + c0), v);
        else for (int k = 0; k < 16; k++) v[k] = 0.f;
        for (int k = 0; k < 16; k++) v[k] = silu(v[k] + bias[c0 + k]);
        *reinterpret_cast<uint4 *>(c.sm + out_off + tc::kmajor_off(r, c0, 64)) = pack8(v);
        *reinterpret_cast<uint4 *>(c.sm + out_off + tc::kmajor_off(r, c0 + 8, 64)) = pack8(v + 8);
    }
}

__device__ __forceinline__ void mlp_setup(MlpCtx &c, uint8_t *sm, uint64_t *bar, uint32_t *tmem_slot,
                                          const uint8_t *img, const __nv_bfloat16 *X, int n, int row0, bool train) {
    const int tid = threadIdx.x, warp = tid >> 5;
    c.sm = sm;
    c.bar = bar;
    c.phase = 0;
    c.ok = true;
    if (tid == 0) tc::mbar_init(bar, 1);
    if (warp == 0) tc::tmem_alloc(tmem_slot, kTmemCols);
    // weights: flat copy of the operand images
    const int wbytes = train ? (kSmW3b + 2048 - kSmW1t) : (kSmW2b - kSmW1t);
    for (int o = tid * 16; o < wbytes; o += 128 * 16)
        *reinterpret_cast<uint4 *>(sm + kSmW1t + o) = *reinterpret_cast<const uint4 *>(img + kImgW1t + o);
    // input rows (zero past n)
    const int r = tid, g = row0 + r;
    for (int k8 = 0; k8 < 32; k8 += 8) {
        uint4 u = make_uint4(0, 0, 0, 0);
        if (g < n) u = *reinterpret_cast<const uint4 *>(X + (size_t)g * 32 + k8);
        *reinterpret_cast<uint4 *>(sm + kSmX + tc::kmajor_off(r, k8, 32)) = u;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    c.tmem = *tmem_slot;
}

__device__ __forceinline__ void mlp_forward_core(MlpCtx &c, const float *b1, const float *b2) {
    mlp_gemm(c, kSmX, kSmW1t, 32, 64, 0);
    mlp_hidden_epilogue(c, 0, b1, kSmH1);
    mlp_gemm(c, kSmH1, kSmW2t, 64, 64, 64);
    mlp_hidden_epilogue(c, 64, b2, kSmH2);
    mlp_gemm(c, kSmH2, kSmW3t, 64, 16, 128);
}

__device__ __forceinline__ void mlp_teardown(MlpCtx &c, unsigned *err) {
    if (!c.ok && threadIdx.x == 0 && err) atomicExch(err, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tc::tmem_free(c.tmem, kTmemCols);
}

// inference: out[g] = (y0, y1) for rows g = 128 * blockIdx.x + thread
__global__ void __launch_bounds__(128) k_mlp_forward(const __nv_bfloat16 *X, int n, const uint8_t *img,
                                                    const float *P, float2 *out, unsigned *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_slot;
    MlpCtx c;
    mlp_setup(c, sm, &bar, &tmem_slot, img, X, n, blockIdx.x * 128, false);
    mlp_forward_core(c, P + kMlpB1, P + kMlpB2);
    float v[16];
    if (c.ok) tc::tmem_ld16(row_taddr(c, 128), v);
    else for (int k = 0; k < 16; k++) v[k] = 0.f;
    const int g = blockIdx.x * 128 + threadIdx.x;
    if (g < n) out[g] = make_float2(v[0] + P[kMlpB3], v[1] + P[kMlpB3 + 1]);
    mlp_teardown(c, err);
}

// training: MSE against targets T, gradients (FP32) added into G, loss into *loss
__global__ void __launch_bounds__(128) k_mlp_train(const __nv_bfloat16 *X, const float2 *T, int n, const uint8_t *img,
                                                  const float *P, float *G, float *loss, float inv_count,
                                                  unsigned *err) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_slot;
    MlpCtx c;
    const int tid = threadIdx.x;
    const int g = blockIdx.x * 128 + tid;
    mlp_setup(c, sm, &bar, &tmem_slot, img, X, n, blockIdx.x * 128, true);
    mlp_forward_core(c, P + kMlpB1, P + kMlpB2);
    float *fdy = reinterpret_cast<float *>(sm + kSmFDY);   // [128][16]
    float *fdz = reinterpret_cast<float *>(sm + kSmFDZ);   // [128][64]
    // dL/dy for L = sum (y - t)^2 * inv_count over the 2 outputs
    {
        float v[16];
        if (c.ok) tc::tmem_ld16(row_taddr(c, 128), v);
        else for (int k = 0; k < 16; k++) v[k] = 0.f;
        float dy[16];
        for (int k = 0; k < 16; k++) dy[k] = 0.f;
        float l = 0.f;
        if (g < n) {
            const float2 t = T[g];
            const float y0 = v[0] + P[kMlpB3], y1 = v[1] + P[kMlpB3 + 1];
            const float e0 = y0 - t.x, e1 = y1 - t.y;
            l = (e0 * e0 + e1 * e1) * inv_count;
            dy[0] = 2.f * e0 * inv_count;
            dy[1] = 2.f * e1 * inv_count;
        }
        for (int k = 0; k < 16; k++) fdy[tid * 16 + k] = dy[k];
        *reinterpret_cast<uint4 *>(sm + kSmDY + tc::kmajor_off(tid, 0, 16)) = pack8(dy);
        *reinterpret_cast<uint4 *>(sm + kSmDY + tc::kmajor_off(tid, 8, 16)) = pack8(dy + 8);
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((tid & 31) == 0) atomicAdd(loss, l);
    }
    // dH2 = dY W3^T  (TMEM 144..207)
    mlp_gemm(c, kSmDY, kSmW3b, 16, 64, 144);
    // dZ2 = dH2 * SiLU'(Z2): BF16 A tile for dH1, FP32 copy for dW2
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float dh[16], z[16];
        if (c.ok) {
            tc::tmem_ld16(row_taddr(c, 144 + c0), dh);
            tc::tmem_ld16(row_taddr(c, 64 + c0), z);
        } else {
            for (int k = 0; k < 16; k++) dh[k] = z[k] = 0.f;
        }
        for (int k = 0; k < 16; k++) {
            z[k] = dh[k] * silu_grad(z[k] + P[kMlpB2 + c0 + k]);
            fdz[tid * 64 + c0 + k] = z[k];
        }
        *reinterpret_cast<uint4 *>(sm + kSmDZ + tc::kmajor_off(tid, c0, 64)) = pack8(z);
        *reinterpret_cast<uint4 *>(sm + kSmDZ + tc::kmajor_off(tid, c0 + 8, 64)) = pack8(z + 8);
    }
    // dH1 = dZ2 W2^T  (TMEM 208..271); the barrier inside also publishes fdz/fdy
    mlp_gemm(c, kSmDZ, kSmW2b, 64, 64, 208);
    // dW3[i][o] = sum_r H2[r][i] dY[r][o] (o < 2), db3; dW2[i][o] = sum_r H1[r][i] dZ2[r][o], db2
    {
        const int i = tid >> 1, o = tid & 1;
        float acc = 0.f;
        for (int r = 0; r < 128; r++) acc += bf16_at(sm + kSmH2, r, i, 64) * fdy[r * 16 + o];
        atomicAdd(G + kMlpW3 + i * 16 + o, acc);
        if (tid < 2) {
            float b = 0.f;
            for (int r = 0; r < 128; r++) b += fdy[r * 16 + tid];
            atomicAdd(G + kMlpB3 + tid, b);
        }
        const int o0 = (tid & 1) * 32;
        float a2[32];
        for (int k = 0; k < 32; k++) a2[k] = 0.f;
        for (int r = 0; r < 128; r++) {
            const float h = bf16_at(sm + kSmH1, r, i, 64);
            const float4 *dz = reinterpret_cast<const float4 *>(fdz + r * 64 + o0);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float4 d = dz[q];
                a2[4 * q] += h * d.x; a2[4 * q + 1] += h * d.y; a2[4 * q + 2] += h * d.z; a2[4 * q + 3] += h * d.w;
            }
        }
        for (int k = 0; k < 32; k++) atomicAdd(G + kMlpW2 + i * 64 + o0 + k, a2[k]);
        if (tid < 64) {
            float b = 0.f;
            for (int r = 0; r < 128; r++) b += fdz[r * 64 + tid];
            atomicAdd(G + kMlpB2 + tid, b);
        }
    }
    __syncthreads();   // fdz is overwritten below
    // dZ1 = dH1 * SiLU'(Z1)
    for (int c0 = 0; c0 < 64; c0 += 16) {
        float dh[16], z[16];
        if (c.ok) {
            tc::tmem_ld16(row_taddr(c, 208 + c0), dh);
            tc::tmem_ld16(row_taddr(c, 0 + c0), z);
        } else {
            for (int k = 0; k < 16; k++) dh[k] = z[k] = 0.f;
        }
        for (int k = 0; k < 16; k++) fdz[tid * 64 + c0 + k] = dh[k] * silu_grad(z[k] + P[kMlpB1 + c0 + k]);
    }
    __syncthreads();
    // dW1[i][o] = sum_r X[r][i] dZ1[r][o] for the 22 real inputs, db1
    for (int e = tid; e < kMlpIn * 64; e += 128) {
        const int i = e / 64, o = e % 64;
        float acc = 0.f;
        for (int r = 0; r < 128; r++) acc += bf16_at(sm + kSmX, r, i, 32) * fdz[r * 64 + o];
        atomicAdd(G + kMlpW1 + i * 64 + o, acc);
    }
    if (tid < 64) {
        float b = 0.f;
        for (int r = 0; r < 128; r++) b += fdz[r * 64 + tid];
        atomicAdd(G + kMlpB1 + tid, b);
    }
    mlp_teardown(c, err);
}

// Adam over the FP32 master parameters; clears the gradients
__global__ void k_mlp_adam(float *P, float *G, float *M, float *V, float lr, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kMlpParams) return;
    const float g = G[i];
    G[i] = 0.f;
    if (!finite_bits(g)) return;
    const float m = 0.9f * M[i] + 0.1f * g, v = 0.999f * V[i] + 0.001f * g * g;
    M[i] = m;
    V[i] = v;
    P[i] -= lr * (m / bc1) / (sqrtf(v / bc2) + 1e-8f);
}

void mlp_pack(const float *P, uint8_t *img, cudaStream_t s) { k_mlp_pack<<<16, 256, 0, s>>>(P, img); }

// The MLP kernels take 124 KB of shared memory, so one CTA holds an SM and
// its 512 tensor-memory columns: allocation never waits on another CTA.
// Set once on each device (function attributes belong to the current device).
static void mlp_attrs() {
    static bool done[64] = {false};
    static std::mutex mu;
    once_per_device(mu, done, []() {   // (a failure stays in cudaGetLastError for the launch check)
        cudaError_t e = cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTrainEnd);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmTrainEnd);
        return e;
    });
}

void mlp_forward(const __nv_bfloat16 *X, int n, const uint8_t *img, const float *P, float2 *out, unsigned *err,
                 cudaStream_t s) {
    if (n <= 0) return;
    mlp_attrs();
    k_mlp_forward<<<(n + 127) / 128, 128, kSmTrainEnd, s>>>(X, n, img, P, out, err);
}

void mlp_train_batch(const __nv_bfloat16 *X, const float2 *T, int n, const uint8_t *img, const float *P, float *G,
                     float *loss, unsigned *err, cudaStream_t s) {
    if (n <= 0) return;
    mlp_attrs();
    k_mlp_train<<<(n + 127) / 128, 128, kSmTrainEnd, s>>>(X, T, n, img, P, G, loss, 1.f / (float)n, err);
}

void mlp_adam(float *P, float *G, float *M, float *V, float lr, int step, cudaStream_t s) {
    const float bc1 = 1.f - powf(0.9f, (float)step), bc2 = 1.f - powf(0.999f, (float)step);
    k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, s>>>(P, G, M, V, lr, bc1, bc2);
}

// ---------------------------------------------------------------------------
// Features and training targets of the learned relocation proposal.
// 22 inputs per Gaussian: mean (3), log-scale (3), unit quaternion (4),
// opacity logit (1), SH DC (3), activity (2: log of the mean |dL/d centre|
// while visible, visible fraction of its life), age (1, in kilo-steps), four
// host-candidate descriptors (sigmoid(opacity), largest scale, distance from
// the scene centre, log(1 + visible steps)) and the screen radius in the
// last view (log).  Inputs 22..31 are zero.
// ---------------------------------------------------------------------------

constexpr float kActScale = 1e5f;   // gradient magnitudes of a normalised loss are ~1e-7..1e-4

__global__ void k_mlp_features(MlpFeatArgs a) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.rows) return;
    const int i = a.idx ? a.idx[r] : r;
    float f[32];
    for (int k = 0; k < 32; k++) f[k] = 0.f;
    for (int k = 0; k < 3; k++) {
        f[k] = a.means[3 * (size_t)i + k];
        f[3 + k] = a.scales[3 * (size_t)i + k];
        f[11 + k] = a.features_dc[3 * (size_t)i + k];
    }
    const float4 q = *reinterpret_cast<const float4 *>(a.quats + 4 * (size_t)i);
    const float qn = rsqrtf(fmaxf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w, 1e-12f));
    f[6] = q.x * qn; f[7] = q.y * qn; f[8] = q.z * qn; f[9] = q.w * qn;
    const float o = a.opacities[i];
    f[10] = o;
    const float4 st = a.gstats ? a.gstats[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    f[14] = log1pf(kActScale * st.x / fmaxf(st.y, 1.f));
    f[15] = st.y / fmaxf(st.z, 1.f);
    f[16] = st.z * 1e-3f;
    f[17] = 1.f / (1.f + __expf(-o));
    f[18] = __expf(fmaxf(fmaxf(f[3], f[4]), f[5]));
    f[19] = sqrtf(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    f[20] = log1pf(st.y);
    f[21] = a.radii ? log1pf((float)max(a.radii[i], 0)) : 0.f;   // screen radius of the last view
    for (int k = 0; k < 32; k++) {
        if (!finite_bits(f[k])) f[k] = 0.f;
        f[k] = fminf(fmaxf(f[k], -64.f), 64.f);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(a.X + (size_t)r * 32);
    for (int k = 0; k < 4; k++) dst[k] = pack8(f + 8 * k);
}

__global__ void k_mlp_snapshot(const int *idx, int S, const float4 *gstats, const float *opacities, float4 *snap) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    float4 st = gstats[idx[s]];
    const float sig = 1.f / (1.f + __expf(-opacities[idx[s]]));
    st.w = finite_bits(sig) ? sig : 0.f;
    snap[s] = st;
}

__global__ void k_mlp_eval(const float2 *pred, const float2 *T, const float4 *snap, int S, float *sums) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    float e[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (s < S) {
        const float2 p = pred[s], t = T[s];
        const float4 then = snap[s];
        const float act_then = then.y > 0.f ? log1pf(kActScale * then.x / then.y) : 0.f;
        const float naive_act = finite_bits(act_then) ? act_then : 0.f;
        e[0] = (p.x - t.x) * (p.x - t.x);
        e[1] = (then.w - t.x) * (then.w - t.x);
        e[2] = (p.y - t.y) * (p.y - t.y);
        e[3] = (naive_act - t.y) * (naive_act - t.y);
        e[4] = 1.f;
    }
#pragma unroll
    for (int k = 0; k < 5; k++) {
        float v = e[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(sums + k, v);
    }
}

__global__ void k_mlp_targets(const int *idx, const float4 *snap, int S, const float *opacities, const float4 *gstats,
                              float2 *T) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const int i = idx[s];
    const float4 now = gstats[i], then = snap[s];
    if (now.z < then.z) {   // the slot was cleared (relocated onto or regrown) since the snapshot
        T[s] = make_float2(0.f, 0.f);
        return;
    }
    const float sig = 1.f / (1.f + __expf(-opacities[i]));
    const float vis = now.y - then.y;
    const float act = vis > 0.f ? log1pf(kActScale * (now.x - then.x) / vis) : 0.f;
    T[s] = make_float2(finite_bits(sig) ? sig : 0.f, finite_bits(act) ? act : 0.f);
}

// sampling weight: predicted opacity a window ahead, raised by predicted activity
__global__ void k_mlp_scores(const float2 *y, int n, float *score) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 v = y[i];
    const float o = fminf(fmaxf(v.x, 0.f), 1.f);
    const float act = fminf(fmaxf(v.y, 0.f), 8.f);
    score[i] = fmaxf(o * (1.f + 0.25f * act), 1e-6f);
}

// Forecast pruning: a Gaussian whose forecast opacity one window ahead is at
// most tau gets an opacity logit of -20, so the relocation round that follows
// classifies it dead (sigmoid <= 0.005) and moves it now.  At most max_n per
// round (counted in *count, zeroed by the caller): a forecast that condemns
// much of the model cannot empty it in one round.
__global__ void k_forecast_prune(const float2 *y, int n, float *opacities, float tau, unsigned *count,
                                 unsigned max_n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (y[i].x <= tau && atomicAdd(count, 1u) < max_n) opacities[i] = -20.f;
}

cudaError_t mlp_forecast_prune(const float2 *y, int n, float *opacities, float tau, unsigned *count, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const cudaError_t e = cudaMemsetAsync(count, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    k_forecast_prune<<<(n + 255) / 256, 256, 0, s>>>(y, n, opacities, tau, count, (unsigned)(n / 20));
    return cudaGetLastError();
}

void mlp_features(const MlpFeatArgs &a, cudaStream_t s) {
    if (a.rows > 0) k_mlp_features<<<(a.rows + 255) / 256, 256, 0, s>>>(a);
}
void mlp_snapshot(const int *idx, int S, const float4 *gstats, const float *opacities, float4 *snap,
                  cudaStream_t s) {
    if (S > 0) k_mlp_snapshot<<<(S + 255) / 256, 256, 0, s>>>(idx, S, gstats, opacities, snap);
}
void mlp_targets(const int *idx, const float4 *snap, int S, const float *opacities, const float4 *gstats, float2 *T,
                 cudaStream_t s) {
    if (S > 0) k_mlp_targets<<<(S + 255) / 256, 256, 0, s>>>(idx, snap, S, opacities, gstats, T);
}
void mlp_eval(const float2 *pred, const float2 *T, const float4 *snap, int S, float *sums, cudaStream_t s) {
    if (S > 0) k_mlp_eval<<<(S + 255) / 256, 256, 0, s>>>(pred, T, snap, S, sums);
}
void mlp_scores(const float2 *y, int n, float *score, cudaStream_t s) {
    if (n > 0) k_mlp_scores<<<(n + 255) / 256, 256, 0, s>>>(y, n, score);
}

}  // namespace msplat


// ---- C ABI of the MLP (device pointers; `stream` is a cudaStream_t or NULL) ----

extern "C" int msplat_mlp_pack(const float *P, uint8_t *img, void *stream) {
    msplat::mlp_pack(P, img, static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int msplat_mlp_forward(const uint16_t *X, int n, const uint8_t *img, const float *P, float *out,
                                  unsigned *err, void *stream) {
    msplat::mlp_forward(reinterpret_cast<const __nv_bfloat16 *>(X), n, img, P, reinterpret_cast<float2 *>(out), err,
                        static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int msplat_mlp_train_batch(const uint16_t *X, const float *T, int n, const uint8_t *img, const float *P,
                                      float *G, float *loss, unsigned *err, void *stream) {
    msplat::mlp_train_batch(reinterpret_cast<const __nv_bfloat16 *>(X), reinterpret_cast<const float2 *>(T), n, img, P,
                            G, loss, err, static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

extern "C" int msplat_mlp_adam(float *P, float *G, float *M, float *V, float lr, int step, void *stream) {
    msplat::mlp_adam(P, G, M, V, lr, step, static_cast<cudaStream_t>(stream));
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

// Self-test of the tensor-core path on host buffers (allocates, runs, copies
// back): D[128 x N] = A[128 x K] * B[N x K]^T with BF16 bit patterns in, F32
// out.  Returns 0, -1 for unsupported N/K, -2 on a CUDA error, -3 when the
// MMA did not complete in time.
extern "C" int msplat_tc_gemm_check(const uint16_t *A, const uint16_t *B, float *D, int N, int K) {
    void *dA = nullptr, *dB = nullptr;
    float *dD = nullptr;
    unsigned *derr = nullptr;
    unsigned herr = 0;
    int rc = 0;
    if ((N != 16 && N != 32 && N != 64) || (K != 16 && K != 32 && K != 64)) return -1;
    if (cudaMalloc(&dA, 128 * K * 2) != cudaSuccess || cudaMalloc(&dB, (size_t)N * K * 2) != cudaSuccess ||
        cudaMalloc(&dD, 128 * (size_t)N * 4) != cudaSuccess || cudaMalloc(&derr, 4) != cudaSuccess) {
        rc = -2;
    } else {
        cudaMemcpy(dA, A, 128 * K * 2, cudaMemcpyHostToDevice);
        cudaMemcpy(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice);
        cudaMemset(derr, 0, 4);
        cudaMemset(dD, 0, 128 * (size_t)N * 4);
        rc = msplat::tc_gemm_probe(dA, dB, dD, N, K, derr, nullptr);
        if (rc == 0 && cudaDeviceSynchronize() != cudaSuccess) rc = -2;
        if (rc == 0) {
            cudaMemcpy(D, dD, 128 * (size_t)N * 4, cudaMemcpyDeviceToHost);
            cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
            if (herr) rc = -3;
        }
    }
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dD);
    cudaFree(derr);
    return rc;
}
