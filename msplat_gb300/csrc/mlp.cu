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

}  // namespace msplat

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
