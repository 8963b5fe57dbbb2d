// Host-side interface of the learned relocation proposal (mlp.cu): the
// MLP's parameter layout, its operand images, and the launchers.  Safe to
// include from host-only translation units.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace msplat {

// FP32 master parameters, flat: W1 [32][64] (rows past kMlpIn unused), b1 [64],
// W2 [64][64], b2 [64], W3 [64][16] (columns past 2 unused), b3 [16]
constexpr int kMlpIn = 22;
constexpr int kMlpW1 = 0, kMlpB1 = 2048, kMlpW2 = 2112, kMlpB2 = 6208, kMlpW3 = 6272, kMlpB3 = 7296;
constexpr int kMlpParams = 7312;
// BF16 operand images (bytes): forward W1t, W2t, W3t; backward W2b, W3b
constexpr int kImgW1t = 0, kImgW2t = 4096, kImgW3t = 12288, kImgW2b = 14336, kImgW3b = 22528, kImgBytes = 24576;
void mlp_pack(const float *P, uint8_t *img, cudaStream_t s);
void mlp_forward(const __nv_bfloat16 *X, int n, const uint8_t *img, const float *P, float2 *out, unsigned *err,
                 cudaStream_t s);
void mlp_train_batch(const __nv_bfloat16 *X, const float2 *T, int n, const uint8_t *img, const float *P, float *G,
                     float *loss, unsigned *err, cudaStream_t s);
void mlp_adam(float *P, float *G, float *M, float *V, float lr, int step, cudaStream_t s);
struct MlpFeatArgs {
    int rows;                       // rows of X to fill
    const int *idx;                 // Gaussian of each row, or null for row = Gaussian
    const float *means, *scales, *quats, *features_dc, *opacities;
    const float4 *gstats;
    const int *radii;               // last step's screen radii, or null
    __nv_bfloat16 *X;               // [rows, 32]
};
void mlp_features(const MlpFeatArgs &a, cudaStream_t s);
// targets of the samples taken at a snapshot: (sigmoid(opacity), log activity)
// now, or (0, 0) when the slot was relocated or regrown since
void mlp_targets(const int *idx, const float4 *snap, int S, const float *opacities, const float4 *gstats,
                 float2 *T, cudaStream_t s);
// the sampled Gaussians' activity statistics, w = sigmoid(opacity), at the snapshot
void mlp_snapshot(const int *idx, int S, const float4 *gstats, const float *opacities, float4 *snap,
                  cudaStream_t s);
// Held-out check of a round's predictions before training on its labels:
// adds to sums[0..4] the squared errors of the MLP (opacity, activity), of the
// persistence forecast (the snapshot's own opacity and mean activity) and the
// sample count
void mlp_eval(const float2 *pred, const float2 *T, const float4 *snap, int S, float *sums, cudaStream_t s);
// sampling weights from the MLP outputs
void mlp_scores(const float2 *y, int n, float *score, cudaStream_t s);
// forecast pruning: the logit of each Gaussian whose forecast opacity is at
// most tau becomes -20 (at most n / 20 of them); returns the launch status
cudaError_t mlp_forecast_prune(const float2 *y, int n, float *opacities, float tau, unsigned *count, cudaStream_t s);

}  // namespace msplat
