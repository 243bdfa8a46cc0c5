// gs_mlp.h -- the learned residual network: 32 -> 64 -> 64 -> 64 -> 3, SiLU,
// BF16 operands, FP32 accumulation (tcgen05 kernels in k_mlp.cu).
#pragma once

#include "gs_internal.h"

namespace gs {

constexpr int MLP_IN = 32;
constexpr int MLP_H = 64;
constexpr int MLP_OUT = 3;
constexpr int MLP_OUT_PAD = 16;    // last layer padded to the minimum MMA N
constexpr int MLP_TILE = 128;      // samples per tile (MMA M)

// Parameter block (FP32 master copy), contiguous:
//   W1[64][32] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[16][64] b4[16]
// (W4 rows 3..15 and b4[3..15] stay zero).
constexpr int MLP_OFF_W1 = 0;
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H * MLP_H;
constexpr int MLP_OFF_W4 = MLP_OFF_B3 + MLP_H;
constexpr int MLP_OFF_B4 = MLP_OFF_W4 + MLP_OUT_PAD * MLP_H;
constexpr int MLP_NPARAM = MLP_OFF_B4 + MLP_OUT_PAD;

// Forward FLOP per sample (2 per multiply-add, real output width 3).
constexpr double MLP_FLOP_FWD = 2.0 * (MLP_IN * MLP_H + MLP_H * MLP_H * 2 + MLP_H * MLP_OUT);

struct MlpDevice {
    DBuf params;     // float[MLP_NPARAM] master weights
    DBuf grads;      // float[MLP_NPARAM]
    DBuf adam_m, adam_v;
    DBuf loss;       // float[2]: sum of squared error, samples
    DBuf status;     // unsigned
    int adam_t = 0;
    ErrorStatus setup(unsigned long long seed, cudaStream_t s);
    // pred[n][3] = net(feat[n][32]) (FP32 in and out).
    ErrorStatus forward(const float *feat, int n, float *pred, cudaStream_t s);
    // One Adam step on the mean squared error over n samples.
    ErrorStatus train_step(const float *feat, const float *target, int n, float lr,
                           cudaStream_t s);
    // Gradient of the mean squared error into `grads` (added), no update.
    ErrorStatus gradients(const float *feat, const float *target, int n, cudaStream_t s);
    ErrorStatus read_loss(cudaStream_t s, double *mse);   // synchronises
    ErrorStatus check(cudaStream_t s);                    // synchronises
};

}  // namespace gs
