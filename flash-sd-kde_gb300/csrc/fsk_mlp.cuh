// fsk_mlp.cuh - surrogate MLP: parameter layout and launchers.
#pragma once
#include "fsk_common.cuh"

namespace fsk {
namespace mlp {

constexpr int MLP_IN = 16;
constexpr int MLP_H = 256;
// FP32 parameters of one ensemble member, contiguous:
// W1 [256][16] b1 [256] W2 [256][256] b2 [256] W3 [256][256] b3 [256] w4 [256] b4
constexpr int64_t OFF_W1 = 0;
constexpr int64_t OFF_B1 = OFF_W1 + MLP_H * MLP_IN;
constexpr int64_t OFF_W2 = OFF_B1 + MLP_H;
constexpr int64_t OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int64_t OFF_W3 = OFF_B2 + MLP_H;
constexpr int64_t OFF_B3 = OFF_W3 + MLP_H * MLP_H;
constexpr int64_t OFF_W4 = OFF_B3 + MLP_H;
constexpr int64_t OFF_B4 = OFF_W4 + MLP_H;
constexpr int64_t MLP_PARAMS = OFF_B4 + 1;   // 136193
static_assert(MLP_PARAMS == 136193, "parameter layout");

// Activations kept between the training forward and backward (caller workspace).
struct TrainBufs {
  float* a0;       // [batch][16]
  float* z[3];     // [members][batch][256] pre-activations (overwritten by dz in backward)
  float* a[3];     // [members][batch][256] bf16-exact activations
  float* da;       // [members][batch][256] dz of the last hidden layer
};

TrainBufs carve_train(WsCarver& c, int members, int64_t batch);
void launch_forward(const float* params, int members, const float* x, int64_t batch, const float* in_mean,
                    const float* in_inv_std, const TrainBufs& t, float* y, cudaStream_t s);
void launch_backward(const float* params, int members, int64_t batch, const TrainBufs& t, const float* dy,
                     float* grads, cudaStream_t s);
void launch_mse(const float* y, const float* target, int64_t batch, int members, float* dy, double* loss,
                cudaStream_t s);
void launch_adam(float* p, const float* g, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
                 float eps, float wd, int step, cudaStream_t s);

// Tensor-core inference (fsk_mlp_tc.cu).
size_t packed_bytes(int members);
int launch_pack(const float* params, int members, const float* in_mean, const float* in_inv_std, float out_scale,
                float out_shift, void* packed, cudaStream_t s);
int launch_infer(const void* packed, int members, const float* x, int64_t batch, float* y, cudaStream_t s);
void launch_combine(const float* y, int members, int64_t batch, const float* x, const float* in_mean,
                    const float* in_inv_std, float base_a, float base_b, float spread_tol, float r2_max, float* mean,
                    float* spread, uint8_t* served, cudaStream_t s);

}  // namespace mlp
}  // namespace fsk
