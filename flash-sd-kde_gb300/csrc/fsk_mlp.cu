// fsk_mlp.cu - training kernels of the learned surrogate: an ensemble of
// MLPs 16 -> 256 -> 256 -> 256 -> 1 with SiLU, bf16 weights and activations,
// FP32 accumulation (the model of the tensor-core inference kernel in
// fsk_mlp_tc.cu), trained on (query, exact log-density) pairs.
//
// Forward (per member, batch rows b):
//   a0 = bf16((x - in_mean) * in_inv_std)
//   z_l = bf16(W_l) a_{l-1} + b_l,  a_l = bf16(silu(z_l))   l = 1..3
//   y = bf16(w4) . a3 + b4
// Backward treats the bf16 roundings as identity (straight-through);
// weight gradients are FP32 with split-batch atomics.  AdamW with bias
// correction.  The GEMMs run on CUDA cores (a batched 64x64x16 SIMT tile):
// training is a small part of the surrogate's cost; the inference path is
// the tensor-core kernel.
#include "fsk_kernels.cuh"
#include "fsk_mlp.cuh"

namespace fsk {
namespace mlp {

namespace {

__device__ __forceinline__ float bf16r(float v) {   // round to nearest bf16 (ties to even), as FP32
  const uint32_t u = __float_as_uint(v);
  if ((u & 0x7F800000u) == 0x7F800000u) return v;  // inf / nan unchanged
  const uint32_t r = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  return __uint_as_float(r);
}

// SiLU through tanh.approx, the same arithmetic as the inference kernel:
// silu(z) = h + h tanh(h), h = z / 2; sigmoid(z) = (1 + tanh(h)) / 2.
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float silu(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_approx(h), h);
}
__device__ __forceinline__ float silu_grad(float z) {
  const float s = fmaf(0.5f, tanh_approx(0.5f * z), 0.5f);
  return s * (1.0f + z * (1.0f - s));
}

enum Epi { EPI_FWD = 0, EPI_DGRAD = 1, EPI_ATOMIC = 2 };

struct GemmArgs {
  const float* A;      // opA (M x K)
  const float* B;      // opB (K x N)
  int64_t lda, ldb;    // leading dimensions of the stored arrays
  int64_t sA, sB;      // per-member strides (0: shared)
  int M, N, K;
  int k_chunk;         // split-K chunk (multiple of 16); gridDim.z = members * splits
  int splits;
  int round_b;         // round B elements to bf16 (weights)
  // epilogue
  float* C;  int64_t ldc, sC;          // FWD: z, DGRAD: dz, ATOMIC: grad (accumulated)
  const float* bias; int64_t sBias;    // FWD
  float* Anext; int64_t sAnext;        // FWD: bf16(silu(z)), same layout as C
  const float* Zprev; int64_t sZ;      // DGRAD: z of the layer below, same layout as C
};

constexpr int BM = 64, BN = 64, BK = 16;

// C[m][n] = sum_k opA[m][k] opB[k][n], 256 threads, 4x4 per thread.
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) gemm_kernel(GemmArgs g) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  const int member = blockIdx.z / g.splits;
  const int split = blockIdx.z % g.splits;
  const float* A = g.A + member * g.sA;
  const float* B = g.B + member * g.sB;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int k_begin = split * g.k_chunk;
  const int k_end = min(g.K, k_begin + g.k_chunk);
  const int t = threadIdx.x;
  const int tx = t & 15, ty = t >> 4;
  float acc[4][4] = {};
  for (int k0 = k_begin; k0 < k_end; k0 += BK) {
    // A tile: BM x BK elements, 4 per thread
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int e = t + i * 256;
      int mm, kk;
      if (TA) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < g.M && k < k_end) v = TA ? A[(int64_t)k * g.lda + m] : A[(int64_t)m * g.lda + k];
      As[kk][mm] = v;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int e = t + i * 256;
      int nn, kk;
      if (TB) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      const int n = n0 + nn, k = k0 + kk;
      float v = 0.f;
      if (n < g.N && k < k_end) v = TB ? B[(int64_t)n * g.ldb + k] : B[(int64_t)k * g.ldb + n];
      Bs[kk][nn] = g.round_b ? bf16r(v) : v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n >= g.N) continue;
      const int64_t o = (int64_t)m * g.ldc + n;
      if (EPI == EPI_FWD) {
        const float z = acc[i][j] + g.bias[member * g.sBias + n];
        g.C[member * g.sC + o] = z;
        g.Anext[member * g.sAnext + o] = bf16r(silu(z));
      } else if (EPI == EPI_DGRAD) {
        g.C[member * g.sC + o] = acc[i][j] * silu_grad(g.Zprev[member * g.sZ + o]);
      } else {
        atomicAdd(&g.C[member * g.sC + o], acc[i][j]);
      }
    }
  }
}

template <bool TA, bool TB, int EPI>
void gemm(const GemmArgs& g, int members, cudaStream_t s) {
  dim3 grid((unsigned)((g.N + BN - 1) / BN), (unsigned)((g.M + BM - 1) / BM), (unsigned)(members * g.splits));
  gemm_kernel<TA, TB, EPI><<<grid, 256, 0, s>>>(g);
  count_launch();
}

// a0 = bf16((x - mean) * inv_std), shared by all members.
__global__ void input_kernel(const float* __restrict__ x, int64_t batch, const float* __restrict__ mean,
                             const float* __restrict__ inv_std, float* __restrict__ a0) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= batch * MLP_IN) return;
  const int k = (int)(e % MLP_IN);
  a0[e] = bf16r((x[e] - mean[k]) * inv_std[k]);
}

// y[member][b] = bf16(w4) . a3[b] + b4, one warp per (member, row).
__global__ void output_kernel(const float* __restrict__ params, const float* __restrict__ a3, int64_t batch,
                              int members, float* __restrict__ y) {
  const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= batch * members) return;
  const int member = (int)(wid / batch);
  const int64_t b = wid % batch;
  const float* w4 = params + (int64_t)member * MLP_PARAMS + OFF_W4;
  const float* row = a3 + ((int64_t)member * batch + b) * MLP_H;
  float s = 0.f;
  for (int k = lane; k < MLP_H; k += 32) s = fmaf(bf16r(w4[k]), row[k], s);
#pragma unroll
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[wid] = s + params[(int64_t)member * MLP_PARAMS + OFF_B4];
}

// Output layer backward: grads of w4 (atomics over rows), b4, and
// dz3[b][k] = dy[b] bf16(w4[k]) silu'(z3[b][k]).
__global__ void output_bwd_kernel(const float* __restrict__ params, const float* __restrict__ a3,
                                  const float* __restrict__ z3, const float* __restrict__ dy, int64_t batch,
                                  int members, float* __restrict__ dz3, float* __restrict__ grads) {
  const int member = blockIdx.y;
  const int k = threadIdx.x;               // 256 threads = features
  const int64_t rows_per_block = (batch + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * rows_per_block, b1 = min(batch, b0 + rows_per_block);
  const float w = bf16r(params[(int64_t)member * MLP_PARAMS + OFF_W4 + k]);
  float gw = 0.f, gb = 0.f;
  for (int64_t b = b0; b < b1; ++b) {
    const int64_t r = (int64_t)member * batch + b;
    const float d = dy[r];
    gw = fmaf(d, a3[r * MLP_H + k], gw);
    gb += d;
    dz3[r * MLP_H + k] = d * w * silu_grad(z3[r * MLP_H + k]);
  }
  atomicAdd(&grads[(int64_t)member * MLP_PARAMS + OFF_W4 + k], gw);
  if (k == 0) atomicAdd(&grads[(int64_t)member * MLP_PARAMS + OFF_B4], gb);
}

// bias gradient: grads[off + n] += sum_b dz[b][n]
__global__ void bias_grad_kernel(const float* __restrict__ dz, int64_t batch, int members, int64_t off,
                                 float* __restrict__ grads) {
  const int member = blockIdx.y;
  const int n = threadIdx.x;  // 256
  const int64_t rows_per_block = (batch + gridDim.x - 1) / gridDim.x;
  const int64_t b0 = blockIdx.x * rows_per_block, b1 = min(batch, b0 + rows_per_block);
  float s = 0.f;
  for (int64_t b = b0; b < b1; ++b) s += dz[((int64_t)member * batch + b) * MLP_H + n];
  atomicAdd(&grads[(int64_t)member * MLP_PARAMS + off + n], s);
}

__global__ void zero_kernel(float* p, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0.f;
}

__global__ void mse_kernel(const float* __restrict__ y, const float* __restrict__ target, int64_t batch,
                           int members, float* __restrict__ dy, double* __restrict__ loss) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < batch * members) {
    const float r = y[i] - target[i % batch];
    dy[i] = 2.0f * r / (float)batch;
    l = (double)r * r;
  }
  if (loss) {
#pragma unroll
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0) atomicAdd(loss, l / (double)batch);
  }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, int64_t count, float lr, float beta1, float beta2, float eps,
                            float wd, float bc1, float bc2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float gi = g[i];
  const float mi = fmaf(beta1, m[i], (1.0f - beta1) * gi);
  const float vi = fmaf(beta2, v[i], (1.0f - beta2) * gi * gi);
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / bc1, vh = vi / bc2;
  p[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * p[i]);
}

}  // namespace

TrainBufs carve_train(WsCarver& c, int members, int64_t batch) {
  TrainBufs t;
  t.a0 = c.take<float>((size_t)batch * MLP_IN);
  const size_t act = (size_t)members * batch * MLP_H;
  for (int l = 0; l < 3; ++l) {
    t.z[l] = c.take<float>(act);
    t.a[l] = c.take<float>(act);
  }
  t.da = c.take<float>(act);
  return t;
}

void launch_forward(const float* params, int members, const float* x, int64_t batch, const float* in_mean,
                    const float* in_inv_std, const TrainBufs& t, float* y, cudaStream_t s) {
  const int64_t ne = batch * MLP_IN;
  input_kernel<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(x, batch, in_mean, in_inv_std, t.a0);
  count_launch();
  const int64_t act = batch * MLP_H;
  const int64_t w_off[3] = {OFF_W1, OFF_W2, OFF_W3}, b_off[3] = {OFF_B1, OFF_B2, OFF_B3};
  for (int l = 0; l < 3; ++l) {
    GemmArgs g{};
    g.A = l == 0 ? t.a0 : t.a[l - 1];
    g.lda = l == 0 ? MLP_IN : MLP_H;
    g.sA = l == 0 ? 0 : act;
    g.B = params + w_off[l];
    g.ldb = l == 0 ? MLP_IN : MLP_H;
    g.sB = MLP_PARAMS;
    g.M = (int)batch;
    g.N = MLP_H;
    g.K = l == 0 ? MLP_IN : MLP_H;
    g.k_chunk = g.K;
    g.splits = 1;
    g.round_b = 1;
    g.C = t.z[l];
    g.ldc = MLP_H;
    g.sC = act;
    g.bias = params + b_off[l];
    g.sBias = MLP_PARAMS;
    g.Anext = t.a[l];
    g.sAnext = act;
    gemm<false, true, EPI_FWD>(g, members, s);
  }
  const int64_t warps = batch * members;
  output_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(params, t.a[2], batch, members, y);
  count_launch();
}

void launch_backward(const float* params, int members, int64_t batch, const TrainBufs& t, const float* dy,
                     float* grads, cudaStream_t s) {
  const int64_t total = (int64_t)members * MLP_PARAMS;
  zero_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(grads, total);
  count_launch();
  const int64_t act = batch * MLP_H;
  const int row_blocks = (int)imin<int64_t>(512, (batch + 63) / 64);
  // output layer -> dz3 (stored in da)
  output_bwd_kernel<<<dim3((unsigned)row_blocks, (unsigned)members), MLP_H, 0, s>>>(params, t.a[2], t.z[2], dy,
                                                                                     batch, members, t.da, grads);
  count_launch();
  const int64_t w_off[3] = {OFF_W1, OFF_W2, OFF_W3}, b_off[3] = {OFF_B1, OFF_B2, OFF_B3};
  float* dz = t.da;   // dz of layer l lives in t.da (l = 3) or in t.z[l] (overwritten, l < 3)
  for (int l = 2; l >= 0; --l) {
    // weight gradient: dW_l[o][k] = sum_b dz[b][o] a_{l-1}[b][k], split over the batch
    GemmArgs g{};
    g.A = dz;
    g.lda = MLP_H;
    g.sA = act;
    g.B = l == 0 ? t.a0 : t.a[l - 1];
    g.ldb = l == 0 ? MLP_IN : MLP_H;
    g.sB = l == 0 ? 0 : act;
    g.M = MLP_H;
    g.N = l == 0 ? MLP_IN : MLP_H;
    g.K = (int)batch;
    g.splits = (int)imax<int64_t>(1, imin<int64_t>(64, batch / 256));
    g.k_chunk = (int)(((batch + g.splits - 1) / g.splits + BK - 1) / BK * BK);
    g.splits = (int)((batch + g.k_chunk - 1) / g.k_chunk);
    g.round_b = 0;
    g.C = grads + w_off[l];
    g.ldc = g.N;
    g.sC = MLP_PARAMS;
    gemm<true, false, EPI_ATOMIC>(g, members, s);
    bias_grad_kernel<<<dim3((unsigned)row_blocks, (unsigned)members), MLP_H, 0, s>>>(dz, batch, members, b_off[l],
                                                                                    grads);
    count_launch();
    if (l == 0) break;
    // data gradient into the layer below: dz_{l-1} = (dz W_l) * silu'(z_{l-1}), written over z_{l-1}
    GemmArgs d{};
    d.A = dz;
    d.lda = MLP_H;
    d.sA = act;
    d.B = params + w_off[l];
    d.ldb = MLP_H;
    d.sB = MLP_PARAMS;
    d.M = (int)batch;
    d.N = MLP_H;
    d.K = MLP_H;
    d.k_chunk = MLP_H;
    d.splits = 1;
    d.round_b = 1;
    d.C = t.z[l - 1];
    d.ldc = MLP_H;
    d.sC = act;
    d.Zprev = t.z[l - 1];
    d.sZ = act;
    gemm<false, false, EPI_DGRAD>(d, members, s);
    dz = t.z[l - 1];
  }
}

void launch_mse(const float* y, const float* target, int64_t batch, int members, float* dy, double* loss,
                cudaStream_t s) {
  const int64_t n = batch * members;
  mse_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(y, target, batch, members, dy, loss);
  count_launch();
}

void launch_adam(float* p, const float* g, float* m, float* v, int64_t count, float lr, float beta1, float beta2,
                 float eps, float wd, int step, cudaStream_t s) {
  const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(p, g, m, v, count, lr, beta1, beta2, eps, wd, bc1, bc2);
  count_launch();
}

}  // namespace mlp
}  // namespace fsk
