// fsk_mlp_tc.cu - tensor-core (tcgen05 / TMEM) inference of the surrogate
// MLP ensemble: 16 -> 256 -> 256 -> 256 -> 1, SiLU, bf16 weights and
// activations, FP32 accumulation, one ensemble member per CTA.
//
// Per tile of 128 queries (one TMEM lane each):
//   A0 = bf16((x - mean) * inv_std)         epilogue warps -> TMEM cols 256..263
//   D  = A0 . W1^T                           1 MMA, M=128, N=256, K=16
//   A1 = bf16(silu(D + b1))                  TMEM -> registers -> TMEM cols 256..383
//   D  = A1 . W2^T                           16 MMAs (K steps), N=256
//   A2 = bf16(silu(D + b2)); D = A2 . W3^T   16 MMAs
//   y  = bf16(silu(D + b3)) . bf16(w4) + b4  per-thread dot, four feature quarters combined
// The activations stay in tensor memory as the A operand of the next layer
// (tcgen05.mma with A in TMEM), so nothing is transposed through shared
// memory.  W2 and W3 (128 KB each in bf16) do not fit in shared memory next
// to anything else, so they stream from L2 as 8 KB K slices ([256 out][16 in],
// core-matrix K-major) through a ring of RING slots; W1, the biases, w4 and
// the input normalisation are loaded once per CTA.
//
// Warps: 0-15 epilogue (warp w: TMEM lane quarter w&3, feature quarter
// w>>2), 16 producer (bulk copies), 17 MMA issue + TMEM owner.
#include <cuda_bf16.h>

#include "fsk_kernels.cuh"
#include "fsk_mlp.cuh"
#include "fsk_tc.cuh"
#include "fsk_tc_ops.cuh"

namespace fsk {
namespace mlp {

namespace {

constexpr int QT = 128;                         // queries per tile
constexpr int SLICE_BYTES = MLP_H * 16 * 2;     // one K slice: [256][16] bf16 = 8 KB
constexpr int N_SLICES = MLP_H / 16;            // 16 per hidden layer
constexpr int RING = 24;                        // slices in flight: hides L2 latency across layers
// packed member image (global):
//   header 256 B: in_mean[16] in_inv_std[16] out_scale out_shift b4 (FP32)
//   b1 b2 b3 w4 (FP32, w4 bf16-rounded) 4 KB
//   W1 image [256][16] bf16 8 KB, W2 slices 16 x 8 KB, W3 slices 16 x 8 KB
constexpr int HDR_BYTES = 256;
constexpr int VEC_BYTES = 4 * MLP_H * 4;
constexpr int W1_OFF = HDR_BYTES + VEC_BYTES;
constexpr int W2_OFF = W1_OFF + SLICE_BYTES;
constexpr int W3_OFF = W2_OFF + N_SLICES * SLICE_BYTES;
constexpr int MEMBER_BYTES = W3_OFF + N_SLICES * SLICE_BYTES;
// shared memory
constexpr int SM_CONST_BYTES = W2_OFF;                     // header + vectors + W1 image (one copy)
constexpr int SM_RING_OFF = SM_CONST_BYTES;
constexpr int SM_YSUM_OFF = SM_RING_OFF + RING * SLICE_BYTES;
constexpr int SM_BAR_OFF = SM_YSUM_OFF + 3 * QT * 4;
constexpr int N_BARS = 5 + 2 * RING;             // cready, full/empty ring, aready, dfull, ycomb, drain
constexpr int SMEM_BYTES = SM_BAR_OFF + (N_BARS + 1) * 8;   // + the TMEM address slot
constexpr int EPI_WARPS = 16;
constexpr int PROD_WARP = 16;
constexpr int MMA_WARP = 17;
constexpr int THREADS = 18 * 32;
constexpr int T_D = 0;       // accumulator: 256 FP32 columns
constexpr int T_A = 256;     // activations: 128 columns of packed bf16 pairs
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory");
static_assert(MEMBER_BYTES % 16 == 0 && W1_OFF % 16 == 0, "bulk copy alignment");

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  return (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(a)) |
         ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(b)) << 16);
}

__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// silu(z) = z sigmoid(z) = 0.5 z (1 + tanh(z / 2))
__device__ __forceinline__ float silu_fast(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_approx(h), h);
}

struct InferParams {
  const uint8_t* packed;
  int members;
  const float* x;
  int64_t batch;
  float* y;            // [members][batch]
  int64_t tiles;
};

__global__ void __launch_bounds__(THREADS, 1) mlp_infer_kernel(InferParams p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const float* hdr = reinterpret_cast<const float*>(smem);
  const float* vec = reinterpret_cast<const float*>(smem + HDR_BYTES);   // b1 b2 b3 w4
  uint8_t* ring = smem + SM_RING_OFF;
  float* ysum = reinterpret_cast<float*>(smem + SM_YSUM_OFF);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SM_BAR_OFF);
  uint64_t* cready = bars;               // constants loaded
  uint64_t* full = bars + 1;             // [RING]
  uint64_t* empty = bars + 1 + RING;     // [RING]
  uint64_t* aready = bars + 1 + 2 * RING;  // activations (or inputs) stored, all epilogue warps
  uint64_t* dfull = bars + 2 + 2 * RING;   // layer accumulator complete
  uint64_t* ycomb = bars + 3 + 2 * RING;   // partial dots of feature quarters 1-3 stored, 12 warps
  uint64_t* drain = bars + 4 + 2 * RING;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 5 + 2 * RING);
  int64_t n_ring_copies = 0;
  int n_const_copies = 0;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int member = blockIdx.x % p.members;
  const int group = blockIdx.x / p.members, groups = gridDim.x / p.members;
  const uint8_t* img = p.packed + (int64_t)member * MEMBER_BYTES;

  if (threadIdx.x == 0) {
    mbar_init(cready, 1);
    for (int i = 0; i < RING; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(aready, EPI_WARPS);
    mbar_init(dfull, 1);
    mbar_init(ycomb, 12);
    mbar_init(drain, 1);
    fence_barrier_init();
  }
  if (warp == MMA_WARP) {
    tmem_alloc(tmem_slot, 512);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == PROD_WARP) {
    if (lane == 0) {
      mbar_arrive_expect_tx(cready, SM_CONST_BYTES);
      bulk_g2s(smem, img, SM_CONST_BYTES, cready);
      n_const_copies = 1;
      int64_t g = 0;
      for (int64_t t = group; t < p.tiles; t += groups) {
        for (int sl = 0; sl < 2 * N_SLICES; ++sl, ++g) {
          const int s = (int)(g % RING);
          if (!mbar_wait(&empty[s], (uint32_t)(((g / RING) & 1) ^ 1), 51)) goto done;
          mbar_arrive_expect_tx(&full[s], SLICE_BYTES);
          bulk_g2s(ring + s * SLICE_BYTES, img + W2_OFF + sl * SLICE_BYTES, SLICE_BYTES, &full[s]);
          n_ring_copies = g + 1;
        }
      }
    }
  } else if (warp == MMA_WARP) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_f32(QT, MLP_H);
      const uint64_t w1d = smem_desc_kmajor(smem_u32(smem + W1_OFF), 128, 8 * 32);
      const uint64_t r0 = smem_desc_kmajor(smem_u32(ring), 128, 8 * 32);
      if (!mbar_wait(cready, 0, 52)) goto done;
      int64_t g = 0;
      int k = 0;   // layer phases completed (aready / dfull parity)
      for (int64_t t = group; t < p.tiles; t += groups) {
        // layer 1: inputs stored by the epilogue
        if (!mbar_wait(aready, (uint32_t)(k & 1), 53)) goto done;
        tc_fence_after();
        mma_f16_ts(tmem + T_D, tmem + T_A, w1d, idesc, 0u);
        mma_commit(dfull);
        ++k;
        for (int layer = 0; layer < 2; ++layer) {
          if (!mbar_wait(aready, (uint32_t)(k & 1), 54)) goto done;
          tc_fence_after();
          for (int ks = 0; ks < N_SLICES; ++ks, ++g) {
            const int s = (int)(g % RING);
            if (!mbar_wait(&full[s], (uint32_t)((g / RING) & 1), 55)) goto done;
            tc_fence_after();
            mma_f16_ts(tmem + T_D, tmem + T_A + 8 * ks, r0 + (uint64_t)((s * SLICE_BYTES) >> 4), idesc,
                           ks ? 1u : 0u);
            mma_commit(&empty[s]);
          }
          mma_commit(dfull);
          ++k;
        }
      }
    }
  } else {
    // ---------------- epilogue: thread = one query, one feature quarter ----------------
    const int quarter = warp & 3, fq = warp >> 2;   // TMEM lane quarter, feature quarter (64 features)
    const int row = quarter * 32 + lane;
    const uint32_t lane_off = (uint32_t)(quarter * 32) << 16;
    if (!mbar_wait(cready, 0, 56)) goto done;
    const float* mean = hdr;
    const float* inv_std = hdr + 16;
    const float out_scale = hdr[32], out_shift = hdr[33], b4 = hdr[34];
    int k = 0;
    // this thread's 4 input features of a tile (features 4 fq .. 4 fq + 3);
    // the next tile's are loaded while the current one runs
    auto load_x = [&](int64_t tile) {
      const int64_t qq = tile * QT + row;
      if (tile < p.tiles && qq < p.batch) return __ldg(reinterpret_cast<const float4*>(p.x + qq * MLP_IN + 4 * fq));
      return make_float4(mean[4 * fq], mean[4 * fq + 1], mean[4 * fq + 2], mean[4 * fq + 3]);
    };
    float4 xv = load_x(group);
    for (int64_t t = group; t < p.tiles; t += groups) {
      const int64_t q = t * QT + row;
      {
        const float4 v = xv;
        xv = load_x(t + groups);
        const int f = 4 * fq;
        uint32_t pk[2];
        pk[0] = pack_bf16((v.x - mean[f]) * inv_std[f], (v.y - mean[f + 1]) * inv_std[f + 1]);
        pk[1] = pack_bf16((v.z - mean[f + 2]) * inv_std[f + 2], (v.w - mean[f + 3]) * inv_std[f + 3]);
        tmem_st2(tmem + lane_off + T_A + 2 * fq, pk);
        tmem_st_wait();
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(aready);
      }
      float acc_y = 0.f;
      for (int layer = 0; layer < 3; ++layer) {
        if (!mbar_wait(dfull, (uint32_t)(k & 1), 57)) goto done;
        tc_fence_after();
        ++k;
        const float* bias = vec + layer * MLP_H + 64 * fq;
        const float* w4 = vec + 3 * MLP_H + 64 * fq;
#pragma unroll 1
        for (int c = 0; c < 2; ++c) {
          uint32_t r[32];
          tmem_ld32(tmem + lane_off + T_D + 64 * fq + 32 * c, r);
          tmem_ld_wait();
          if (layer < 2) {
            uint32_t pk[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const float2 bb = *reinterpret_cast<const float2*>(bias + 32 * c + 2 * j);
              pk[j] = pack_bf16(silu_fast(__uint_as_float(r[2 * j]) + bb.x), silu_fast(__uint_as_float(r[2 * j + 1]) + bb.y));
            }
            tmem_st16(tmem + lane_off + T_A + 32 * fq + 16 * c, pk);
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float a = __bfloat162float(__float2bfloat16_rn(silu_fast(__uint_as_float(r[j]) + bias[32 * c + j])));
              acc_y = fmaf(a, w4[32 * c + j], acc_y);
            }
          }
        }
        if (layer < 2) {
          tmem_st_wait();
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(aready);
        }
      }
      // combine the four feature quarters of each query's dot product
      tc_fence_before();
      if (fq != 0) {
        ysum[(fq - 1) * QT + row] = acc_y;
        __syncwarp();
        if (lane == 0) mbar_arrive(ycomb);
      } else {
        const int kt = (int)((t - group) / groups);
        if (!mbar_wait(ycomb, (uint32_t)(kt & 1), 58)) goto done;
        const float v = acc_y + ysum[row] + ysum[QT + row] + ysum[2 * QT + row] + b4;
        if (q < p.batch) p.y[(int64_t)member * p.batch + q] = fmaf(v, out_scale, out_shift);
      }
    }
  }
done:
  if (warp == PROD_WARP && lane == 0) {
    for (int64_t i = imax<int64_t>(0, n_ring_copies - RING); i < n_ring_copies; ++i)
      mbar_wait(&full[i % RING], (uint32_t)((i / RING) & 1), 59);
    if (n_const_copies) mbar_wait(cready, 0, 60);
  }
  if (warp == MMA_WARP && lane == 0) {
    mma_commit(drain);
    mbar_wait(drain, 0, 61);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == MMA_WARP) tmem_dealloc(tmem, 512);
}

// ---- packing: FP32 member parameters -> the image above -------------------------
__device__ __forceinline__ void put_bf16(uint8_t* img, int r, int k, float v) {
  // [256 rows][16 K] core-matrix K-major, 32-byte rows
  const uint32_t off = (uint32_t)(r >> 3) * 256u + (uint32_t)(k >> 3) * 128u + (uint32_t)(r & 7) * 16u +
                       (uint32_t)(k & 7) * 2u;
  *reinterpret_cast<__nv_bfloat16*>(img + off) = __float2bfloat16_rn(v);
}

__global__ void pack_kernel(const float* __restrict__ params, int members, const float* __restrict__ in_mean,
                            const float* __restrict__ in_inv_std, float out_scale, float out_shift,
                            uint8_t* __restrict__ packed) {
  const int member = blockIdx.y;
  const float* P = params + (int64_t)member * MLP_PARAMS;
  uint8_t* img = packed + (int64_t)member * MEMBER_BYTES;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float* hdr = reinterpret_cast<float*>(img);
  float* vec = reinterpret_cast<float*>(img + HDR_BYTES);
  if (i < 64) {
    float v = 0.f;
    if (i < 16) v = in_mean[i];
    else if (i < 32) v = in_inv_std[i - 16];
    else if (i == 32) v = out_scale;
    else if (i == 33) v = out_shift;
    else if (i == 34) v = P[OFF_B4];
    hdr[i] = v;
  }
  if (i < MLP_H) {
    vec[i] = P[OFF_B1 + i];
    vec[MLP_H + i] = P[OFF_B2 + i];
    vec[2 * MLP_H + i] = P[OFF_B3 + i];
    vec[3 * MLP_H + i] = __bfloat162float(__float2bfloat16_rn(P[OFF_W4 + i]));
  }
  if (i < MLP_H * MLP_IN) {
    const int r = (int)(i / MLP_IN), kk = (int)(i % MLP_IN);
    put_bf16(img + W1_OFF, r, kk, P[OFF_W1 + i]);
  }
  if (i < MLP_H * MLP_H) {
    const int r = (int)(i / MLP_H), kk = (int)(i % MLP_H);
    const int sl = kk / 16, kin = kk % 16;
    put_bf16(img + W2_OFF + sl * SLICE_BYTES, r, kin, P[OFF_W2 + i]);
    put_bf16(img + W3_OFF + sl * SLICE_BYTES, r, kin, P[OFF_W3 + i]);
  }
}

// Ensemble statistics and the serving gate, per query b:
//   r2 = |(x_b - mean) * inv_std|^2 (whitened radius, if x is given)
//   mean[b] = average over members of y + base_a + base_b r2
//   spread[b] = max - min over members
//   served[b] = spread <= spread_tol and r2 <= r2_max
__global__ void combine_kernel(const float* __restrict__ y, int members, int64_t batch, const float* __restrict__ x,
                               const float* __restrict__ in_mean, const float* __restrict__ in_inv_std, float base_a,
                               float base_b, float spread_tol, float r2_max, float* __restrict__ mean,
                               float* __restrict__ spread, uint8_t* __restrict__ served) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= batch) return;
  float s = 0.f, lo = INFINITY, hi = -INFINITY;
  for (int m = 0; m < members; ++m) {
    const float v = y[(int64_t)m * batch + b];
    s += v;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  float r2 = 0.f;
  if (x) {
#pragma unroll
    for (int k = 0; k < MLP_IN; ++k) {
      const float u = (x[b * MLP_IN + k] - in_mean[k]) * in_inv_std[k];
      r2 = fmaf(u, u, r2);
    }
  }
  const float sp = hi - lo;
  if (mean) mean[b] = s / (float)members + base_a + base_b * r2;
  if (spread) spread[b] = sp;
  if (served) served[b] = (sp <= spread_tol && r2 <= r2_max) ? 1 : 0;
}

}  // namespace

size_t packed_bytes(int members) { return (size_t)members * MEMBER_BYTES; }

int launch_pack(const float* params, int members, const float* in_mean, const float* in_inv_std, float out_scale,
                float out_shift, void* packed, cudaStream_t s) {
  const int64_t n = (int64_t)MLP_H * MLP_H;
  pack_kernel<<<dim3((unsigned)((n + 255) / 256), (unsigned)members), 256, 0, s>>>(
      params, members, in_mean, in_inv_std, out_scale, out_shift, static_cast<uint8_t*>(packed));
  count_launch();
  return cuda_status(cudaGetLastError());
}

int launch_infer(const void* packed, int members, const float* x, int64_t batch, float* y, cudaStream_t s) {
  InferParams p;
  p.packed = static_cast<const uint8_t*>(packed);
  p.members = members;
  p.x = x;
  p.batch = batch;
  p.y = y;
  p.tiles = (batch + QT - 1) / QT;
  const int sms = sm_count();
  int groups = (int)imax<int64_t>(1, imin<int64_t>(sms / members, p.tiles));
  cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  if (e != cudaSuccess) return cuda_status(e);
  TimerScope ts(K_MLP_INFER, (double)batch * members, s);
  mlp_infer_kernel<<<groups * members, THREADS, SMEM_BYTES, s>>>(p);
  count_launch();
  return cuda_status(cudaGetLastError());
}

void launch_combine(const float* y, int members, int64_t batch, const float* x, const float* in_mean,
                    const float* in_inv_std, float base_a, float base_b, float spread_tol, float r2_max, float* mean,
                    float* spread, uint8_t* served, cudaStream_t s) {
  combine_kernel<<<(unsigned)((batch + 255) / 256), 256, 0, s>>>(y, members, batch, x, in_mean, in_inv_std, base_a,
                                                                 base_b, spread_tol, r2_max, mean, spread, served);
  count_launch();
}

}  // namespace mlp

unsigned int mlp_tc_take_device_error() { return take_unit_device_error(); }

}  // namespace fsk
